/* -*- c++ -*- ----------------------------------------------------------
   kolmogorov/crespi/full/gb300: pair_style kolmogorov/crespi/full evaluated by the
   GB300 engine.  settings/coeff/read_file/init_one are the stock ones
   (USER-MISC/pair_kolmogorov_crespi_full.cpp:133-392); compute() (:430-445: KC_neigh,
   calc_normal, calc_FvdW, calc_FRep) is replaced by one engine call.
------------------------------------------------------------------------- */

#ifdef PAIR_CLASS

PairStyle(kolmogorov/crespi/full/gb300,PairKolmogorovCrespiFullGB300)

#else

#ifndef LMP_PAIRKOLMOGOROVCRESPIFULLGB300_H
#define LMP_PAIRKOLMOGOROVCRESPIFULLGB300_H

#include "pair_kolmogorov_crespi_full.h"
#include "gb300_common.h"

namespace LAMMPS_NS {

class PairKolmogorovCrespiFullGB300 : public PairKolmogorovCrespiFull, public GB300Style {
 public:
  PairKolmogorovCrespiFullGB300(class LAMMPS *);
  virtual ~PairKolmogorovCrespiFullGB300() {}
  virtual void compute(int, int);
  void init_style();
  virtual void fill_params(lmff_lammps::StyleParams &);
};

}

#endif
#endif
