/* -*- c++ -*- ----------------------------------------------------------
   ilp/graphene/hbn/gb300: pair_style ilp/graphene/hbn evaluated by the GB300
   engine.  settings/coeff/read_file/init_one are the stock ones
   (USER-MISC/pair_ilp_graphene_hbn.cpp:132-387); compute() (:428-443: ILP_neigh,
   calc_normal, calc_FvdW, calc_FRep) is replaced by one engine call.
------------------------------------------------------------------------- */

#ifdef PAIR_CLASS

PairStyle(ilp/graphene/hbn/gb300,PairILPGrapheneHBNGB300)

#else

#ifndef LMP_PAIRILPGRAPHENEHBNGB300_H
#define LMP_PAIRILPGRAPHENEHBNGB300_H

#include "pair_ilp_graphene_hbn.h"
#include "gb300_common.h"

namespace LAMMPS_NS {

class PairILPGrapheneHBNGB300 : public PairILPGrapheneHBN, public GB300Style {
 public:
  PairILPGrapheneHBNGB300(class LAMMPS *);
  virtual ~PairILPGrapheneHBNGB300() {}
  virtual void compute(int, int);
  void init_style();
  virtual void fill_params(lmff_lammps::StyleParams &);
};

}

#endif
#endif
