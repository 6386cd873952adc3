/* -*- c++ -*- ----------------------------------------------------------
   tersoff/gb300: pair_style tersoff evaluated by the GB300 engine.
   Parameters are read by the stock PairTersoff::coeff/read_file/setup_params
   (MANYBODY/pair_tersoff.cpp:293-580) and copied into the engine; compute()
   (pair_tersoff.cpp:86-265) is replaced by one engine call.
------------------------------------------------------------------------- */

#ifdef PAIR_CLASS

PairStyle(tersoff/gb300,PairTersoffGB300)

#else

#ifndef LMP_PAIR_TERSOFF_GB300_H
#define LMP_PAIR_TERSOFF_GB300_H

#include "pair_tersoff.h"
#include "gb300_common.h"

namespace LAMMPS_NS {

class PairTersoffGB300 : public PairTersoff, public GB300Style {
 public:
  PairTersoffGB300(class LAMMPS *);
  virtual ~PairTersoffGB300() {}
  virtual void compute(int, int);
  virtual void init_style();
  virtual void fill_params(lmff_lammps::StyleParams &);
};

}

#endif
#endif
