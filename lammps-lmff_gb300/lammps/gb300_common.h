/* -*- c++ -*- ----------------------------------------------------------
   Parts the GB300 pair styles share (tersoff/gb300, ilp/graphene/hbn/gb300,
   kolmogorov/crespi/full/gb300): the engine set-up, including one engine for a
   Tersoff and an interlayer gb300 sub-style of the same hybrid/overlay, and the
   per-step call in the periodic form (one MPI rank) or the subdomain form (one rank of
   a domain decomposition: owned + ghost atoms, ghost forces folded by LAMMPS's
   reverse communication, verlet.cpp:307-332).
------------------------------------------------------------------------- */

#ifndef LMP_GB300_COMMON_H
#define LMP_GB300_COMMON_H

#include <memory>

#include "lmff_lammps_adapter.h"

namespace LAMMPS_NS {

class LAMMPS;
class Pair;

class GB300Style {
 public:
  virtual ~GB300Style() {}
  // this style's part of the engine parameters (its pair_coeff data), plus ntypes/skin
  virtual void fill_params(lmff_lammps::StyleParams &sp) = 0;

  std::shared_ptr<lmff_lammps::Shared> gb;
  Pair *partner = nullptr;         // the other gb300 style sharing gb, or NULL
  bool set_by_partner = false;     // gb was made by the partner's init_style this time
};

namespace gb300 {

// The engine of style `self` (slot 0 Tersoff, 1 interlayer): shared with the partner
// style when both are sub-styles of one hybrid/overlay, else its own.
void setup(LAMMPS *lmp, Pair *self, GB300Style *me, int slot, const char *name);

// One evaluation for style `self`; forces into atom->f, per-atom energy into self's
// eatom when eflag_atom, the style's energy, virial and pvector into out.
void compute(LAMMPS *lmp, Pair *self, GB300Style *me, int slot, int eflag, int vflag, int eflag_atom,
             int vflag_atom, const char *name, lmff_lammps::StyleOut &out);

}  // namespace gb300
}  // namespace LAMMPS_NS

#endif
