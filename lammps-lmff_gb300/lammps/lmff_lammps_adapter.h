// Host adapter between a LAMMPS pair style and the GB300 engine's C ABI.
//
// It is independent of the LAMMPS headers, so the same code runs inside LAMMPS (through
// pair_tersoff_gb300 / pair_ilp_graphene_hbn_gb300) and in the adapter's own GPU test.
// One adapter = one pair sub-style = one engine holding only that style's parameters,
// so energies, virials and the ILP pvector stay attributed per style as
// PairHybrid::compute expects (pair_hybrid.cpp:146-156).
//
// Calling convention mirrors Pair::compute(eflag, vflag) on one MPI rank: owned atoms
// x[0..nlocal) (LAMMPS stores x and f as one contiguous nmax*3 block), periodic box,
// forces accumulated into f (ghost forces untouched: the engine handles periodic images
// itself, so nothing is left for reverse communication to fold), per-style energy into
// eng_vdwl, global virial into virial[6], per-atom energy into eatom.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "lmff_gb300.h"

namespace lmff_lammps {

struct StyleOut {
  double eng_vdwl = 0.0;
  double virial[6] = {0, 0, 0, 0, 0, 0};
  double pvector[2] = {0, 0};
};

class Adapter {
 public:
  Adapter() = default;
  ~Adapter();
  Adapter(const Adapter &) = delete;
  Adapter &operator=(const Adapter &) = delete;

  // (Re)create the engine from the style's parameters after coeff().  precision:
  // LMFF_FP64 or LMFF_MIXED; device: CUDA ordinal.  Returns 0 or an LMFF_E* code.
  int create(const lmff_params &p, int device, int precision, std::string &err);
  bool ready() const { return e_ != nullptr; }

  // One evaluation.  which: LMFF_TERSOFF or LMFF_ILP.  mol / tag may be 32- or 64-bit
  // (LAMMPS tagint); pass the matching pointer and nullptr for the other.  reneighbored:
  // LAMMPS rebuilt its lists this step (atoms may have been reordered or exchanged), so
  // the identity arrays are sent again.
  int compute(int which, int nlocal, const double *x, const int *type, const int32_t *mol32, const int64_t *mol64,
              const int32_t *tag32, const int64_t *tag64, bool reneighbored, const double boxlo[3],
              const double boxhi[3], const int periodic[3], double *f, double *eatom, int eflag, int vflag,
              StyleOut &out, std::string &err);

 private:
  lmff_engine *e_ = nullptr;
  std::vector<int64_t> mol_, tag_;
  bool have_identity_ = false;
  int last_n_ = -1;
};

// Environment selection of the precision for the drop-in styles:
// LMFF_GB300_PRECISION = "fp64" (default) or "mixed"; LMFF_GB300_DEVICE = ordinal.
int precision_from_env();
int device_from_env();

}  // namespace lmff_lammps
