// Host adapter between the LAMMPS pair styles and the GB300 engine's C ABI.
//
// It is independent of the LAMMPS headers, so the same code runs inside LAMMPS (through
// pair_tersoff_gb300, pair_ilp_graphene_hbn_gb300, pair_kolmogorov_crespi_full_gb300)
// and in the adapter's own GPU test (tests/lammps_adapter_driver.cpp).
//
// Calling convention mirrors Pair::compute(eflag, vflag) on one MPI rank.  LAMMPS
// stores x and f as contiguous nmax*3 blocks, owned atoms [0, nlocal) first, then the
// ghost atoms [nlocal, nall).  Two forms:
//  - periodic: the rank owns the whole system (one MPI rank); the engine takes the owned
//    atoms and the periodic box and handles the images itself, ghost forces stay zero;
//  - subdomain: one rank of a domain decomposition; the engine takes owned and ghost
//    atoms (lmff_compute_ghost), evaluates the interactions this rank owns and writes
//    forces and per-atom energies for all nall atoms, which LAMMPS's reverse
//    communication folds onto their owners.
// Forces are accumulated into f, energies per style into StyleOut::eng_vdwl, the global
// virial into StyleOut::virial, per-atom energy into eatom, per-atom virial (rows of 6,
// LAMMPS's vatom) into vatom.
//
// With pair_style hybrid/overlay of a Tersoff and an interlayer gb300 style, both share
// one engine (Shared): PairHybrid::compute (pair_hybrid.cpp:93-137) calls the sub-styles
// one after the other, and the first one called evaluates both in one engine call (one
// list build, one short-list pass, one launch sequence); the second takes its energies,
// virial and pvector from that evaluation and adds no force (per-atom energies and
// virials of both styles go to the first style's arrays, whose sum PairHybrid forms).
#pragma once

#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "lmff_gb300.h"

namespace lmff_lammps {

struct StyleOut {
  double eng_vdwl = 0.0;
  double virial[6] = {0, 0, 0, 0, 0, 0};
  double pvector[2] = {0, 0};
};

// The parameters one or two pair styles give an engine; lmff_params points into these
// vectors, so they live as long as the engine is being created.
struct StyleParams {
  int ntypes = 0;
  double skin = 2.0;
  bool tersoff = false;
  int t_nelements = 0;
  std::vector<lmff_tersoff_param> t_params;
  std::vector<int> t_elem2param, t_map;
  double t_cutmax = 0.0;
  bool interlayer = false;
  int model = LMFF_INTERLAYER_ILP;
  int i_nelements = 0;
  std::vector<lmff_ilp_param> ilp_params;
  std::vector<lmff_kc_param> kc_params;
  std::vector<int> i_elem2param, i_map;
  std::vector<double> i_cutsq;
  double cut_global = 0.0;
  int tap_flag = 1;
  // the present styles' fields of p (the others are left as they are)
  void fill(lmff_params &p) const;
  // this style's parameters and the other's, for one shared engine
  void merge(const StyleParams &other);
};

class Adapter {
 public:
  Adapter() = default;
  ~Adapter();
  Adapter(const Adapter &) = delete;
  Adapter &operator=(const Adapter &) = delete;

  // (Re)create the engine from the styles' parameters after coeff().  precision:
  // LMFF_FP64 or LMFF_MIXED; device: CUDA ordinal.  Returns 0 or an LMFF_E* code.
  int create(const lmff_params &p, int device, int precision, std::string &err);
  int create(const StyleParams &sp, int device, int precision, std::string &err);
  bool ready() const { return e_ != nullptr; }

  // One evaluation.  which: LMFF_TERSOFF and/or LMFF_ILP.  subdomain: x, type, mol and
  // tag hold nall atoms (owned, then ghosts) and f, eatom receive nall; otherwise nall
  // is ignored and only the nlocal owned atoms are used.  mol / tag may be 32- or 64-bit
  // (LAMMPS tagint); pass the matching pointer and nullptr for the other.
  // reneighbored: LAMMPS rebuilt its lists this step (atoms may have been reordered or
  // exchanged), so the identity arrays are sent again.  out[0]: Tersoff, out[1]: the
  // interlayer style.  eatom, vatom: nullptr when not asked (eflag_atom, vflag_atom).
  int compute(int which, int nlocal, int nall, bool subdomain, const double *x, const int *type, const int32_t *mol32,
              const int64_t *mol64, const int32_t *tag32, const int64_t *tag64, bool reneighbored,
              const double boxlo[3], const double boxhi[3], const int periodic[3], double *f, double *eatom,
              double *vatom, int eflag, int vflag, StyleOut out[2], std::string &err);

 private:
  lmff_engine *e_ = nullptr;
  std::vector<int64_t> mol_, tag_;
  bool have_identity_ = false;
  int last_n_ = -1, last_nlocal_ = -1;
  bool last_subdomain_ = false;
};

// The engine of one style, or the one engine a Tersoff style and an interlayer style of
// hybrid/overlay share.  slot: 0 Tersoff, 1 interlayer.
class Shared {
 public:
  Adapter ad;
  // partner_computes: the other style shares this engine and is computed in the same
  // PairHybrid::compute (its compute_flag is on).  The first of the two calls evaluates
  // both styles and keeps the partner's outputs; the partner's call returns them and
  // adds no force.
  int evaluate(int slot, bool partner_computes, int nlocal, int nall, bool subdomain, const double *x, const int *type,
               const int32_t *mol32, const int64_t *mol64, const int32_t *tag32, const int64_t *tag64,
               bool reneighbored, const double boxlo[3], const double boxhi[3], const int periodic[3], double *f,
               double *eatom, double *vatom, int eflag, int vflag, StyleOut &out, std::string &err);
  void reset() { pending_[0] = pending_[1] = false; }

 private:
  StyleOut cache_[2];
  bool pending_[2] = {false, false};
};

// Environment selection for the drop-in styles: LMFF_GB300_PRECISION = "fp64" (default)
// or "mixed"; LMFF_GB300_DEVICE = ordinal; LMFF_GB300_SUBDOMAIN = 1 uses the subdomain
// form on a single rank too (it is always used with more than one rank).
int precision_from_env();
int device_from_env();
bool subdomain_from_env();

}  // namespace lmff_lammps
