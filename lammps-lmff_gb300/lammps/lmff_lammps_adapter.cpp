// Host adapter between a LAMMPS pair style and the GB300 engine (see the header).
#include "lmff_lammps_adapter.h"

#include <cstdlib>
#include <cstring>

namespace lmff_lammps {

Adapter::~Adapter() {
  if (e_) lmff_destroy(e_);
}

int Adapter::create(const lmff_params &p, int device, int precision, std::string &err) {
  if (e_) lmff_destroy(e_);
  e_ = nullptr;
  have_identity_ = false;
  last_n_ = -1;
  int rc = lmff_create(&e_, &p, device);
  if (rc != LMFF_OK) {
    err = lmff_last_error(nullptr);
    e_ = nullptr;
    return rc;
  }
  rc = lmff_set_precision(e_, precision);
  if (rc != LMFF_OK) err = lmff_last_error(e_);
  return rc;
}

int Adapter::compute(int which, int nlocal, const double *x, const int *type, const int32_t *mol32,
                     const int64_t *mol64, const int32_t *tag32, const int64_t *tag64, bool reneighbored,
                     const double boxlo[3], const double boxhi[3], const int periodic[3], double *f, double *eatom,
                     int eflag, int vflag, StyleOut &out, std::string &err) {
  out = StyleOut();
  if (!e_) {
    err = "GB300 engine not initialised (pair_coeff missing?)";
    return LMFF_EINVAL;
  }
  int rc = lmff_set_box(e_, boxlo, boxhi, 0.0, 0.0, 0.0, periodic);
  if (rc != LMFF_OK) {
    err = lmff_last_error(e_);
    return rc;
  }
  bool send_identity = reneighbored || !have_identity_ || nlocal != last_n_;
  if (send_identity) {
    mol_.resize(nlocal);
    tag_.resize(nlocal);
    for (int i = 0; i < nlocal; i++) {
      mol_[i] = mol64 ? mol64[i] : (mol32 ? (int64_t)mol32[i] : 0);
      tag_[i] = tag64 ? tag64[i] : (tag32 ? (int64_t)tag32[i] : (int64_t)(i + 1));
    }
    have_identity_ = true;
    last_n_ = nlocal;
  }
  lmff_result res;
  memset(&res, 0, sizeof res);
  int flags = which | (send_identity ? 0 : LMFF_SAME_ATOMS);
  rc = lmff_compute(e_, nlocal, x, type, mol_.data(), tag_.data(), flags, eflag, vflag, f, eatom, &res);
  if (rc != LMFF_OK) {
    err = lmff_last_error(e_);
    have_identity_ = false;
    return rc;
  }
  if (which & LMFF_TERSOFF) {
    out.eng_vdwl += res.e_tersoff;
    for (int k = 0; k < 6; k++) out.virial[k] += res.virial_tersoff[k];
  }
  if (which & LMFF_ILP) {
    out.eng_vdwl += res.e_ilp;
    for (int k = 0; k < 6; k++) out.virial[k] += res.virial_ilp[k];
    out.pvector[0] = res.pvector[0];
    out.pvector[1] = res.pvector[1];
  }
  return LMFF_OK;
}

int precision_from_env() {
  const char *s = getenv("LMFF_GB300_PRECISION");
  if (s && (strcmp(s, "mixed") == 0 || strcmp(s, "MIXED") == 0)) return LMFF_MIXED;
  return LMFF_FP64;
}

int device_from_env() {
  const char *s = getenv("LMFF_GB300_DEVICE");
  return s ? atoi(s) : 0;
}

}  // namespace lmff_lammps
