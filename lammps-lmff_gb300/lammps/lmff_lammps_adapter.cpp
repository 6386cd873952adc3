// Host adapter between the LAMMPS pair styles and the GB300 engine (see the header).
#include "lmff_lammps_adapter.h"

#include <cstdlib>
#include <cstring>

namespace lmff_lammps {

void StyleParams::fill(lmff_params &p) const {
  p.ntypes = ntypes;
  p.skin = skin;
  if (tersoff) {
    p.tersoff_nelements = t_nelements;
    p.tersoff_nparams = (int)t_params.size();
    p.tersoff_params = t_params.data();
    p.tersoff_elem2param = t_elem2param.data();
    p.tersoff_map = t_map.data();
    p.tersoff_cutmax = t_cutmax;
  }
  if (interlayer) {
    p.interlayer_model = model;
    p.ilp_nelements = i_nelements;
    if (model == LMFF_INTERLAYER_KC) {
      p.ilp_nparams = (int)kc_params.size();
      p.kc_params = kc_params.data();
    } else {
      p.ilp_nparams = (int)ilp_params.size();
      p.ilp_params = ilp_params.data();
    }
    p.ilp_elem2param = i_elem2param.data();
    p.ilp_map = i_map.data();
    p.ilp_cutILPsq = i_cutsq.data();
    p.ilp_cut_global = cut_global;
    p.ilp_tap_flag = tap_flag;
  }
}

void StyleParams::merge(const StyleParams &o) {
  if (o.tersoff && !tersoff) {
    tersoff = true;
    t_nelements = o.t_nelements;
    t_params = o.t_params;
    t_elem2param = o.t_elem2param;
    t_map = o.t_map;
    t_cutmax = o.t_cutmax;
  }
  if (o.interlayer && !interlayer) {
    interlayer = true;
    model = o.model;
    i_nelements = o.i_nelements;
    ilp_params = o.ilp_params;
    kc_params = o.kc_params;
    i_elem2param = o.i_elem2param;
    i_map = o.i_map;
    i_cutsq = o.i_cutsq;
    cut_global = o.cut_global;
    tap_flag = o.tap_flag;
  }
}

Adapter::~Adapter() {
  if (e_) lmff_destroy(e_);
}

int Adapter::create(const lmff_params &p, int device, int precision, std::string &err) {
  if (e_) lmff_destroy(e_);
  e_ = nullptr;
  have_identity_ = false;
  last_n_ = last_nlocal_ = -1;
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

int Adapter::create(const StyleParams &sp, int device, int precision, std::string &err) {
  lmff_params p;
  memset(&p, 0, sizeof p);
  sp.fill(p);
  return create(p, device, precision, err);
}

int Adapter::compute(int which, int nlocal, int nall, bool subdomain, const double *x, const int *type,
                     const int32_t *mol32, const int64_t *mol64, const int32_t *tag32, const int64_t *tag64,
                     bool reneighbored, const double boxlo[3], const double boxhi[3], const int periodic[3], double *f,
                     double *eatom, double *vatom, int eflag, int vflag, StyleOut out[2], std::string &err) {
  out[0] = StyleOut();
  out[1] = StyleOut();
  if (!e_) {
    err = "GB300 engine not initialised (pair_coeff missing?)";
    return LMFF_EINVAL;
  }
  const int n = subdomain ? nall : nlocal;
  int rc;
  if (!subdomain) {
    rc = lmff_set_box(e_, boxlo, boxhi, 0.0, 0.0, 0.0, periodic);
    if (rc != LMFF_OK) {
      err = lmff_last_error(e_);
      return rc;
    }
  }
  bool send_identity = reneighbored || !have_identity_ || n != last_n_ || nlocal != last_nlocal_ ||
                       subdomain != last_subdomain_;
  if (send_identity) {
    mol_.resize(n);
    tag_.resize(n);
    for (int i = 0; i < n; i++) {
      mol_[i] = mol64 ? mol64[i] : (mol32 ? (int64_t)mol32[i] : 0);
      tag_[i] = tag64 ? tag64[i] : (tag32 ? (int64_t)tag32[i] : (int64_t)(i + 1));
    }
    have_identity_ = true;
    last_n_ = n;
    last_nlocal_ = nlocal;
    last_subdomain_ = subdomain;
  }
  lmff_result res;
  memset(&res, 0, sizeof res);
  int flags = which | (send_identity ? 0 : LMFF_SAME_ATOMS);
  if (subdomain)
    rc = lmff_compute_ghost(e_, nlocal, nall, x, type, mol_.data(), tag_.data(), flags, eflag, vflag, f, eatom, &res);
  else
    rc = lmff_compute(e_, nlocal, x, type, mol_.data(), tag_.data(), flags, eflag, vflag, f, eatom, &res);
  if (rc == LMFF_OK && vatom && n > 0)
    rc = lmff_compute_vatom(e_, which & (LMFF_TERSOFF | LMFF_ILP), n, vatom);
  if (rc != LMFF_OK) {
    err = lmff_last_error(e_);
    have_identity_ = false;
    return rc;
  }
  if (which & LMFF_TERSOFF) {
    out[0].eng_vdwl = res.e_tersoff;
    for (int k = 0; k < 6; k++) out[0].virial[k] = res.virial_tersoff[k];
  }
  if (which & LMFF_ILP) {
    out[1].eng_vdwl = res.e_ilp;
    for (int k = 0; k < 6; k++) out[1].virial[k] = res.virial_ilp[k];
    out[1].pvector[0] = res.pvector[0];
    out[1].pvector[1] = res.pvector[1];
  }
  return LMFF_OK;
}

int Shared::evaluate(int slot, bool partner_computes, int nlocal, int nall, bool subdomain, const double *x,
                     const int *type, const int32_t *mol32, const int64_t *mol64, const int32_t *tag32,
                     const int64_t *tag64, bool reneighbored, const double boxlo[3], const double boxhi[3],
                     const int periodic[3], double *f, double *eatom, double *vatom, int eflag, int vflag,
                     StyleOut &out, std::string &err) {
  if (pending_[slot]) {   // the partner's call this step evaluated this style too
    pending_[slot] = false;
    out = cache_[slot];
    return LMFF_OK;
  }
  const int mine = slot == 0 ? LMFF_TERSOFF : LMFF_ILP;
  const int other = slot == 0 ? LMFF_ILP : LMFF_TERSOFF;
  StyleOut o[2];
  int rc = ad.compute(mine | (partner_computes ? other : 0), nlocal, nall, subdomain, x, type, mol32, mol64, tag32,
                      tag64, reneighbored, boxlo, boxhi, periodic, f, eatom, vatom, eflag, vflag, o, err);
  if (rc != LMFF_OK) return rc;
  out = o[slot];
  if (partner_computes) {
    cache_[1 - slot] = o[1 - slot];
    pending_[1 - slot] = true;
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

bool subdomain_from_env() {
  const char *s = getenv("LMFF_GB300_SUBDOMAIN");
  return s && atoi(s) != 0;
}

}  // namespace lmff_lammps
