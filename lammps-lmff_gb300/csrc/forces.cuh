// Force kernels of the Tersoff + ILP engine, templated on the arithmetic type R
// (double: all-FP64 drop-in; float: mixed precision, FP32 pair/three-body arithmetic on
// displacements formed from double-float positions, FP64 per-atom accumulation,
// reductions and normal-derivative assembly).
//
// Formulation: a deterministic gather, no force atomics.  Every owned atom sums every
// force on itself:
//   * ILP (pair_ilp_graphene_hbn.cpp:449-675): for each interlayer neighbour j the vdW
//     force, the repulsion of the term that uses i's normal (calc_FRep with i as owner)
//     and the repulsion of the term that uses j's normal (i plays calc_FRep's "j").
//     The normal-derivative forces of the terms owned by i are reverse-accumulated: the
//     pair loop sums g_i = sum_j Tap*prod*fpair1*del, then (dn_i/dx_m)^T g_i is applied
//     once per intralayer neighbour m (the LMFF dprodni idea, LMFF/pair_lmff.cpp:916-1025).
//     Those per-neighbour forces are left in ilp_c slots and gathered by their targets.
//   * Tersoff (pair_tersoff.cpp:117-262): each atom evaluates the bonds it centres (zeta,
//     force_zeta, attractive over k) and leaves the forces on its bond partners in
//     ters_g slots; repulsion is evaluated from both ends.
//   * k_finish gathers the slots of the neighbours (slot of a in N(j) found by matching
//     the reversed image code), so every force sum has a fixed order.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "engine.cuh"

namespace lmff {

// ------------------------------------------------------------------ precision policy

template <class R>
struct Math;

template <>
struct Math<double> {
  static __device__ __forceinline__ double ex(double a) { return exp(a); }
  // exp(-lambda (r - z0)) and friends in the reference's own form
  static __device__ __forceinline__ double exp_rep0(const IlpP<double> &p, double r) { return exp(-p.lambda * (r - p.z0)); }
  static __device__ __forceinline__ double exp_rep1(const IlpP<double> &p, double rhosq) { return exp(-(rhosq * p.delta2inv)); }
  static __device__ __forceinline__ double exp_ts(const IlpP<double> &p, double r) { return exp(-p.d * (r / p.seff - 1.0)); }
  static __device__ __forceinline__ double rcp(double a) { return 1.0 / a; }
  static __device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }
  static __device__ __forceinline__ double pow_(double a, double b) { return pow(a, b); }
  static __device__ __forceinline__ void sincospi_(double a, double *s, double *c) { sincospi(a, s, c); }
};

// Single hardware approximations (PTX ex2/rsqrt/rcp .approx.ftz): relative error about
// 2^-22, the accuracy of the FP32 pair arithmetic around them.  Flushing subnormals is
// harmless here: the exponentials underflow to 0 only far beyond any contribution that
// matters, and distances are bounded away from 0.
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <>
struct Math<float> {
  static __device__ __forceinline__ float ex(float a) { return expf(a); }
  // lambda log2e (z0 - r): the constant's rounding scales a small argument instead of
  // shifting every pair's exponent by the same absolute amount
  static __device__ __forceinline__ float exp_rep0(const IlpP<float> &p, float r) { return ex2_ftz(p.lam_l2e * (p.z0 - r)); }
  static __device__ __forceinline__ float exp_rep1(const IlpP<float> &p, float rhosq) { return ex2_ftz(p.nd2_l2e * rhosq); }
  // exp(-d (r/seff - 1)) = exp2((d/seff) log2e (seff - r))
  static __device__ __forceinline__ float exp_ts(const IlpP<float> &p, float r) { return ex2_ftz(p.ts_a * (p.seff - r)); }
  static __device__ __forceinline__ float rcp(float a) { return rcp_ftz(a); }
  static __device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
  static __device__ __forceinline__ float pow_(float a, float b) { return powf(a, b); }
  static __device__ __forceinline__ void sincospi_(float a, float *s, float *c) { sincospif(a, s, c); }
};

// atom info packed next to the position: (mol_dense << 8) | type
__device__ __forceinline__ int info_type(long long w) { return (int)(w & 255); }
__device__ __forceinline__ long long info_mol(long long w) { return w >> 8; }

// --------------------------------------------------------------- position access

struct AtomArrays {
  const d4 *xq;
  const float4 *xh;
  const float4 *xl;
  const SysDesc *sys;
  const int *sysid;
  // mixed pair kernel's j data, one 48-byte record per atom written by k_short each
  // step: hi parts + info, lo parts, normal -- the three loads of a pair hit one line
  const float4 *jrec;
  // the same without the info word, 32 bytes: (hi x, y, z, lo x|y as two FP16), (normal,
  // lo z as FP16) -- for the single-element loop, which needs no molecule or type
  const float4 *jrec2;
};

template <class R>
struct AtomI;

template <>
struct AtomI<double> {
  double x, y, z;
  long long info;
  __device__ __forceinline__ void load(const AtomArrays &A, int i) {
    d4 q = A.xq[i];
    x = q.x; y = q.y; z = q.z;
    info = __double_as_longlong(q.w);
  }
  // del = x_i - (x_j + s L): the reference's delx = xtmp - x[j][0] on a ghost x[j] = x + prd
  __device__ __forceinline__ void disp(const AtomArrays &A, const SysDesc &sd, int j, int sx, int sy, int sz,
                                       double &dx, double &dy, double &dz, long long &jinfo) const {
    d4 q = A.xq[j];
    double xj = sx ? __dadd_rn(q.x, sx * sd.L[0]) : q.x;
    double yj = sy ? __dadd_rn(q.y, sy * sd.L[1]) : q.y;
    double zj = sz ? __dadd_rn(q.z, sz * sd.L[2]) : q.z;
    dx = __dsub_rn(x, xj);
    dy = __dsub_rn(y, yj);
    dz = __dsub_rn(z, zj);
    jinfo = __double_as_longlong(q.w);
  }
  // the same split into a load (issued early) and the arithmetic
  struct J {
    d4 q;
  };
  __device__ __forceinline__ J fetch(const AtomArrays &A, int j) const { return J{A.xq[j]}; }
  __device__ __forceinline__ void disp_from(const J &t, const SysDesc &sd, int sx, int sy, int sz, double &dx,
                                            double &dy, double &dz, long long &jinfo) const {
    double xj = sx ? __dadd_rn(t.q.x, sx * sd.L[0]) : t.q.x;
    double yj = sy ? __dadd_rn(t.q.y, sy * sd.L[1]) : t.q.y;
    double zj = sz ? __dadd_rn(t.q.z, sz * sd.L[2]) : t.q.z;
    dx = __dsub_rn(x, xj);
    dy = __dsub_rn(y, yj);
    dz = __dsub_rn(z, zj);
    jinfo = __double_as_longlong(t.q.w);
  }
};

template <>
struct AtomI<float> {
  float hx, hy, hz, lx, ly, lz;
  long long info;
  __device__ __forceinline__ void load(const AtomArrays &A, int i) {
    float4 h = A.xh[i];
    float4 l = A.xl[i];
    hx = h.x; hy = h.y; hz = h.z;
    lx = l.x; ly = l.y; lz = l.z;
    info = (long long)__float_as_int(h.w);
  }
  // del = x_i - x_j(image) from double-float parts: the hi difference is exact (both
  // hi parts share one binade), the lo parts carry the remaining 24 bits.
  __device__ __forceinline__ void disp(const AtomArrays &A, const SysDesc &sd, int j, int sx, int sy, int sz,
                                       float &dx, float &dy, float &dz, long long &jinfo) const {
    float4 h = __ldg(&A.xh[j]);
    float4 l = __ldg(&A.xl[j]);
    float sxh = (float)sx * sd.Lhi[0], syh = (float)sy * sd.Lhi[1], szh = (float)sz * sd.Lhi[2];
    float sxl = (float)sx * sd.Llo[0], syl = (float)sy * sd.Llo[1], szl = (float)sz * sd.Llo[2];
    dx = ((hx - h.x) - sxh) + ((lx - l.x) - sxl);
    dy = ((hy - h.y) - syh) + ((ly - l.y) - syl);
    dz = ((hz - h.z) - szh) + ((lz - l.z) - szl);
    jinfo = (long long)__float_as_int(h.w);
  }
  struct J {
    float4 h, l;
  };
  __device__ __forceinline__ J fetch(const AtomArrays &A, int j) const {
    return J{__ldg(&A.jrec[3 * (size_t)j]), __ldg(&A.jrec[3 * (size_t)j + 1])};
  }
  __device__ __forceinline__ void disp_from(const J &t, const SysDesc &sd, int sx, int sy, int sz, float &dx, float &dy,
                                            float &dz, long long &jinfo) const {
    float sxh = (float)sx * sd.Lhi[0], syh = (float)sy * sd.Lhi[1], szh = (float)sz * sd.Lhi[2];
    float sxl = (float)sx * sd.Llo[0], syl = (float)sy * sd.Llo[1], szl = (float)sz * sd.Llo[2];
    dx = ((hx - t.h.x) - sxh) + ((lx - t.l.x) - sxl);
    dy = ((hy - t.h.y) - syh) + ((ly - t.l.y) - syl);
    dz = ((hz - t.h.z) - szh) + ((lz - t.l.z) - szl);
    jinfo = (long long)__float_as_int(t.h.w);
  }
};

// exact FP64 squared distance in the reference's evaluation order (no contraction)
__device__ __forceinline__ double rsq_rn(double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// FP64 displacement x_i - x_j(image) used for set decisions and FP64 assembly
__device__ __forceinline__ void disp64(const d4 *xq, const SysDesc &sd, int i, int j, int sx, int sy, int sz,
                                       double &dx, double &dy, double &dz) {
  d4 a = xq[i];
  d4 b = xq[j];
  double xj = b.x, yj = b.y, zj = b.z;
  // one branch for the (rare) periodic image: b + 0 * L = b, so a zero component of a
  // non-zero shift gives the same value as no shift
  if ((sx | sy | sz) != 0) {
    xj = __dadd_rn(b.x, sx * sd.L[0]);
    yj = __dadd_rn(b.y, sy * sd.L[1]);
    zj = __dadd_rn(b.z, sz * sd.L[2]);
  }
  dx = __dsub_rn(a.x, xj);
  dy = __dsub_rn(a.y, yj);
  dz = __dsub_rn(a.z, zj);
}

// --------------------------------------------------------------- kernel arguments

// the second velocity half-kick of an NVE step, applied by the gather kernel to the force
// it has just summed (fix_nve.cpp final_integrate: v += dtf / m f): v SoA, dtf / m per type
struct KickArgs {
  double *v;
  double dtfm[MAXTYPE + 1];
  // drift != 0: the gather also makes the next step's first half (velocity half-kick and
  // position drift, k_nve1's arithmetic) -- steps between rebuild tests inside one step
  // graph; an atom moved more than skin/2 since the last build raises ST_SKIN_TRIP
  int drift;
  int do_hilo;
  double dtv, trig2;
  d4 *xq;
  const double *xhold;
  float4 *xh, *xl;
  const SysDesc *sys;
  const int *sysid;
  int *status;
};

// Threads per block of the one-thread-per-atom kernels: 128, halved (down to 32) while
// the grid would give fewer than two blocks per SM.  A small system then spreads over
// every SM instead of filling a few with four warps each: the FP64-bound kernels
// (Tersoff, the normal-derivative assembly, the integrator) take their time from the
// FP64 pipe of the SMs they occupy (7,200 atoms: 57 blocks of 128 on 152 SMs).
inline int per_atom_block(int n) {
  static const int sms = [] {
    int d = 0, v = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
    return v > 0 ? v : 1;
  }();
  int b = 128;
  while (b > 32 && (n + b - 1) / b < 2 * sms) b >>= 1;
  return b;
}

// Velocity Verlet's position drift of atom q (fix_nve.cpp:89-91) on its half-kicked
// velocity, with the double-float split of the mixed kernels refreshed; returns the
// squared displacement since the last build.  k_nve1 and the gather's drift share it.
__device__ __forceinline__ double nve_drift(int q, double vx, double vy, double vz, double dtv, d4 *xq,
                                            const double *xhold, float4 *xh, float4 *xl, const SysDesc *sys,
                                            const int *sysid, int do_hilo) {
  const d4 w = xq[q];
  const double x = w.x + dtv * vx, y = w.y + dtv * vy, z = w.z + dtv * vz;
  xq[q].x = x;
  xq[q].y = y;
  xq[q].z = z;
  const double dx = x - xhold[3 * q], dy = y - xhold[3 * q + 1], dz = z - xhold[3 * q + 2];
  if (do_hilo) {
    const SysDesc &sd = sys[sysid[q]];
    const double X = x - sd.lo[0] + 32.0 + sd.base;
    const double Y = y - sd.lo[1] + 32.0 + sd.base;
    const double Z = z - sd.lo[2] + 32.0 + sd.base;
    const float hx = (float)X, hy = (float)Y, hz = (float)Z;
    const float4 h = xh[q];
    xh[q] = make_float4(hx, hy, hz, h.w);
    xl[q] = make_float4((float)(X - (double)hx), (float)(Y - (double)hy), (float)(Z - (double)hz), 0.f);
  }
  return dx * dx + dy * dy + dz * dz;
}

template <class R>
struct ForceArgs {
  AtomArrays A;
  ListCode lc;
  int n;
  const int64_t *tag;
  const int64_t *list_off;
  const uint32_t *list;
  const uint8_t *list_img;    // 1 when atom i's list holds periodic-image entries
  const int *short_cnt;
  const uint32_t *short_nb;
  int *ilp_cnt;
  uint32_t *ilp_nb;
  int *ters_cnt;
  uint32_t *ters_nb;
  d4 *nrm64;
  float4 *nrm32;
  float4 *jrec;        // 3 per atom (mixed path): see AtomArrays::jrec
  float4 *jrec2;       // 2 per atom (mixed path): see AtomArrays::jrec2
  d4 *ters_g;
  double *ters_f;
  double *ilp_f;
  d4 *ilp_c;
  d4 *ilp_g;           // reverse-accumulated dE/dn_i of the terms owned by i (k_ilp -> k_nderiv)
  d4 *nframe;          // 4 per atom: the normal frame k_nframe leaves for k_nderiv, or null
                       // (k_nderiv then assembles in one piece)
  double *stat_ilp;    // 8 * n SoA: e_vdw/2, e_rep/2, virial[6]    (EV only)
  double *stat_ters;   // 8 * n SoA: e, 0, virial[6]
  double *eatom_ilp;   // n (EATOM only)
  double *eatom_ters;  // n
  double *f_out;       // 3*n SoA (k_finish)
  // per-atom virial pass (FP64 kernels run on request after an evaluation), 6 doubles
  // per entry in LAMMPS order xx yy zz xy xz yz: each atom's own share per style (va_t,
  // va_i: n entries) and the shares it leaves for its Tersoff bond partners (va_ts:
  // MAXTERS per atom, by short-list slot) and intralayer neighbours (va_is: MAXILP per atom)
  double *va_t, *va_i, *va_ts, *va_is;
  float4 *va_tens;     // mixed pass: 7 per atom, the frame's partner-share tensors (k_va_tens)
  int *status;
  int do_ters, do_ilp;
  int list_full;       // the pair list also holds same-molecule / non-ILP pairs
  // subdomain (ghost-atom) mode: non-null when the caller passes owned atoms followed by
  // ghost atoms; sorted atom s is owned when own_perm[s] < nown.  Only interactions owned
  // by owned atoms are evaluated (two-body terms by the reference's tag-parity half of
  // the full list, three-body and normal terms by their centre atom); every atom, ghosts
  // included, receives its share of their forces.
  const int *own_perm;
  int nown;
  // list entries a lane of the mixed force-only pair kernel takes per loop iteration:
  // 2 (the two-entry loop, where it applies) or 1 (the one-entry loop); a tuning knob
  int pair_tile;
  // Tersoff runs with no pair kernel beside it (no interlayer style, or the two kernels
  // serialised): small systems then take one lane per bond (k_tersoff_lanes); beside
  // the pair kernel the one-thread kernel is kept, whose fewer instructions take fewer
  // issue slots from it
  int ters_alone;
  // 1: the large-system kernels at every size (option small_variants 0: the lanes-per-atom
  // variants of the short lists, the gather and Tersoff are not used)
  int no_small;
  int kc;              // interlayer style is kolmogorov/crespi/full
  // programmatic dependent launch (PDL) of the step's chain kernels, a PDL_* mask: which
  // kernels are launched early behind the kernel before them on the stream (the pair
  // kernel, the normal-derivative kernel, the gather, and inside a step graph the
  // intralayer-list kernel after the previous step's gather), and whether the kernels
  // let their dependents be scheduled as soon as they start (PDL_TRIGGER) or only as
  // their blocks exit
  int pdl;
};

enum : int { PDL_ILP = 1, PDL_NDERIV = 2, PDL_FINISH = 4, PDL_SHORT = 8, PDL_TRIGGER = 16 };

// First statement of a kernel that may be launched early: wait until the kernels it
// depends on have completed and their writes are visible (griddepcontrol.wait; a no-op
// for an ordinary launch), then, with trigger, let its own dependents be scheduled.
// Waiting before any load or store covers both orders of hazard with the previous kernel.
__device__ __forceinline__ void pdl_enter(int pdl) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (pdl & PDL_TRIGGER) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// <<<grid, block, 0, s>>> with programmatic stream serialisation when pdl is set: the
// kernel may be scheduled before the previous kernel on s completes and waits in
// pdl_enter.  Only for launches whose predecessor on s is always a kernel.
template <typename... KP, typename... A>
inline void launch_pdl(bool pdl, void (*k)(KP...), int grid, int block, cudaStream_t s, A... args) {
  if (!pdl) {
    k<<<grid, block, 0, s>>>(args...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

}  // namespace lmff
