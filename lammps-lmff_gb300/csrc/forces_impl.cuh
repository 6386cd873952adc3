// Kernel bodies; included by forces64.cu (LMFF_REAL = double) and forces32.cu
// (LMFF_REAL = float), each of which owns one __constant__ copy of the potential.
#pragma once

#include <cuda_fp16.h>

#include <cmath>
#include <type_traits>

#include "forces.cuh"

namespace lmff {
namespace LMFF_NS {

using R = LMFF_REAL;
__constant__ PotConst<R> c_pot;

// FP16 pairs <-> 32-bit words (the compact j record's lo parts)
__device__ __forceinline__ unsigned h2_bits(__half2 h) {
  unsigned u;
  memcpy(&u, &h, sizeof u);
  return u;
}
__device__ __forceinline__ __half2 bits_h2(unsigned u) {
  __half2 h;
  memcpy(&h, &u, sizeof h);
  return h;
}

// the mixed single-element pair loop evaluates two list entries per iteration
#ifdef LMFF_PACKED_X2
constexpr bool TWO_PAIR_BODY = true;
#else
constexpr bool TWO_PAIR_BODY = false;
#endif

// whether the two-pair loop applies (set with the constants by upload_pot, read by the
// launch): element 0's C >= 0 (single element); symmetric element-pair constants with
// C >= 0 (several elements)
static int h_two_one = 0, h_two_multi = 0;

__device__ __forceinline__ R cR(double v) { return (R)v; }

__device__ __forceinline__ void raise_status(int *status, int bit) { atomicOr(status, bit); }

// squared distance in R; for FP64 in the reference's rounding
__device__ __forceinline__ R rsqR(R dx, R dy, R dz) {
  if constexpr (sizeof(R) == 8) return rsq_rn(dx, dy, dz);
  else return dx * dx + dy * dy + dz * dz;
}

// rsq < thr decided exactly as FP64 would (mixed: FP32 first, FP64 when within 1e-5)
__device__ __forceinline__ bool lt_exact(R rsq, R thr, const d4 *xq, const SysDesc &sd, int i, int j, int sx,
                                         int sy, int sz, double thr64) {
  if constexpr (sizeof(R) == 8) {
    return rsq < thr;
  } else {
    float m = 1e-5f * thr;
    if (rsq < thr - m) return true;
    if (rsq > thr + m) return false;
    double dx, dy, dz;
    disp64(xq, sd, i, j, sx, sy, sz, dx, dy, dz);
    return rsq_rn(dx, dy, dz) < thr64;
  }
}

// ============================================================== k_short ==========
// Per atom: the current-step ILP intralayer list (ILP_neigh, pair_ilp_graphene_hbn.cpp:
// 723-743: same molecule, rsq != 0, rsq < cutILPsq) and the Tersoff short list
// (pair_tersoff.cpp:132-147: rsq < cutmax^2), both taken in candidate order from the
// short candidate list built with skin; then the unit normal (calc_normal :776-1074).
// SG lanes per atom share its short candidates.  Each round the lanes test one
// candidate each; ballots over the atom's lanes give every accepted entry its position
// in candidate order, so the lists equal a one-lane walk's, and the bond vectors of the
// first three intralayer neighbours reach every lane by shuffles.  SG = 16 up to 16,384
// atoms and 4 up to 65,536, whose few threads cannot hide the candidate loop's chain of
// dependent loads (7,200 atoms, per step: SG 1 82.4 us, SG 4 66.7, SG 16 63.7); SG = 1
// for large ones, where the ballots only add work (2.7M atoms: 0.87 vs 1.09 ms with the
// normal-derivative kernel).
constexpr int SHORT_SG16_MAX_ATOMS = 16384;
constexpr int SHORT_SG_MAX_ATOMS = 65536;
template <int SG>
__global__ void k_short(ForceArgs<R> a, const double *cutILPsq64, double tcutmaxsq64) {
  pdl_enter(a.pdl);
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gtid / SG;
  if (i >= a.n) return;   // whole groups: blockDim is a multiple of SG
  const int wl = threadIdx.x & 31;
  const unsigned gmask = SG == 1 ? 0u : ((1u << SG) - 1) << (wl & ~(SG - 1));
  const unsigned below = gmask & ((1u << wl) - 1);
  const SysDesc &sd = a.A.sys[a.A.sysid[i]];
  AtomI<R> ai;
  ai.load(a.A, i);
  int ti = info_type(ai.info);
  long long mi = info_mol(ai.info);
  int ie = c_pot.i_enabled ? c_pot.i_map[ti] : -1;
  int te = c_pot.t_enabled ? c_pot.t_map[ti] : -1;
  int nilp = 0, nters = 0;   // the same in every lane of the atom
  R vx[MAXILP], vy[MAXILP], vz[MAXILP];
  const int cnt = a.short_cnt[i];
  for (int c0 = 0; c0 < cnt; c0 += SG) {
    const int c = c0 + (wl & (SG - 1));
    bool take_ilp = false, take_ters = false;
    uint32_t e = 0;
    R dx = 0, dy = 0, dz = 0;
    if (c < cnt) {
      e = a.short_nb[(size_t)i * MAXSHORT + c];
      int j, sx, sy, sz;
      decode_entry(e, a.lc, j, sx, sy, sz);
      long long jinfo;
      ai.disp(a.A, sd, j, sx, sy, sz, dx, dy, dz, jinfo);
      R rsq = rsqR(dx, dy, dz);
      int tj = info_type(jinfo);
      if (ie >= 0 && info_mol(jinfo) == mi) {
        int je = c_pot.i_map[tj];
        if (je >= 0 && rsq != R(0)) {
          int pe = ie * MAXELEM + je;
          take_ilp = lt_exact(rsq, c_pot.i_cutILPsq[pe], a.A.xq, sd, i, j, sx, sy, sz, cutILPsq64[pe]);
        }
      }
      if (te >= 0 && c_pot.t_map[tj] >= 0)
        take_ters = lt_exact(rsq, c_pot.t_cutmaxsq, a.A.xq, sd, i, j, sx, sy, sz, tcutmaxsq64);
    }
    unsigned bi, bt;
    if constexpr (SG == 1) {
      bi = take_ilp;
      bt = take_ters;
    } else {
      bi = __ballot_sync(gmask, take_ilp) & gmask;
      bt = __ballot_sync(gmask, take_ters) & gmask;
    }
    if (take_ilp) {
      const int pos = nilp + __popc(bi & below);
      if (pos < MAXILP) a.ilp_nb[(size_t)i * MAXILP + pos] = e;
    }
    if (take_ters) {
      const int pos = nters + __popc(bt & below);
      if (pos < MAXTERS) a.ters_nb[(size_t)i * MAXTERS + pos] = e;
    }
    // constant indices keep the bond vectors in registers
#pragma unroll
    for (int q = 0; q < MAXILP; q++) {
      if (q >= nilp && q < nilp + __popc(bi)) {   // the same in every lane of the atom
        if constexpr (SG == 1) {
          vx[q] = -dx;
          vy[q] = -dy;
          vz[q] = -dz;
        } else {
          unsigned m = bi;   // the (q - nilp)-th accepting lane
          for (int t = nilp; t < q; t++) m &= m - 1;
          const int src = __ffs(m) - 1;
          vx[q] = -__shfl_sync(gmask, dx, src);
          vy[q] = -__shfl_sync(gmask, dy, src);
          vz[q] = -__shfl_sync(gmask, dz, src);
        }
      }
    }
    nilp += __popc(bi);
    nters += __popc(bt);
  }
  if ((wl & (SG - 1)) != 0) return;
  if (nilp > MAXILP) {
    raise_status(a.status, ST_TOO_MANY_ILP);
    nilp = MAXILP;
  }
  if (nters > MAXTERS) {
    raise_status(a.status, ST_TERS_OVERFLOW);
    nters = MAXTERS;
  }
  a.ilp_cnt[i] = nilp;
  a.ters_cnt[i] = nters;
  // unit normal
  R nx = 0, ny = 0, nz = 1;
  if (nilp >= 2) {
    R n1x = vy[0] * vz[1] - vy[1] * vz[0];
    R n1y = vz[0] * vx[1] - vz[1] * vx[0];
    R n1z = vx[0] * vy[1] - vx[1] * vy[0];
    if (nilp == 3) {
      // (v1 x v2 + v3 x v1 + v2 x v3) / 3
      n1x += vy[2] * vz[0] - vy[0] * vz[2];
      n1y += vz[2] * vx[0] - vz[0] * vx[2];
      n1z += vx[2] * vy[0] - vx[0] * vy[2];
      n1x += vy[1] * vz[2] - vy[2] * vz[1];
      n1y += vz[1] * vx[2] - vz[2] * vx[1];
      n1z += vx[1] * vy[2] - vx[2] * vy[1];
      n1x /= R(3); n1y /= R(3); n1z /= R(3);
    }
    R nn = Math<R>::sqrt_(n1x * n1x + n1y * n1y + n1z * n1z);
    if (nn == R(0)) {
      raise_status(a.status, ST_ZERO_NORMAL);
    } else {
      nx = n1x / nn; ny = n1y / nn; nz = n1z / nn;
    }
  }
#ifdef LMFF_PACKED_X2
  a.nrm32[i] = make_float4(nx, ny, nz, 0.f);
  a.jrec[3 * (size_t)i] = make_float4(ai.hx, ai.hy, ai.hz, __int_as_float((int)ai.info));
  a.jrec[3 * (size_t)i + 1] = make_float4(ai.lx, ai.ly, ai.lz, 0.f);
  a.jrec[3 * (size_t)i + 2] = make_float4(nx, ny, nz, 0.f);
  a.jrec2[2 * (size_t)i] = make_float4(ai.hx, ai.hy, ai.hz, __uint_as_float(h2_bits(__floats2half2_rn(ai.lx, ai.ly))));
  a.jrec2[2 * (size_t)i + 1] = make_float4(
      nx, ny, nz, __uint_as_float((h2_bits(__floats2half2_rn(ai.lz, 0.f)) & 0xffffu) | ((unsigned)(ie & 0xffff) << 16)));
#else
  a.nrm64[i] = make_d4(nx, ny, nz, 0.0);
#endif
}

// ============================================================ Tersoff math ========
// pair_tersoff.cpp:663-734 and pair_tersoff.h:90-107, in R
__device__ __forceinline__ void ters_fc_both(R r, const TersP<R> &p, R &fc, R &fcd) {
  if (r < p.rlo) { fc = R(1); fcd = R(0); return; }
  if (r > p.rhi) { fc = R(0); fcd = R(0); return; }
  R s, c;
  Math<R>::sincospi_(R(0.5) * (r - p.bigr) / p.bigd, &s, &c);
  fc = R(0.5) * (R(1) - s);
  fcd = -p.pi4_over_D * c;
}

__device__ __forceinline__ R ters_fc(R r, const TersP<R> &p) {
  R fc, fcd;
  ters_fc_both(r, p, fc, fcd);
  return fc;
}

__device__ __forceinline__ R ters_gijk(R costheta, const TersP<R> &p) {
  R hcth = p.h - costheta;
  if constexpr (sizeof(R) == 8) {
    return p.gamma * (R(1) + p.cd2 - p.c2 / (p.d2 + hcth * hcth));
  } else {
    // c^2/d^2 - c^2/(d^2 + u^2) = c^2 u^2 / (d^2 (d^2 + u^2)): the same value without the
    // cancellation of two ~1e8 terms (BNC.tersoff carbon) that FP32 cannot afford
    R u2 = hcth * hcth;
    return p.gamma * (R(1) + p.c2 * u2 / (p.d2 * (p.d2 + u2)));
  }
}

__device__ __forceinline__ R ters_gijk_d(R costheta, const TersP<R> &p) {
  R hcth = p.h - costheta;
  R numerator = R(-2) * p.c2 * hcth;
  R den = R(1) / (p.d2 + hcth * hcth);
  return p.gamma * numerator * den * den;
}

// g(theta) and dg/dcos(theta) from u = h - cos(theta) (FP32 mode: u comes from an FP64
// cosine, since h - cos(theta) cancels to ~0.07 for carbon)
__device__ __forceinline__ R ters_g_u(R u, const TersP<R> &p) {
  R u2 = u * u;
  return p.gamma * (R(1) + p.c2 * u2 / (p.d2 * (p.d2 + u2)));
}

__device__ __forceinline__ R ters_gd_u(R u, const TersP<R> &p) {
  R den = R(1) / (p.d2 + u * u);
  return p.gamma * (R(-2) * p.c2 * u) * den * den;
}

__device__ __forceinline__ R ters_exdelr(R rij, R rik, const TersP<R> &p) {
  R arg = p.powermint == 3 ? (p.lam3 * (rij - rik)) * (p.lam3 * (rij - rik)) * (p.lam3 * (rij - rik))
                           : p.lam3 * (rij - rik);
  if (arg > R(69.0776)) return R(1.e30);
  if (arg < R(-69.0776)) return R(0);
  return Math<R>::ex(arg);
}

__device__ __forceinline__ R ters_bij(R zeta, const TersP<R> &p) {
  R tmp = p.beta * zeta;
  if (tmp > p.c1) return R(1) / Math<R>::sqrt_(tmp);
  if (tmp > p.c2t) return (R(1) - Math<R>::pow_(tmp, -p.powern) * p.inv2n) / Math<R>::sqrt_(tmp);
  if (tmp < p.c4) return R(1);
  if (tmp < p.c3) return R(1) - Math<R>::pow_(tmp, p.powern) * p.inv2n;
  return Math<R>::pow_(R(1) + Math<R>::pow_(tmp, p.powern), -p.inv2n);
}

__device__ __forceinline__ R ters_bij_d(R zeta, const TersP<R> &p) {
  R tmp = p.beta * zeta;
  if (tmp > p.c1) return p.beta * R(-0.5) * Math<R>::pow_(tmp, R(-1.5));
  if (tmp > p.c2t)
    return p.beta * (R(-0.5) * Math<R>::pow_(tmp, R(-1.5)) *
                     (R(1) - (R(1) + p.inv2n) * Math<R>::pow_(tmp, -p.powern)));
  if (tmp < p.c4) return R(0);
  if (tmp < p.c3) return R(-0.5) * p.beta * Math<R>::pow_(tmp, p.powern - R(1));
  R tmp_n = Math<R>::pow_(tmp, p.powern);
  return R(-0.5) * Math<R>::pow_(R(1) + tmp_n, R(-1) - p.inv2n) * tmp_n / zeta;
}

// tag-parity half selection of a full list (pair_tersoff.cpp:150-158,
// pair_ilp_graphene_hbn.cpp:488-496); with periodic images the coordinate tie-break of
// equal tags compares the image shift lexicographically on (z, y, x)
__device__ __forceinline__ bool keep_half(long long itag, long long jtag, int sx, int sy, int sz) {
  if (itag > jtag) return ((itag + jtag) & 1) != 0;
  if (itag < jtag) return ((itag + jtag) & 1) == 0;
  if (sz != 0) return sz > 0;
  if (sy != 0) return sy > 0;
  return sx > 0;
}
// the same selection with the reference's own tie-break for equal tags (a ghost copy of
// an atom's owner): compare the coordinates of j against i on (z, y, x), r = x_j - x_i
template <class T>
__device__ __forceinline__ bool keep_half_r(long long itag, long long jtag, T rx, T ry, T rz) {
  if (itag > jtag) return ((itag + jtag) & 1) != 0;
  if (itag < jtag) return ((itag + jtag) & 1) == 0;
  if (rz != T(0)) return rz > T(0);
  if (ry != T(0)) return ry > T(0);
  return rx > T(0);
}
// subdomain mode: whether sorted atom s is owned
__device__ __forceinline__ bool owned(const ForceArgs<R> &a, int s) { return a.own_perm[s] < a.nown; }

// ============================================================ k_tersoff ==========
// One thread per centre atom i: the bonds i-j it centres (zeta over k, force_zeta,
// attractive over k, pair_tersoff.cpp:181-258) and the repulsion of every bond from i's
// end (:132-175).  Forces on bond partners go to ters_g slots (gathered in k_finish).
//
// Precision: the radial bond terms (repulsion A e^{-lam1 r} and the attraction
// b_ij f_A(r), which nearly cancel at the equilibrium bond length) keep FP64 accuracy in
// both modes, from FP64 displacements (in FP32 mode through exp_x32 and rsqrt_nr below,
// ~1e-9 relative); b_ij enters as 1 + delta with delta computed as
// expm1(-log1p((beta zeta)^n)/(2n)), which keeps its full relative accuracy in FP32.
// zeta, g(theta) and the three-body derivatives are evaluated in R.
__device__ __forceinline__ void ters_fc_both64(double r, const TersP<R> &p, double &fc, double &fcd) {
  if (r < p.rlo64) { fc = 1.0; fcd = 0.0; return; }
  if (r > p.rhi64) { fc = 0.0; fcd = 0.0; return; }
  double s, c;
  sincospi(0.5 * (r - p.R64) / p.D64, &s, &c);
  fc = 0.5 * (1.0 - s);
  fcd = -p.pi4D64 * c;
}

// b_ij - 1 and db_ij/dzeta (ters_bij, ters_bij_d, pair_tersoff.cpp:704-734)
__device__ __forceinline__ void ters_bij_delta(R zeta, const TersP<R> &p, double &bm1, R &bd) {
  R tmp = p.beta * zeta;
  if (tmp > p.c1) {
    bm1 = (double)(R(1) / Math<R>::sqrt_(tmp)) - 1.0;
    bd = p.beta * R(-0.5) * Math<R>::pow_(tmp, R(-1.5));
    return;
  }
  if (tmp > p.c2t) {
    bm1 = (double)((R(1) - Math<R>::pow_(tmp, -p.powern) * p.inv2n) / Math<R>::sqrt_(tmp)) - 1.0;
    bd = p.beta * (R(-0.5) * Math<R>::pow_(tmp, R(-1.5)) * (R(1) - (R(1) + p.inv2n) * Math<R>::pow_(tmp, -p.powern)));
    return;
  }
  if (tmp < p.c4) {
    bm1 = 0.0;
    bd = R(0);
    return;
  }
  if (tmp < p.c3) {
    R tn = Math<R>::pow_(tmp, p.powern);
    bm1 = -(double)(tn * p.inv2n);
    bd = R(-0.5) * p.beta * Math<R>::pow_(tmp, p.powern - R(1));
    return;
  }
  R tmp_n = Math<R>::pow_(tmp, p.powern);
  if constexpr (sizeof(R) == 8) {
    bm1 = pow(1.0 + tmp_n, -p.inv2n) - 1.0;
  } else {
    bm1 = (double)expm1f(-log1pf(tmp_n) * p.inv2n);
  }
  bd = R(-0.5) * Math<R>::pow_(R(1) + tmp_n, R(-1) - p.inv2n) * tmp_n / zeta;
}

// ---- FP32-mode radial helpers: the bond terms keep FP64 accuracy with a fraction of the
// FP64 instructions of sqrt, division and exp (the FP64 pipe runs at 1/64 of the FP32
// rate on this GPU).
//
// e^x by Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15, 1989): with
// t = 32 x = k + f, k = rint(t), |f| <= 1/2, e^x = e^{k/32} e^{f/32}.  e^{k/32} comes
// from a table of FP64 values; e^{f/32} - 1 (|f/32| <= 1/64) from its Taylor series to
// 4th order in FP32 (truncation < 1e-11, rounding ~3e-9 of the result).
constexpr int EXP_TAB_N = 1024;   // e^{-m/32}, m = 0..1023: arguments down to -31.97
__device__ double g_exptab[EXP_TAB_N];

__global__ void k_fill_exptab() {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < EXP_TAB_N) g_exptab[m] = exp(-(double)m / 32.0);
}

// e^{t/32} with t = r c given as FP32 pairs r = rh + rl, c = ch + cl (|rl| <= ulp(rh)/2,
// |cl| <= ulp(ch)/2): the product's rounding error is recovered exactly with an FMA
// (Dekker's error-free product), so f = t - k is accurate to ~3e-8 without FP64 work.
__device__ __forceinline__ double exp_x32f(float rh, float rl, float ch, float cl) {
  const float th = __fmul_rn(rh, ch);
  const float te = __fmaf_rn(rh, ch, -th);
  const float k = rintf(th);
  const float f = __fadd_rn(__fsub_rn(th, k), te + __fmaf_rn(rh, cl, rl * ch));
  const int m = -(int)k;
  if (m < 0 || m >= EXP_TAB_N) return exp(((double)rh + (double)rl) * ((double)ch + (double)cl) * 0.03125);
  const float x = f * 0.03125f;
  const float q = x * (1.f + x * (0.5f + x * (1.f / 6.f + x * (1.f / 24.f))));
  const double T = __ldg(&g_exptab[m]);
  return fma(T, (double)q, T);
}

// 1/sqrt(x) for x in the FP32 normal range: FP32 estimate and one FP64 Newton step
// (relative error ~1e-13)
__device__ __forceinline__ double rsqrt_nr(double x) {
  const double y = (double)rsqrt_ftz((float)x);
  const double e = fma(-(x * y), y, 1.0);
  return fma(0.5 * y, e, y);
}

// ---- FP32 double-float arithmetic (error-free transformations: Knuth's TwoSum, the
// FMA-based TwoProduct) for the FP32 mode's bond geometry: lengths and cosines to
// ~1e-13 relative from the hi/lo position parts, with no FP64 instruction.
__device__ __forceinline__ void ef_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) = a . b for vectors a = ah + al, b = bh + bl with |al| << |ah|, |bl| << |bh|
__device__ __forceinline__ void df_dot3(const float *ah, const float *al, const float *bh, const float *bl, float &sh,
                                        float &sl) {
  const float p0 = __fmul_rn(ah[0], bh[0]), e0 = __fmaf_rn(ah[0], bh[0], -p0);
  const float p1 = __fmul_rn(ah[1], bh[1]), e1 = __fmaf_rn(ah[1], bh[1], -p1);
  const float p2_ = __fmul_rn(ah[2], bh[2]), e2 = __fmaf_rn(ah[2], bh[2], -p2_);
  float s0, t1, s1, t2;
  ef_two_sum(p0, p1, s0, t1);
  ef_two_sum(s0, p2_, s1, t2);
  float lo = __fadd_rn(__fadd_rn(e0, e1), __fadd_rn(e2, __fadd_rn(t1, t2)));
  lo = __fmaf_rn(ah[0], bl[0], __fmaf_rn(al[0], bh[0], lo));
  lo = __fmaf_rn(ah[1], bl[1], __fmaf_rn(al[1], bh[1], lo));
  lo = __fmaf_rn(ah[2], bl[2], __fmaf_rn(al[2], bh[2], lo));
  sh = __fadd_rn(s1, lo);
  sl = __fsub_rn(lo, __fsub_rn(sh, s1));
}

// One centre atom's bonds.  NB is the number of bond slots held in registers (loops
// fully unrolled when NB is small; cnt <= NB).
//
// FP32 mode keeps the FP64 pipe (1/64 of the FP32 rate) for what needs it: positions,
// bond lengths, the radial terms' final products and the force sums.  Cut-off tests run
// on FP32 bond lengths (every term vanishes continuously at its cut-off), h - cos(theta)
// is formed in FP64 once per bond pair, and the three-body forces on each partner are
// summed in FP32 before one FP64 addition.
// GH (subdomain mode): a bond's repulsion counts when the end the tag-parity half keeps
// is owned, the bond-order terms when the centre i is owned.
// VA (per-atom virial, FP64 instantiation only): the virial split over atoms as the
// reference tallies it -- ev_tally of the repulsion and of force_zeta's pair force, half
// to each end (pair_tersoff.cpp:173, :223), v_tally3 of each triplet, a third to each of
// i, j, k (:253).  i's shares go to va_t[i]; its partners' shares to i's per-bond slots
// va_ts, which the per-atom virial gather collects.
template <int NB, bool EV, bool GH, bool VA = false>
__device__ __forceinline__ void tersoff_atom(const ForceArgs<R> &a, int i, int ie, int cnt) {
  constexpr bool F32 = sizeof(R) == 4;
  constexpr int UNR = NB <= 4 ? NB : 1;
  const SysDesc &sd = a.A.sys[a.A.sysid[i]];
  double dxd[NB], dyd[NB], dzd[NB], r64[NB], ri64[NB], rs64[NB];
  R dx[NB], dy[NB], dz[NB], rf[NB], rl[NB];
  float vh[NB][3], vl[NB][3];   // FP32 mode: delr as hi + lo parts
  int el[NB];
  uint32_t ev_[NB];
  // radial force on each partner (gx), three-body forces on each partner (tx), bond energy
  double gx[NB], gy[NB], gz[NB], ge[NB];
  R tx[NB], ty[NB], tz[NB];
  float cq0[NB][NB], cq1[NB][NB];   // FP32 mode: cos(theta_jik) of each bond pair as hi + lo
  R uf[NB][NB];          // FP32 mode: h_ijk - cos(theta_jik)
  double fx = 0, fy = 0, fz = 0, eng = 0;
  double v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
  double vo[6] = {0, 0, 0, 0, 0, 0};   // VA: i's own share
  double vs[VA ? NB : 1][6];           // VA: the shares of i's bond partners
  if constexpr (VA) {
#pragma unroll UNR
    for (int s = 0; s < NB; s++)
#pragma unroll
      for (int c = 0; c < 6; c++) vs[s][c] = 0.0;
  }
#pragma unroll UNR
  for (int s = 0; s < NB; s++) {
    if (s < cnt) {
      const uint32_t e = a.ters_nb[(size_t)i * MAXTERS + s];
      int j, sx, sy, sz;
      decode_entry(e, a.lc, j, sx, sy, sz);
      if constexpr (F32) {
        // delr = x_j(image) - x_i from the double-float position parts: the hi sum is
        // exact (a small multiple of the hi parts' ulp, one FMA), the lo sum carries the
        // rest; |delr| as an FP32 pair from a double-float dot and one Newton step
        const float4 hi4 = a.A.xh[i], lo4 = a.A.xl[i];
        const float4 hj = __ldg(&a.A.xh[j]), lj = __ldg(&a.A.xl[j]);
        const float fsx = (float)sx, fsy = (float)sy, fsz = (float)sz;
        vh[s][0] = __fmaf_rn(fsx, sd.Lhi[0], __fsub_rn(hj.x, hi4.x));
        vh[s][1] = __fmaf_rn(fsy, sd.Lhi[1], __fsub_rn(hj.y, hi4.y));
        vh[s][2] = __fmaf_rn(fsz, sd.Lhi[2], __fsub_rn(hj.z, hi4.z));
        vl[s][0] = __fmaf_rn(fsx, sd.Llo[0], __fsub_rn(lj.x, lo4.x));
        vl[s][1] = __fmaf_rn(fsy, sd.Llo[1], __fsub_rn(lj.y, lo4.y));
        vl[s][2] = __fmaf_rn(fsz, sd.Llo[2], __fsub_rn(lj.z, lo4.z));
        float sh, sl;
        df_dot3(vh[s], vl[s], vh[s], vl[s], sh, sl);
        const float ri0 = rsqrt_ftz(sh);
        const float r0 = __fmul_rn(sh, ri0);
        const float corr = __fmul_rn(__fadd_rn(__fmaf_rn(-r0, r0, sh), sl), __fmul_rn(0.5f, ri0));
        const float rh = __fadd_rn(r0, corr);
        rf[s] = rh;
        rl[s] = __fsub_rn(corr, __fsub_rn(rh, r0));
        ri64[s] = (double)__fmaf_rn(__fmul_rn(-corr, ri0), ri0, ri0);
        dx[s] = __fadd_rn(vh[s][0], vl[s][0]);
        dy[s] = __fadd_rn(vh[s][1], vl[s][1]);
        dz[s] = __fadd_rn(vh[s][2], vl[s][2]);
        dxd[s] = (double)dx[s]; dyd[s] = (double)dy[s]; dzd[s] = (double)dz[s];
        el[s] = c_pot.t_map[info_type((long long)__float_as_int(hj.w))];
      } else {
        double ddx, ddy, ddz;
        disp64(a.A.xq, sd, i, j, sx, sy, sz, ddx, ddy, ddz);
        dxd[s] = -ddx; dyd[s] = -ddy; dzd[s] = -ddz;  // delr = x_j - x_i
        const double rs = rsq_rn(ddx, ddy, ddz);
        rs64[s] = rs;
        r64[s] = sqrt(rs);
        ri64[s] = 0.0;
        rf[s] = r64[s];
        rl[s] = 0.0;
        dx[s] = (R)dxd[s]; dy[s] = (R)dyd[s]; dz[s] = (R)dzd[s];
        el[s] = c_pot.t_map[info_type(__double_as_longlong(a.A.xq[j].w))];
      }
      ev_[s] = e;
      gx[s] = gy[s] = gz[s] = ge[s] = 0.0;
      tx[s] = ty[s] = tz[s] = R(0);
    }
  }
  if constexpr (F32) {
#pragma unroll UNR
    for (int s = 0; s < NB; s++) {
#pragma unroll UNR
      for (int k = s + 1; k < NB; k++) {
        if (k < cnt) {
          // cos = delr_s . delr_k / (r_s r_k) in double-float: q0 + q1
          float Dh, Dl;
          df_dot3(vh[s], vl[s], vh[k], vl[k], Dh, Dl);
          const float nh = __fmul_rn(rf[s], rf[k]);
          const float nl = __fmaf_rn(rf[s], rl[k], __fmaf_rn(rl[s], rf[k], __fmaf_rn(rf[s], rf[k], -nh)));
          const float inv = rcp_ftz(nh);
          const float q0 = __fmul_rn(Dh, inv);
          const float q1 = __fmul_rn(__fadd_rn(__fmaf_rn(-q0, nh, Dh), __fmaf_rn(-q0, nl, Dl)), inv);
          cq0[s][k] = cq0[k][s] = q0;
          cq1[s][k] = cq1[k][s] = q1;
        }
      }
    }
  }
  const long long itag = (c_pot.rep_sym && !GH) ? 0 : a.tag[i];
  const bool iown = !GH || owned(a, i);
#pragma unroll UNR
  for (int s = 0; s < NB; s++) {
    if (s >= cnt) continue;
    const int je = el[s];
    const TersP<R> &pij = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + je];
    const R rR = rf[s];
    // FP64 bond length: the FP64 path's own; the FP32 path needs it only inside the
    // cut-off function's transition region
    const double r = F32 ? (double)rf[s] + (double)rl[s] : r64[s];
    double fr = 0.0;   // radial force on i along delr, from both terms of this bond
    // ---- repulsion (:584-595) in FP64, from both ends of the bond, with the parameters
    // of the end the reference's half list keeps
    {
      const TersP<R> *pr = &pij;
      bool rep_on = true;
      if (!c_pot.rep_sym || GH) {
        int j, sx, sy, sz;
        decode_entry(ev_[s], a.lc, j, sx, sy, sz);
        const bool keep = GH ? keep_half_r(itag, a.tag[j], dxd[s], dyd[s], dzd[s]) : keep_half(itag, a.tag[j], sx, sy, sz);
        if (!keep && !c_pot.rep_sym) pr = &c_pot.ters[(je * MAXELEM + ie) * MAXELEM + ie];
        if (GH) rep_on = keep ? iown : owned(a, j);
      }
      if (rep_on && (F32 ? rR < pr->rhi : rs64[s] < pr->cutsq64)) {
        double tmp_exp, fpair, fc;
        if constexpr (F32) {
          tmp_exp = exp_x32f(rR, rl[s], pr->nl1h, pr->nl1l);
          if (rR < pr->rlo) {   // fc = 1, fc' = 0
            fc = 1.0;
            fpair = pr->Al1_64 * tmp_exp * ri64[s];
          } else {
            double fcd;
            ters_fc_both64(r, *pr, fc, fcd);
            fpair = -pr->A64 * tmp_exp * (fcd - fc * pr->lam1_64) * ri64[s];
          }
        } else {
          double fcd;
          ters_fc_both64(r, *pr, fc, fcd);
          tmp_exp = exp(-pr->lam1_64 * r);
          fpair = -pr->A64 * tmp_exp * (fcd - fc * pr->lam1_64) / r;
        }
        fr -= fpair;
        if constexpr (VA) {
          // ev_tally(i, j, .., fpair, del): del (x) del fpair, half to this end
          const double w[6] = {dxd[s] * dxd[s] * fpair, dyd[s] * dyd[s] * fpair, dzd[s] * dzd[s] * fpair,
                               dxd[s] * dyd[s] * fpair, dxd[s] * dzd[s] * fpair, dyd[s] * dzd[s] * fpair};
#pragma unroll
          for (int c = 0; c < 6; c++) vo[c] += 0.5 * w[c];
        }
        if (EV) {
          eng += 0.5 * fc * pr->A64 * tmp_exp;
          double h = 0.5 * fpair;
          v0 += h * dxd[s] * dxd[s]; v1 += h * dyd[s] * dyd[s]; v2 += h * dzd[s] * dzd[s];
          v3 += h * dxd[s] * dyd[s]; v4 += h * dxd[s] * dzd[s]; v5 += h * dyd[s] * dzd[s];
        }
      }
    }
    if (!iown || !(F32 ? rR < pij.rhi : rs64[s] < pij.cutsq64)) {
      fx += dxd[s] * fr; fy += dyd[s] * fr; fz += dzd[s] * fr;
      continue;
    }
    // ---- zeta_ij over k (:197-210), in R
    R zeta = 0;
#pragma unroll UNR
    for (int k = 0; k < NB; k++) {
      if (k == s || k >= cnt) continue;
      const TersP<R> &pk = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + el[k]];
      const R rik = rf[k];
      if (!(F32 ? rik < pk.rhi : rs64[k] < pk.cutsq64)) continue;
      R ex = pk.lam3 == R(0) ? R(1) : ters_exdelr(rR, rik, pk);
      R g;
      if constexpr (F32) {
        uf[s][k] = __fadd_rn(__fsub_rn(pk.hhi, cq0[s][k]), __fsub_rn(pk.hlo, cq1[s][k]));
        g = ters_g_u(uf[s][k], pk);
      } else {
        R cost = (dx[s] * dx[k] + dy[s] * dy[k] + dz[s] * dz[k]) / (rR * rik);
        g = ters_gijk(cost, pk);
      }
      zeta += ters_fc(rik, pk) * g * ex;
    }
    // ---- force_zeta (:621-634): radial part in FP64
    double fa = 0.0, fa_d = 0.0;
    if constexpr (F32) {
      const double ex2 = exp_x32f(rR, rl[s], pij.nl2h, pij.nl2l);
      if (rR < pij.rlo) {   // fc = 1, fc' = 0
        fa = -pij.B64 * ex2;
        fa_d = pij.Bl2_64 * ex2;
      } else {
        double fc, fcd;
        ters_fc_both64(r, pij, fc, fcd);
        fa = -pij.B64 * ex2 * fc;
        fa_d = pij.B64 * ex2 * (pij.lam2_64 * fc - fcd);
      }
    } else {
      double fc, fcd;
      ters_fc_both64(r, pij, fc, fcd);
      if (!(r > pij.rhi64)) {
        double ex2 = exp(-pij.lam2_64 * r);
        fa = -pij.B64 * ex2 * fc;
        fa_d = pij.B64 * ex2 * (pij.lam2_64 * fc - fcd);
      }
    }
    double bm1;
    R bd;
    ters_bij_delta(zeta, pij, bm1, bd);
    const double bij = 1.0 + bm1;
    const double fpair = F32 ? 0.5 * bij * fa_d * ri64[s] : 0.5 * bij * fa_d / r;
    const R prefactor = (R)(-0.5 * fa) * bd;
    fr += fpair;
    fx += dxd[s] * fr; fy += dyd[s] * fr; fz += dzd[s] * fr;
    const double fjx = -dxd[s] * fpair, fjy = -dyd[s] * fpair, fjz = -dzd[s] * fpair;
    gx[s] = fjx; gy[s] = fjy; gz[s] = fjz;   // the only radial contribution to partner s
    if constexpr (VA) {
      // ev_tally(i, j, .., -fpair, -delr1): half to i, half to j
      const double w[6] = {dxd[s] * fjx, dyd[s] * fjy, dzd[s] * fjz, dxd[s] * fjy, dxd[s] * fjz, dyd[s] * fjz};
#pragma unroll
      for (int c = 0; c < 6; c++) {
        vo[c] += 0.5 * w[c];
        vs[s][c] += 0.5 * w[c];
      }
    }
    if (EV) {
      double eb = 0.5 * bij * fa;
      eng += eb;
      ge[s] += eb;
      v0 += dxd[s] * fjx; v1 += dyd[s] * fjy; v2 += dzd[s] * fjz;
      v3 += dxd[s] * fjy; v4 += dxd[s] * fjz; v5 += dyd[s] * fjz;
    }
    // ---- attractive over k (:228-254) -> ters_zetaterm_d (:738-793), in R.  The force
    // on i is minus the forces on j and k (:766-774); it is taken from the partners'
    // three-body totals after the loop.
    if (prefactor != R(0)) {
      R rinv = R(1) / rR;
      R rhx = dx[s] * rinv, rhy = dy[s] * rinv, rhz = dz[s] * rinv;
      R ajx = 0, ajy = 0, ajz = 0;
#pragma unroll UNR
      for (int k = 0; k < NB; k++) {
        if (k == s || k >= cnt) continue;
        const TersP<R> &pk = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + el[k]];
        const R rik = rf[k];
        if (!(F32 ? rik < pk.rhi : rs64[k] < pk.cutsq64)) continue;
        R rikinv = R(1) / rik;
        R khx = dx[k] * rikinv, khy = dy[k] * rikinv, khz = dz[k] * rikinv;
        R fck, dfck;
        ters_fc_both(rik, pk, fck, dfck);
        R exd, exd_d;
        if (pk.lam3 == R(0)) {
          exd = R(1);
          exd_d = R(0);
        } else {
          exd = ters_exdelr(rR, rik, pk);
          exd_d = pk.powermint == 3 ? R(3) * pk.lam3 * pk.lam3 * pk.lam3 * (rR - rik) * (rR - rik) * exd
                                    : pk.lam3 * exd;
        }
        R cs = rhx * khx + rhy * khy + rhz * khz;
        R g, gd;
        if constexpr (F32) {
          g = ters_g_u(uf[s][k], pk);
          gd = ters_gd_u(uf[s][k], pk);
        } else {
          g = ters_gijk(cs, pk);
          gd = ters_gijk_d(cs, pk);
        }
        // costheta_d (:797-811)
        R djx = (-cs * rhx + khx) * rinv, djy = (-cs * rhy + khy) * rinv, djz = (-cs * rhz + khz) * rinv;
        R dkx = (-cs * khx + rhx) * rikinv, dky = (-cs * khy + rhy) * rikinv, dkz = (-cs * khz + rhz) * rikinv;
        R A1 = fck * gd * exd, A2 = fck * g * exd_d, A3 = dfck * g * exd;
        R fkx_ = prefactor * (A3 * khx + A1 * dkx - A2 * khx);
        R fky_ = prefactor * (A3 * khy + A1 * dky - A2 * khy);
        R fkz_ = prefactor * (A3 * khz + A1 * dkz - A2 * khz);
        ajx += prefactor * (A1 * djx + A2 * rhx);
        ajy += prefactor * (A1 * djy + A2 * rhy);
        ajz += prefactor * (A1 * djz + A2 * rhz);
        tx[k] += fkx_; ty[k] += fky_; tz[k] += fkz_;
        if constexpr (VA) {
          // v_tally3(i, j, k, fj, fk, delr1, delr2): a third to each of i, j, k
          const double third = 1.0 / 3.0;
          const double fjx_ = prefactor * (A1 * djx + A2 * rhx), fjy_ = prefactor * (A1 * djy + A2 * rhy),
                       fjz_ = prefactor * (A1 * djz + A2 * rhz);
          const double w[6] = {third * (dx[s] * fjx_ + dx[k] * fkx_), third * (dy[s] * fjy_ + dy[k] * fky_),
                               third * (dz[s] * fjz_ + dz[k] * fkz_), third * (dx[s] * fjy_ + dx[k] * fky_),
                               third * (dx[s] * fjz_ + dx[k] * fkz_), third * (dy[s] * fjz_ + dy[k] * fkz_)};
#pragma unroll
          for (int c = 0; c < 6; c++) {
            vo[c] += w[c];
            vs[s][c] += w[c];
            vs[k][c] += w[c];
          }
        }
        if (EV) {
          v0 += (double)(dx[k] * fkx_); v1 += (double)(dy[k] * fky_); v2 += (double)(dz[k] * fkz_);
          v3 += (double)(dx[k] * fky_); v4 += (double)(dx[k] * fkz_); v5 += (double)(dy[k] * fkz_);
        }
      }
      tx[s] += ajx; ty[s] += ajy; tz[s] += ajz;
      if (EV) {
        v0 += (double)(dx[s] * ajx); v1 += (double)(dy[s] * ajy); v2 += (double)(dz[s] * ajz);
        v3 += (double)(dx[s] * ajy); v4 += (double)(dx[s] * ajz); v5 += (double)(dy[s] * ajz);
      }
    }
  }
#pragma unroll UNR
  for (int s = 0; s < NB; s++) {
    if (s < cnt) {
      const double ux = (double)tx[s], uy = (double)ty[s], uz = (double)tz[s];
      fx -= ux; fy -= uy; fz -= uz;
      a.ters_g[(size_t)i * MAXTERS + s] = make_d4(gx[s] + ux, gy[s] + uy, gz[s] + uz, ge[s]);
    }
  }
  a.ters_f[i] = fx;
  a.ters_f[a.n + i] = fy;
  a.ters_f[2 * a.n + i] = fz;
  if constexpr (VA) {
#pragma unroll
    for (int c = 0; c < 6; c++) a.va_t[6 * (size_t)i + c] = vo[c];
#pragma unroll UNR
    for (int s = 0; s < NB; s++)
      if (s < cnt)
#pragma unroll
        for (int c = 0; c < 6; c++) a.va_ts[((size_t)i * MAXTERS + s) * 6 + c] = vs[s][c];
  }
  if (EV) {
    double *st = a.stat_ters;
    st[i] = eng;
    st[(size_t)a.n + i] = 0.0;
    st[(size_t)2 * a.n + i] = v0; st[(size_t)3 * a.n + i] = v1; st[(size_t)4 * a.n + i] = v2;
    st[(size_t)5 * a.n + i] = v3; st[(size_t)6 * a.n + i] = v4; st[(size_t)7 * a.n + i] = v5;
  }
}

// sp2 layers give 3 bonds per atom: those atoms run with their bonds in registers
template <bool EV, bool EATOM, bool GH, bool VA = false>
__global__ void __launch_bounds__(128) k_tersoff(ForceArgs<R> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const long long iinfo = __double_as_longlong(a.A.xq[i].w);
  const int ie = c_pot.t_map[info_type(iinfo)];
  const int cnt = ie < 0 ? 0 : a.ters_cnt[i];
  if (cnt <= 3) tersoff_atom<3, EV, GH, VA>(a, i, ie, cnt);
  else tersoff_atom<MAXTERS, EV, GH, VA>(a, i, ie, cnt);
}

// ---- Tersoff with one lane per bond (small systems) ---------------------------------
// TERS_LANES lanes per centre atom i, lane l taking bond l (an atom with more bonds runs
// the one-thread routine on its group's first lane).  Every lane builds the geometry of
// all of i's bonds, which the zeta and three-body loops need, then evaluates its own
// bond: repulsion, zeta_ij, b_ij and the three-body forces on the other partners.  The
// per-partner three-body sums and the force on i are then formed by shuffles in bond
// order on their owner lanes, the order of the one-thread routine.  For small systems,
// where one thread's walk over three bonds is the kernel's time, when Tersoff runs alone:
// beside the pair kernel its four times as many threads take issue slots from it (7,200
// atoms, per NVE step: Tersoff alone 30.3 -> 26.8 us, the two styles one after the other
// 56.1 -> 52.5 us, side by side 41.2 -> 43.1 us).  Force-only evaluations in periodic
// mode (the energy/virial and subdomain evaluations run k_tersoff).
constexpr int TERS_LANES = 4;
constexpr int TERS_LANES_MAX_ATOMS = 65536;
__global__ void __launch_bounds__(128) k_tersoff_lanes(ForceArgs<R> a) {
  constexpr int NB = TERS_LANES;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gtid / NB;
  if (i >= a.n) return;   // whole groups: blockDim is a multiple of NB
  const int wl = threadIdx.x & 31, l = wl & (NB - 1), gbase = wl & ~(NB - 1);
  const unsigned gmask = ((1u << NB) - 1) << gbase;
  const int ie = c_pot.t_map[info_type(__double_as_longlong(a.A.xq[i].w))];
  const int cnt = ie < 0 ? 0 : a.ters_cnt[i];
  if (cnt > NB) {   // the same in every lane of the group
    if (l == 0) tersoff_atom<MAXTERS, false, false>(a, i, ie, cnt);
    return;
  }
  constexpr bool F32 = sizeof(R) == 4;
  const SysDesc &sd = a.A.sys[a.A.sysid[i]];
  double dxd[NB], dyd[NB], dzd[NB], r64[NB], ri64[NB], rs64[NB];
  R dx[NB], dy[NB], dz[NB], rf[NB], rl[NB];
  float vh[NB][3], vl[NB][3];   // FP32 mode: delr as hi + lo parts
  int el[NB];
  uint32_t ev_[NB];
  float cq0[NB][NB], cq1[NB][NB];   // FP32 mode: cos(theta_jik) of each bond pair as hi + lo
#pragma unroll
  for (int s = 0; s < NB; s++) {
    if (s < cnt) {
      const uint32_t e = a.ters_nb[(size_t)i * MAXTERS + s];
      int j, sx, sy, sz;
      decode_entry(e, a.lc, j, sx, sy, sz);
      if constexpr (F32) {
        // delr = x_j(image) - x_i from the double-float position parts: the hi sum is
        // exact (a small multiple of the hi parts' ulp, one FMA), the lo sum carries the
        // rest; |delr| as an FP32 pair from a double-float dot and one Newton step
        const float4 hi4 = a.A.xh[i], lo4 = a.A.xl[i];
        const float4 hj = __ldg(&a.A.xh[j]), lj = __ldg(&a.A.xl[j]);
        const float fsx = (float)sx, fsy = (float)sy, fsz = (float)sz;
        vh[s][0] = __fmaf_rn(fsx, sd.Lhi[0], __fsub_rn(hj.x, hi4.x));
        vh[s][1] = __fmaf_rn(fsy, sd.Lhi[1], __fsub_rn(hj.y, hi4.y));
        vh[s][2] = __fmaf_rn(fsz, sd.Lhi[2], __fsub_rn(hj.z, hi4.z));
        vl[s][0] = __fmaf_rn(fsx, sd.Llo[0], __fsub_rn(lj.x, lo4.x));
        vl[s][1] = __fmaf_rn(fsy, sd.Llo[1], __fsub_rn(lj.y, lo4.y));
        vl[s][2] = __fmaf_rn(fsz, sd.Llo[2], __fsub_rn(lj.z, lo4.z));
        float sh, sl;
        df_dot3(vh[s], vl[s], vh[s], vl[s], sh, sl);
        const float ri0 = rsqrt_ftz(sh);
        const float r0 = __fmul_rn(sh, ri0);
        const float corr = __fmul_rn(__fadd_rn(__fmaf_rn(-r0, r0, sh), sl), __fmul_rn(0.5f, ri0));
        const float rh = __fadd_rn(r0, corr);
        rf[s] = rh;
        rl[s] = __fsub_rn(corr, __fsub_rn(rh, r0));
        ri64[s] = (double)__fmaf_rn(__fmul_rn(-corr, ri0), ri0, ri0);
        dx[s] = __fadd_rn(vh[s][0], vl[s][0]);
        dy[s] = __fadd_rn(vh[s][1], vl[s][1]);
        dz[s] = __fadd_rn(vh[s][2], vl[s][2]);
        dxd[s] = (double)dx[s]; dyd[s] = (double)dy[s]; dzd[s] = (double)dz[s];
        el[s] = c_pot.t_map[info_type((long long)__float_as_int(hj.w))];
      } else {
        double ddx, ddy, ddz;
        disp64(a.A.xq, sd, i, j, sx, sy, sz, ddx, ddy, ddz);
        dxd[s] = -ddx; dyd[s] = -ddy; dzd[s] = -ddz;  // delr = x_j - x_i
        const double rs = rsq_rn(ddx, ddy, ddz);
        rs64[s] = rs;
        r64[s] = sqrt(rs);
        ri64[s] = 0.0;
        rf[s] = r64[s];
        rl[s] = 0.0;
        dx[s] = (R)dxd[s]; dy[s] = (R)dyd[s]; dz[s] = (R)dzd[s];
        el[s] = c_pot.t_map[info_type(__double_as_longlong(a.A.xq[j].w))];
      }
      ev_[s] = e;
    }
  }
  if constexpr (F32) {
#pragma unroll
    for (int s = 0; s < NB; s++) {
#pragma unroll
      for (int k = s + 1; k < NB; k++) {
        if (k < cnt) {
          // cos = delr_s . delr_k / (r_s r_k) in double-float: q0 + q1
          float Dh, Dl;
          df_dot3(vh[s], vl[s], vh[k], vl[k], Dh, Dl);
          const float nh = __fmul_rn(rf[s], rf[k]);
          const float nl = __fmaf_rn(rf[s], rl[k], __fmaf_rn(rl[s], rf[k], __fmaf_rn(rf[s], rf[k], -nh)));
          const float inv = rcp_ftz(nh);
          const float q0 = __fmul_rn(Dh, inv);
          const float q1 = __fmul_rn(__fadd_rn(__fmaf_rn(-q0, nh, Dh), __fmaf_rn(-q0, nl, Dl)), inv);
          cq0[s][k] = cq0[k][s] = q0;
          cq1[s][k] = cq1[k][s] = q1;
        }
      }
    }
  }
  // this lane's bond, in scalars (a runtime index into the bond arrays would put them in
  // local memory)
  double mdx = 0, mdy = 0, mdz = 0, mr64 = 0, mri64 = 0, mrs64 = 0;
  R mxr = 0, myr = 0, mzr = 0, mrf = 1, mrl = 0;
  int mel = 0;
  uint32_t mev = 0;
  float mq0[NB], mq1[NB];
#pragma unroll
  for (int q = 0; q < NB; q++) {
    mq0[q] = 0.f;
    mq1[q] = 0.f;
  }
#pragma unroll
  for (int q = 0; q < NB; q++) {
    if (q == l && q < cnt) {
      mdx = dxd[q]; mdy = dyd[q]; mdz = dzd[q];
      mri64 = ri64[q];
      if constexpr (!F32) {
        mr64 = r64[q];
        mrs64 = rs64[q];
      }
      mxr = dx[q]; myr = dy[q]; mzr = dz[q];
      mrf = rf[q]; mrl = rl[q];
      mel = el[q];
      mev = ev_[q];
      if constexpr (F32) {
#pragma unroll
        for (int k = 0; k < NB; k++) {
          if (k != q) {
            mq0[k] = cq0[q][k];
            mq1[k] = cq1[q][k];
          }
        }
      }
    }
  }
  const long long itag = c_pot.rep_sym ? 0 : a.tag[i];
  double fr = 0.0, fjx = 0.0, fjy = 0.0, fjz = 0.0;
  R fkx[NB], fky[NB], fkz[NB];   // three-body force of this bond on partner k (k != l)
  R ajx = 0, ajy = 0, ajz = 0;   // ... on partner l
#pragma unroll
  for (int k = 0; k < NB; k++) fkx[k] = fky[k] = fkz[k] = R(0);
  if (l < cnt) {
    const int je = mel;
    const TersP<R> &pij = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + je];
    const R rR = mrf;
    const double r = F32 ? (double)mrf + (double)mrl : mr64;
    // ---- repulsion, from both ends of the bond, with the parameters of the end the
    // reference's half list keeps
    {
      const TersP<R> *pr = &pij;
      if (!c_pot.rep_sym) {
        int j, sx, sy, sz;
        decode_entry(mev, a.lc, j, sx, sy, sz);
        if (!keep_half(itag, a.tag[j], sx, sy, sz)) pr = &c_pot.ters[(je * MAXELEM + ie) * MAXELEM + ie];
      }
      if (F32 ? rR < pr->rhi : mrs64 < pr->cutsq64) {
        double tmp_exp, fpair, fc;
        if constexpr (F32) {
          tmp_exp = exp_x32f(rR, mrl, pr->nl1h, pr->nl1l);
          if (rR < pr->rlo) {
            fc = 1.0;
            fpair = pr->Al1_64 * tmp_exp * mri64;
          } else {
            double fcd;
            ters_fc_both64(r, *pr, fc, fcd);
            fpair = -pr->A64 * tmp_exp * (fcd - fc * pr->lam1_64) * mri64;
          }
        } else {
          double fcd;
          ters_fc_both64(r, *pr, fc, fcd);
          tmp_exp = exp(-pr->lam1_64 * r);
          fpair = -pr->A64 * tmp_exp * (fcd - fc * pr->lam1_64) / r;
        }
        fr -= fpair;
      }
    }
    if (F32 ? rR < pij.rhi : mrs64 < pij.cutsq64) {
      // ---- zeta_ij over k
      R zeta = 0;
      R ufk[NB];
#pragma unroll
      for (int k = 0; k < NB; k++) {
        ufk[k] = R(0);
        if (k == l || k >= cnt) continue;
        const TersP<R> &pk = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + el[k]];
        const R rik = rf[k];
        if (!(F32 ? rik < pk.rhi : rs64[k] < pk.cutsq64)) continue;
        R ex = pk.lam3 == R(0) ? R(1) : ters_exdelr(rR, rik, pk);
        R g;
        if constexpr (F32) {
          ufk[k] = __fadd_rn(__fsub_rn(pk.hhi, mq0[k]), __fsub_rn(pk.hlo, mq1[k]));
          g = ters_g_u(ufk[k], pk);
        } else {
          R cost = (mxr * dx[k] + myr * dy[k] + mzr * dz[k]) / (rR * rik);
          g = ters_gijk(cost, pk);
        }
        zeta += ters_fc(rik, pk) * g * ex;
      }
      // ---- force_zeta: radial part in FP64
      double fa = 0.0, fa_d = 0.0;
      if constexpr (F32) {
        const double ex2 = exp_x32f(rR, mrl, pij.nl2h, pij.nl2l);
        if (rR < pij.rlo) {
          fa = -pij.B64 * ex2;
          fa_d = pij.Bl2_64 * ex2;
        } else {
          double fc, fcd;
          ters_fc_both64(r, pij, fc, fcd);
          fa = -pij.B64 * ex2 * fc;
          fa_d = pij.B64 * ex2 * (pij.lam2_64 * fc - fcd);
        }
      } else {
        double fc, fcd;
        ters_fc_both64(r, pij, fc, fcd);
        if (!(r > pij.rhi64)) {
          double ex2 = exp(-pij.lam2_64 * r);
          fa = -pij.B64 * ex2 * fc;
          fa_d = pij.B64 * ex2 * (pij.lam2_64 * fc - fcd);
        }
      }
      double bm1;
      R bd;
      ters_bij_delta(zeta, pij, bm1, bd);
      const double bij = 1.0 + bm1;
      const double fpair = F32 ? 0.5 * bij * fa_d * mri64 : 0.5 * bij * fa_d / r;
      const R prefactor = (R)(-0.5 * fa) * bd;
      fr += fpair;
      fjx = -mdx * fpair; fjy = -mdy * fpair; fjz = -mdz * fpair;
      // ---- attractive over k -> ters_zetaterm_d, in R
      if (prefactor != R(0)) {
        R rinv = R(1) / rR;
        R rhx = mxr * rinv, rhy = myr * rinv, rhz = mzr * rinv;
#pragma unroll
        for (int k = 0; k < NB; k++) {
          if (k == l || k >= cnt) continue;
          const TersP<R> &pk = c_pot.ters[(ie * MAXELEM + je) * MAXELEM + el[k]];
          const R rik = rf[k];
          if (!(F32 ? rik < pk.rhi : rs64[k] < pk.cutsq64)) continue;
          R rikinv = R(1) / rik;
          R khx = dx[k] * rikinv, khy = dy[k] * rikinv, khz = dz[k] * rikinv;
          R fck, dfck;
          ters_fc_both(rik, pk, fck, dfck);
          R exd, exd_d;
          if (pk.lam3 == R(0)) {
            exd = R(1);
            exd_d = R(0);
          } else {
            exd = ters_exdelr(rR, rik, pk);
            exd_d = pk.powermint == 3 ? R(3) * pk.lam3 * pk.lam3 * pk.lam3 * (rR - rik) * (rR - rik) * exd
                                      : pk.lam3 * exd;
          }
          R cs = rhx * khx + rhy * khy + rhz * khz;
          R g, gd;
          if constexpr (F32) {
            g = ters_g_u(ufk[k], pk);
            gd = ters_gd_u(ufk[k], pk);
          } else {
            g = ters_gijk(cs, pk);
            gd = ters_gijk_d(cs, pk);
          }
          R djx = (-cs * rhx + khx) * rinv, djy = (-cs * rhy + khy) * rinv, djz = (-cs * rhz + khz) * rinv;
          R dkx = (-cs * khx + rhx) * rikinv, dky = (-cs * khy + rhy) * rikinv, dkz = (-cs * khz + rhz) * rikinv;
          R A1 = fck * gd * exd, A2 = fck * g * exd_d, A3 = dfck * g * exd;
          fkx[k] = prefactor * (A3 * khx + A1 * dkx - A2 * khx);
          fky[k] = prefactor * (A3 * khy + A1 * dky - A2 * khy);
          fkz[k] = prefactor * (A3 * khz + A1 * dkz - A2 * khz);
          ajx += prefactor * (A1 * djx + A2 * rhx);
          ajy += prefactor * (A1 * djy + A2 * rhy);
          ajz += prefactor * (A1 * djz + A2 * rhz);
        }
      }
    }
  }
  // ---- per-partner three-body sums on the partner's lane, in bond order: bond s gives
  // partner k (k != s) its fk and partner s its aj
  R tx = 0, ty = 0, tz = 0;
#pragma unroll
  for (int k = 0; k < NB; k++) {
#pragma unroll
    for (int s = 0; s < NB; s++) {
      const R vx = __shfl_sync(gmask, k == l ? ajx : fkx[k], gbase + s);
      const R vy = __shfl_sync(gmask, k == l ? ajy : fky[k], gbase + s);
      const R vz = __shfl_sync(gmask, k == l ? ajz : fkz[k], gbase + s);
      if (l == k && s < cnt) {
        tx += vx; ty += vy; tz += vz;
      }
    }
  }
  const double ux = (double)tx, uy = (double)ty, uz = (double)tz;
  if (l < cnt) a.ters_g[(size_t)i * MAXTERS + l] = make_d4(fjx + ux, fjy + uy, fjz + uz, 0.0);
  // ---- the force on i on lane 0: the radial terms, then minus the three-body totals
  double fx = 0, fy = 0, fz = 0;
#pragma unroll
  for (int s = 0; s < NB; s++) {
    const double frs = __shfl_sync(gmask, fr, gbase + s);
    if (s < cnt) {
      fx += dxd[s] * frs; fy += dyd[s] * frs; fz += dzd[s] * frs;
    }
  }
#pragma unroll
  for (int s = 0; s < NB; s++) {
    const double vx = __shfl_sync(gmask, ux, gbase + s);
    const double vy = __shfl_sync(gmask, uy, gbase + s);
    const double vz = __shfl_sync(gmask, uz, gbase + s);
    if (s < cnt) {
      fx -= vx; fy -= vy; fz -= vz;
    }
  }
  if (l == 0) {
    a.ters_f[i] = fx;
    a.ters_f[a.n + i] = fy;
    a.ters_f[2 * a.n + i] = fz;
  }
}


// ============================================================== k_ilp ============
// TPA lanes per atom i stride over i's interlayer list.  Per pair (del = x_i - x_j):
//   vdW (calc_FvdW :509-533) from both ends; repulsion of term (i,j) with n_i and of
//   term (j,i) with n_j (calc_FRep :602-647); g_i += Tap*prod*fpair1*del.
// Lane 0 of the group then applies the normal derivatives of i (calc_normal's dnormdri
// and dnormal, :893-926 / :1043-1067) to g_i in FP64: the force on i itself and the
// force on each intralayer neighbour (ilp_c slots).
// ONE: every ILP-mapped type is the same element, so the pair parameters are read at a
// compile-time constant index (constant-bank operands, no per-pair loads).
// Pairs a lane sums in R before the lanes' partial sums go into the atom's FP64
// totals (mixed precision: FP32 pair arithmetic, FP64 per-atom accumulation of forces,
// dE/dn_i, energies and virial).  A flush combines the TPA lanes' FP32 block sums
// (reduce-scatter by shuffles, 7 shuffles and adds per lane) and each lane adds the
// one or two totals it owns in FP64: two FP64 instructions per lane and flush.  Each
// lane holding FP64 totals of its own instead (14 FP64 conversions and adds per flush,
// the FP64 pipe being 1/64 of the FP32 rate) cost 9 % of the 2.7M-atom pair kernel;
// this form costs 3 % at 32 pairs per lane between flushes (2.5 % at 64).
#ifndef LMFF_ILP_FLUSH_PAIRS
#define LMFF_ILP_FLUSH_PAIRS 32
#endif
constexpr int ILP_FLUSH_PAIRS = LMFF_ILP_FLUSH_PAIRS;

// per-atom accumulators of the pair kernel: one lane's partial sums in R (mixed
// precision: over at most ILP_FLUSH_PAIRS pairs of the block since the last flush)
struct IlpAcc {
  R fx = 0, fy = 0, fz = 0, gxa = 0, gya = 0, gza = 0;
  R tpi = 0;   // two-pair loop: sum of the n_i coefficients, applied once (f -= tpi n_i)
  R evdw = 0, erep = 0, w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0, w5 = 0;
};

// Reduce-scatter over the TPA lanes of one atom (lane = thread index mod TPA, m = the
// group's shuffle mask): v[H] of every lane in; out, each lane holds in v[0 .. H/TPA)
// (at least v[0]) the sums over the lanes of the slots rs_slot0(lane) + k.  Halving
// levels first (a lane keeps the half selected by its lane bit and adds the partner's
// copy of it), then, with more lanes than slots, full levels (both partners form the
// same sum, a + b = b + a).  Fixed order: results are bitwise reproducible.
template <int O, int H>
struct LaneRS {
  static __device__ __forceinline__ void run(float *v, int lane, unsigned m) {
    if constexpr (O > 0) {
      if constexpr (H > 1) {
        constexpr int h = H / 2;
        const bool up = (lane & O) != 0;
#pragma unroll
        for (int k = 0; k < h; k++) {
          const float send = up ? v[k] : v[k + h];
          const float keep = up ? v[k + h] : v[k];
          v[k] = keep + __shfl_xor_sync(m, send, O);
        }
        LaneRS<O / 2, h>::run(v, lane, m);
      } else {
        v[0] += __shfl_xor_sync(m, v[0], O);
        LaneRS<O / 2, 1>::run(v, lane, m);
      }
    }
  }
};
template <int TPA, int NS>
__device__ __forceinline__ int rs_slot0(int lane) {
  int base = 0, h = NS;
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1)
    if (h > 1) {
      h >>= 1;
      if (lane & o) base += h;
    }
  return base;
}

// The FP64 totals of one atom, spread over its TPA lanes (mixed precision).  Slots:
// 0-2 force on i (the n_i terms of the two-pair loop folded in), 3-5 dE/dn_i,
// energy/virial kernels also 6 evdw, 7 erep, 8-13 virial, 14 evdw + erep (per-atom
// energy).  With TPA > slots several lanes hold the same total ("primary": the first).
// FP64 (R = double): the accumulators are the totals and nothing here runs.
constexpr bool ILP_TOT_SPLIT = sizeof(R) == 4;
template <int TPA, bool EV, bool EATOM>
struct LaneTot {
  static constexpr int NS = EV ? 16 : 8;
  static constexpr int HOLD = NS > TPA ? NS / TPA : 1;
  // The totals sit in shared memory ([HOLD][256] doubles per block, one column per
  // thread, 2 KB at 8 lanes per atom) and lane and shuffle mask are recomputed at each
  // flush, so that the pair loop holds no register for them (held in registers, they
  // made the two-pair loop spill at 64 registers: 4.3 % slower at 2.7M atoms).
  double *t;
  __device__ __forceinline__ void init(double *s) {
    t = s + threadIdx.x;
#pragma unroll
    for (int k = 0; k < HOLD; k++) t[k * 256] = 0.0;
  }
  __device__ __forceinline__ double get(int k) const { return t[k * 256]; }
  __device__ __forceinline__ void flush(IlpAcc &acc, R nix, R niy, R niz) {
    if constexpr (ILP_TOT_SPLIT) {
      const int lane = threadIdx.x & (TPA - 1);
      const unsigned gmask = TPA == 32 ? 0xffffffffu : ((1u << TPA) - 1u) << ((threadIdx.x & 31) & ~(TPA - 1));
      float v[NS];
      v[0] = fmaf(-acc.tpi, nix, acc.fx);
      v[1] = fmaf(-acc.tpi, niy, acc.fy);
      v[2] = fmaf(-acc.tpi, niz, acc.fz);
      v[3] = acc.gxa; v[4] = acc.gya; v[5] = acc.gza;
      if constexpr (EV) {
        v[6] = acc.evdw; v[7] = acc.erep;
        v[8] = acc.w0; v[9] = acc.w1; v[10] = acc.w2; v[11] = acc.w3; v[12] = acc.w4; v[13] = acc.w5;
        v[14] = EATOM ? acc.evdw + acc.erep : 0.f;
        v[15] = 0.f;
      } else {
        v[6] = 0.f; v[7] = 0.f;
      }
      LaneRS<TPA / 2, NS>::run(v, lane, gmask);
#pragma unroll
      for (int k = 0; k < HOLD; k++) t[k * 256] += (double)v[k];
      acc = IlpAcc{};
    }
  }
};

// normal of j as R
template <class T>
struct NrmJ;
template <>
struct NrmJ<float> {
  float4 q;
  __device__ __forceinline__ static NrmJ load(const ForceArgs<float> &a, int j) {
    return NrmJ{__ldg(&a.A.jrec[3 * (size_t)j + 2])};
  }
};
template <>
struct NrmJ<double> {
  d4 q;
  __device__ __forceinline__ static NrmJ load(const ForceArgs<double> &a, int j) { return NrmJ{a.nrm64[j]}; }
};

// Repulsion of one directed term from exp0 = exp(-lambda (r - z0)) and exp1 =
// exp(-rho^2/delta^2): energy V, the normal-projection factor fpair1 and the radial
// factor fsum (calc_FRep: pair_ilp_graphene_hbn.cpp:602-621 for ILP,
// pair_kolmogorov_crespi_full.cpp:615-631 for KC).
template <bool KC>
__device__ __forceinline__ void rep_term(const IlpP<R> &p, R exp0, R exp1, R rhosq, R rinv, R &V, R &fpair1, R &fsum) {
  if constexpr (KC) {
    R x = rhosq * p.delta2inv;
    R sumC1 = p.kc_C0 + p.kc_C2 * x + p.kc_C4 * x * x;
    R sumC11 = (p.kc_C2 + R(2) * p.kc_C4 * x) * p.delta2inv;
    R Erep = p.eps_half + exp1 * sumC1;
    V = exp0 * Erep;
    fpair1 = R(2) * exp0 * exp1 * (p.delta2inv * sumC1 - sumC11);
    fsum = p.lambda * exp0 * rinv * Erep + fpair1;
  } else {
    R frho = exp1 * p.C;
    R Erep = p.eps_half + frho;
    V = exp0 * Erep;
    fpair1 = R(2) * exp0 * frho * p.delta2inv;
    fsum = p.lambda * exp0 * rinv * Erep + fpair1;
  }
}

// One list entry (i, j, image) with j's position and normal already loaded.
// ---- FP64 pair-kernel arithmetic (the plain form): the FP64 pipe runs at 1/64 of the FP32
// rate, so the exponentials, the square root and the divisions of a pair are written
// with fewer FP64 instructions at full double accuracy (results within a few ulp of the
// library functions, far inside the 1e-10 parity bar).
//
// e^x by Tang's table-driven method (P. T. P. Tang, ACM TOMS 15, 1989): n = rint(256 x /
// ln2), r = x - n ln2/256 (|r| <= ln2/512; one FMA with ln2/256 rounded to double costs
// at most |n| 2^-62 absolute in r, hence in the relative error of e^x: |n| < 2^18, so
// below 6e-14 for |x| < 700 and below 4e-15 for |x| < 40), e^x = 2^(n>>8)
// 2^((n&255)/256) (1 + p(r)), p the degree-4 Taylor polynomial of e^r - 1 (truncation
// below 4e-17 relative: the 256-entry table keeps |r| small enough for degree 4, two FP64
// FMAs fewer than degree 6 over 64 entries).  Outside |x| < 700 the library exp.
constexpr int EXP2_F64_N = 256;
__device__ double g_exp2_f64[EXP2_F64_N];

__global__ void k_fill_exp2_f64() {
  const int j = threadIdx.x;
  if (j < EXP2_F64_N) g_exp2_f64[j] = exp2((double)j / EXP2_F64_N);
}

__device__ __forceinline__ double exp_t64(double x) {
  if (!(fabs(x) < 700.0)) return exp(x);
  const double magic = 6755399441055744.0;   // 1.5 * 2^52
  const double tn = __dadd_rn(x * 369.3299304675746, magic);   // 256 / ln2
  const int n = __double2loint(tn);
  const double nd = __dsub_rn(tn, magic);
  const double r = fma(-nd, 0.0027076061740622863, x);          // ln2 / 256
  double p = fma(r, 1.0 / 24.0, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = p * r;
  const double T = __ldg(&g_exp2_f64[n & (EXP2_F64_N - 1)]);
  const double v = fma(T, p, T);
  return __hiloint2double(__double2hiint(v) + (int)((unsigned)(n >> 8) << 20), __double2loint(v));
}

// 1/sqrt(x), 1/x: FP32 estimates (relative error ~2^-22) and one FP64 Newton step
// (~1e-13 relative, the error squared)
__device__ __forceinline__ double rsqrt_nr1(double x) {
  const double y = (double)rsqrt_ftz((float)x);
  return fma(0.5 * y, fma(-(x * y), y, 1.0), y);
}
__device__ __forceinline__ double rcp_nr1(double x) {
  const double y = (double)rcp_ftz((float)x);
  return fma(y, fma(-x, y, 1.0), y);
}

// Multi-element pair parameters, copied into shared memory by each block of k_ilp: lanes
// index them by their own element pair, which in constant memory would serialise (one
// constant-cache access per distinct address in a warp).
__shared__ IlpP<R> s_ilp[MAXELEM * MAXELEM];

// IMG: the entry may carry a periodic image shift (false: every entry of i's list is
// unshifted, and the image decode and shift are left out)
// GH (subdomain mode, iown: whether i is owned): term (i,j) counts when i is owned,
// term (j,i) when j is, the vdW pair when the end the tag-parity half keeps is.
template <bool EV, bool ONE, bool KC, bool IMG, bool GH>
__device__ __forceinline__ void ilp_pair(const ForceArgs<R> &a, const AtomI<R> &ai, const SysDesc &sdl, uint32_t e,
                                         const typename AtomI<R>::J &J, const NrmJ<R> &N, R nix, R niy, R niz,
                                         int ie, long long mi, long long itag, bool check, bool iown, IlpAcc &acc) {
  int j, sx = 0, sy = 0, sz = 0;
  if (IMG) decode_entry(e, a.lc, j, sx, sy, sz);
  else j = (int)(e & a.lc.imask);
  R dx, dy, dz;
  long long jinfo;
  ai.disp_from(J, sdl, sx, sy, sz, dx, dy, dz, jinfo);
  R rsq = dx * dx + dy * dy + dz * dz;
  if (!(rsq < c_pot.i_cutsq)) return;
  if (check && info_mol(jinfo) == mi) return;
  const int tj = info_type(jinfo);
  if (check && !((c_pot.ilp_typemask >> tj) & 1u)) return;
  const int je = ONE ? 0 : c_pot.i_map[tj];
  const IlpP<R> &pij = ONE ? c_pot.ilp[0] : s_ilp[ie * MAXELEM + je];
  const IlpP<R> &pji = ONE ? c_pot.ilp[0] : s_ilp[je * MAXELEM + ie];
  const R njx = N.q.x, njy = N.q.y, njz = N.q.z;
  R r, rinv;
  if constexpr (sizeof(R) == 8) { rinv = rsqrt_nr1(rsq); r = rsq * rinv; }
  else { rinv = rsqrt_ftz(rsq); r = rsq * rinv; }
  // taper (pair_ilp_graphene_hbn.h:80-115), Tap and dTap in one pass
  R Tap = 1, dTap = 0;
  if (c_pot.tap) {
    // Tap = 1 + x^4 (((20x - 70)x + 84)x - 35); dTap/dx = 140 x^3 (x - 1)^3
    const R x = r * c_pot.i_inv_rcut, x2 = x * x;
    Tap = R(20) * x + R(-70);
    Tap = Tap * x + R(84);
    Tap = Tap * x + R(-35);
    Tap = Tap * (x2 * x2) + R(1);
    const R y = x2 - x;
    dTap = (y * y) * (y * (R(140) * c_pot.i_inv_rcut));
  }
  // ---- vdW (both ends evaluate the pair force; energy halved)
  R wi = 1, wj = 1, wv = 1;
  bool keep;
  if constexpr (GH) {
    keep = keep_half_r(itag, a.tag[j], -dx, -dy, -dz);
    const bool jown = owned(a, j);
    wi = iown ? R(1) : R(0);
    wj = jown ? R(1) : R(0);
    wv = (keep ? iown : jown) ? R(1) : R(0);
  } else {
    keep = c_pot.vdw_sym || keep_half(itag, a.tag[j], sx, sy, sz);
  }
  const IlpP<R> &pv = (c_pot.vdw_sym || keep) ? pij : pji;
  R r2inv = rinv * rinv;
  R r6inv = r2inv * r2inv * r2inv;
  R r8inv = r6inv * r2inv;
  R Vvdw, fpv;
  if constexpr (KC) {
    // pair_kolmogorov_crespi_full.cpp:522-526: undamped -A z0^6 / r^6
    Vvdw = -pv.kc_Az06 * r6inv;
    fpv = R(-6) * pv.kc_Az06 * r8inv;
  } else {
    R TSvdw, TSinv;
    if constexpr (sizeof(R) == 8) {
      // exp(-d (r/seff - 1)) = exp(d - (d/seff) r); (TS - 1)/TS = 1 - 1/TS
      TSvdw = R(1) + exp_t64(fma(-pv.d_over_seff, r, pv.d));
      TSinv = rcp_nr1(TSvdw);
      const R c6t = pv.C6 * TSinv;
      Vvdw = -(c6t * r6inv);
      fpv = (c6t * r8inv) * fma(pv.d_over_seff * (R(1) - TSinv), r, R(-6));
    } else {
      TSvdw = R(1) + Math<R>::exp_ts(pv, r);
      TSinv = Math<R>::rcp(TSvdw);
      Vvdw = -pv.C6 * r6inv * TSinv;
      fpv = pv.C6 * r8inv * TSinv * (R(-6) + pv.d_over_seff * (TSvdw - R(1)) * TSinv * r);
    }
  }
  if constexpr (GH) {
    Vvdw *= wv;
    fpv *= wv;
  }
  R fsum_v = fpv * Tap - Vvdw * dTap * rinv;
  // ---- repulsion of term (i,j) with n_i and of term (j,i) with n_j (del' = -del, prod' = -q)
  R p = nix * dx + niy * dy + niz * dz;
  R rhosq = rsq - p * p;
  R q = njx * dx + njy * dy + njz * dz;
  R rhosq2 = rsq - q * q;
  R V, fpair1, fsum, V2, fpair1b, fsum2, crad;
  if constexpr (sizeof(R) == 8 && !KC) {
    // F = E0 C e^{-rho^2/delta^2}: V = E0 eps/2 + F, fpair1 = 2 F / delta^2, and both
    // terms' radial factors lambda V / r + fpair1 go into crad together
    const R exp0 = exp_t64(-pij.lambda * (r - pij.z0));
    const R exp0b = pji.same_as_swapped ? exp0 : exp_t64(-pji.lambda * (r - pji.z0));
    const R F1 = (exp0 * pij.C) * exp_t64(-(rhosq * pij.delta2inv));
    const R F2 = (exp0b * pji.C) * exp_t64(-(rhosq2 * pji.delta2inv));
    V = fma(exp0, pij.eps_half, F1);
    V2 = fma(exp0b, pji.eps_half, F2);
    fpair1 = R(2) * (F1 * pij.delta2inv);
    fpair1b = R(2) * (F2 * pji.delta2inv);
    if constexpr (GH) {
      V *= wi; fpair1 *= wi;
      V2 *= wj; fpair1b *= wj;
    }
    const R Tr = Tap * rinv, dTr = dTap * rinv;
    crad = fsum_v + Tap * (fpair1 + fpair1b) + fma(Tr, pij.lambda, -dTr) * V + fma(Tr, pji.lambda, -dTr) * V2;
    if (EV) fsum = pij.lambda * rinv * V + fpair1;
  } else {
    R exp0, exp1;
    if constexpr (sizeof(R) == 8) {
      exp0 = exp_t64(-pij.lambda * (r - pij.z0));
      exp1 = exp_t64(-(rhosq * pij.delta2inv));
    } else {
      exp0 = Math<R>::exp_rep0(pij, r);
      exp1 = Math<R>::exp_rep1(pij, rhosq);
    }
    rep_term<KC>(pij, exp0, exp1, rhosq, rinv, V, fpair1, fsum);
    R exp0b, exp1b;
    if constexpr (sizeof(R) == 8) {
      exp0b = pji.same_as_swapped ? exp0 : exp_t64(-pji.lambda * (r - pji.z0));
      exp1b = exp_t64(-(rhosq2 * pji.delta2inv));
    } else {
      exp0b = pji.same_as_swapped ? exp0 : Math<R>::exp_rep0(pji, r);
      exp1b = Math<R>::exp_rep1(pji, rhosq2);
    }
    rep_term<KC>(pji, exp0b, exp1b, rhosq2, rinv, V2, fpair1b, fsum2);
    if constexpr (GH) {
      V *= wi; fpair1 *= wi; fsum *= wi;
      V2 *= wj; fpair1b *= wj; fsum2 *= wj;
    }
    crad = fsum_v + (fsum + fsum2) * Tap - (V + V2) * dTap * rinv;
  }
  // ---- force on i
  R tp1 = Tap * p * fpair1;
  R tq1 = Tap * q * fpair1b;
  acc.fx += crad * dx - tp1 * nix - tq1 * njx;
  acc.fy += crad * dy - tp1 * niy - tq1 * njy;
  acc.fz += crad * dz - tp1 * niz - tq1 * njz;
  acc.gxa += tp1 * dx; acc.gya += tp1 * dy; acc.gza += tp1 * dz;
  if (EV) {
    acc.evdw += R(0.5) * Vvdw * Tap;
    // Kolmogorov-Crespi without the taper tallies V - offset per directed term
    const R eoff = (KC && !c_pot.tap) ? pij.kc_off * wi + pji.kc_off * wj : R(0);
    acc.erep += R(0.5) * ((V + V2) * Tap - eoff);
    // term (i,j): del (x) fkc_ij;  vdW: half of del (x) fsum_v del
    R cr1 = fsum * Tap - V * dTap * rinv + R(0.5) * fsum_v;
    R kx = cr1 * dx - tp1 * nix, ky = cr1 * dy - tp1 * niy, kz = cr1 * dz - tp1 * niz;
    acc.w0 += dx * kx; acc.w1 += dy * ky; acc.w2 += dz * kz;
    acc.w3 += dx * ky; acc.w4 += dx * kz; acc.w5 += dy * kz;
  }
}

#ifdef LMFF_PACKED_X2
// ---- packed FP32x2 form of the same pair body (sm_100+ FFMA2/FADD2/FMUL2)
// The kernel is issue-bound in FP32, and the pair body is full of independent twin
// operations: the repulsion of term (i,j) with n_i and of term (j,i) with n_j, the x and
// y components, and the two Horner chains of Tap and dTap.  Each twin pair is one packed
// instruction.  Same formulas as ilp_pair; the rounding differs from it only by the
// order of a few additions.
__device__ __forceinline__ float2 p2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// Operand pairs of the packed body in constant memory, so that an FP32x2 instruction
// reads them as one 64-bit constant operand instead of a register pair built per pair:
// the Horner coefficients of (Tap, dTap/dx) and, for the single-element path, the
// (i,j) and (j,i) repulsion constants of element 0.
struct PairX2Const {
  float2 tap0, tap1, tap2, tap3;
  float2 nd2_l2e, C, eps_half, d2x2, lambda;
  // the same constants of element 0 duplicated for the two-pair body: taper in r (Tap
  // and dTap/dr with the powers of 1/rcut folded into the coefficients), vdW, the
  // repulsion's distance exponent, log2 C (C e^y = 2^(y log2 e + log2 C)) and eps
  float2 ta0, ta1, ta2, ta3, td0, td1, td2, td3, one;
  float2 nts_a, ts_a_seff, C6, d_over_seff, m6, nlam_l2e, lamz0_l2e, log2C, eps;
};
__constant__ PairX2Const c_x2;

// Multi-element two-pair body: for atom element a and the elements b, c of the two
// neighbours of one iteration, the parameter pairs (X[a][b], X[a][c]) of every per-pair
// constant, one 64-bit shared-memory read each.  Valid when every element pair's
// parameters equal those of the swapped pair (then both repulsion terms and vdW use
// X[a][b]) and C >= 0 (h_two_multi, set by upload_pot).
constexpr int X2M_N = 11;   // nd2_l2e, log2C, eps, 2/delta^2, lambda, -lam log2e, lam z0 log2e,
                            // -ts_a, ts_a seff, C6, d/seff
constexpr int X2M_ROWS = MAXELEM * MAXELEM * MAXELEM;
__device__ float2 g_x2m[X2M_ROWS * X2M_N];
__shared__ float2 s_x2m[X2M_ROWS * X2M_N];


template <bool EV, bool ONE, bool KC, bool IMG, bool GH>
__device__ __forceinline__ void ilp_pair_x2(const ForceArgs<float> &a, const AtomI<float> &ai, const SysDesc &sdl,
                                            uint32_t e, const AtomI<float>::J &J, const NrmJ<float> &N, float nix,
                                            float niy, float niz, int ie, long long mi, long long itag, bool check,
                                            bool iown, IlpAcc &acc) {
  // del = x_i - x_j(image), x and y packed: ((h_i - h_j) - s Lhi) + ((l_i - l_j) - s Llo)
  int j, sx = 0, sy = 0, sz = 0;
  float2 hxy = add2(p2(ai.hx, ai.hy), p2(-J.h.x, -J.h.y));
  float2 lxy = add2(p2(ai.lx, ai.ly), p2(-J.l.x, -J.l.y));
  float dz;
  if constexpr (IMG) {
    decode_entry(e, a.lc, j, sx, sy, sz);
    const float2 sfx = p2((float)sx, (float)sy);
    hxy = add2(hxy, mul2(sfx, p2(-sdl.Lhi[0], -sdl.Lhi[1])));
    lxy = add2(lxy, mul2(sfx, p2(-sdl.Llo[0], -sdl.Llo[1])));
    dz = ((ai.hz - J.h.z) - (float)sz * sdl.Lhi[2]) + ((ai.lz - J.l.z) - (float)sz * sdl.Llo[2]);
  } else {
    j = (int)(e & a.lc.imask);
    dz = (ai.hz - J.h.z) + (ai.lz - J.l.z);
  }
  const float2 dxy = add2(hxy, lxy);
  const float2 sq = mul2(dxy, dxy);
  const float rsq = fmaf(dz, dz, sq.x + sq.y);
  if (!(rsq < c_pot.i_cutsq)) return;
  const long long jinfo = (long long)__float_as_int(J.h.w);
  if (check && info_mol(jinfo) == mi) return;
  const int tj = info_type(jinfo);
  if (check && !((c_pot.ilp_typemask >> tj) & 1u)) return;
  const int je = ONE ? 0 : c_pot.i_map[tj];
  const IlpP<float> &pij = ONE ? c_pot.ilp[0] : s_ilp[ie * MAXELEM + je];
  const IlpP<float> &pji = ONE ? c_pot.ilp[0] : s_ilp[je * MAXELEM + ie];
  const float dx = dxy.x, dy = dxy.y;
  const float njx = N.q.x, njy = N.q.y, njz = N.q.z;
  const float rinv = rsqrt_ftz(rsq);
  const float r = rsq * rinv;
  // Tap and dTap/dx as one packed Horner pass (pair_ilp_graphene_hbn.h:80-115)
  float Tap = 1.f, dTap = 0.f;
  if (c_pot.tap) {
    const float x = r * c_pot.i_inv_rcut;
    const float2 xx = p2(x, x);
    float2 t;
    if constexpr (ONE) {   // (measured: the multi-element body is faster with immediates)
      t = fma2(c_x2.tap0, xx, c_x2.tap1);
      t = fma2(t, xx, c_x2.tap2);
      t = fma2(t, xx, c_x2.tap3);
    } else {
      t = fma2(p2(20.f, 140.f), xx, p2(-70.f, -420.f));
      t = fma2(t, xx, p2(84.f, 420.f));
      t = fma2(t, xx, p2(-35.f, -140.f));
    }
    t = mul2(t, xx);
    t = mul2(t, xx);
    t = mul2(t, xx);
    Tap = fmaf(t.x, x, 1.f);
    dTap = t.y * c_pot.i_inv_rcut;
  }
  // ---- vdW (both ends evaluate the pair force; energy halved)
  float wi = 1.f, wj = 1.f, wv = 1.f;
  bool keep;
  if constexpr (GH) {
    keep = keep_half_r(itag, a.tag[j], -dx, -dy, -dz);
    const bool jown = owned(a, j);
    wi = iown ? 1.f : 0.f;
    wj = jown ? 1.f : 0.f;
    wv = (keep ? iown : jown) ? 1.f : 0.f;
  } else {
    keep = c_pot.vdw_sym || keep_half(itag, a.tag[j], sx, sy, sz);
  }
  const IlpP<float> &pv = (c_pot.vdw_sym || keep) ? pij : pji;
  const float r2inv = rinv * rinv;
  const float r6inv = r2inv * r2inv * r2inv;
  const float r8inv = r6inv * r2inv;
  float Vvdw, fpv;
  if constexpr (KC) {
    Vvdw = -pv.kc_Az06 * r6inv;
    fpv = -6.f * pv.kc_Az06 * r8inv;
  } else {
    const float TSvdw = 1.f + Math<float>::exp_ts(pv, r);
    const float TSinv = Math<float>::rcp(TSvdw);
    const float c6t = pv.C6 * TSinv;
    Vvdw = -c6t * r6inv;
    fpv = c6t * r8inv * (-6.f + pv.d_over_seff * (TSvdw - 1.f) * TSinv * r);
  }
  if constexpr (GH) {
    Vvdw *= wv;
    fpv *= wv;
  }
  const float fsum_v = fpv * Tap - Vvdw * dTap * rinv;
  // ---- the two repulsion terms packed: .x = (i,j) with n_i, .y = (j,i) with n_j.  The
  // projections n.del are scalar: packing them would first copy n_j and del into pairs.
  const float2 PQ = p2(fmaf(niz, dz, fmaf(niy, dy, nix * dx)), fmaf(njz, dz, fmaf(njy, dy, njx * dx)));
  // (the operand forms here and in the force sums below are the faster of packed and
  // scalar, measured per path)
  const float2 RH = ONE ? fma2(p2(-PQ.x, -PQ.y), PQ, p2(rsq, rsq))
                        : p2(fmaf(-PQ.x, PQ.x, rsq), fmaf(-PQ.y, PQ.y, rsq));
  const float e0 = Math<float>::exp_rep0(pij, r);
  const float e0b = pji.same_as_swapped ? e0 : Math<float>::exp_rep0(pji, r);
  const float2 E0 = p2(e0, e0b);
  const float2 EA = mul2(ONE ? c_x2.nd2_l2e : p2(pij.nd2_l2e, pji.nd2_l2e), RH);
  const float2 E1 = p2(ex2_ftz(EA.x), ex2_ftz(EA.y));
  const float2 D2 = p2(pij.delta2inv, pji.delta2inv);
  float2 V, FP1;
  float2 ER;
  if constexpr (KC) {
    const float2 X = mul2(RH, D2);
    const float2 S1 = fma2(fma2(p2(pij.kc_C4, pji.kc_C4), X, p2(pij.kc_C2, pji.kc_C2)), X, p2(pij.kc_C0, pji.kc_C0));
    const float2 S11 = mul2(fma2(p2(2.f * pij.kc_C4, 2.f * pji.kc_C4), X, p2(pij.kc_C2, pji.kc_C2)), D2);
    ER = fma2(E1, S1, p2(pij.eps_half, pji.eps_half));
    V = mul2(E0, ER);
    FP1 = mul2(mul2(p2(2.f, 2.f), mul2(E0, E1)), fma2(D2, S1, p2(-S11.x, -S11.y)));
  } else {
    const float2 FR = mul2(E1, ONE ? c_x2.C : p2(pij.C, pji.C));
    ER = add2(ONE ? c_x2.eps_half : p2(pij.eps_half, pji.eps_half), FR);
    V = mul2(E0, ER);
    FP1 = mul2(mul2(E0, FR), ONE ? c_x2.d2x2 : p2(2.f * pij.delta2inv, 2.f * pji.delta2inv));
  }
  if constexpr (GH) {
    V = mul2(V, p2(wi, wj));
    FP1 = mul2(FP1, p2(wi, wj));
  }
  const float2 FS = fma2(mul2(ONE ? c_x2.lambda : p2(pij.lambda, pji.lambda), V), p2(rinv, rinv), FP1);
  const float2 TPQ = mul2(mul2(p2(Tap, Tap), PQ), FP1);   // (tp1, tq1)
  const float Vsum = V.x + V.y;
  const float crad = fsum_v + (FS.x + FS.y) * Tap - Vsum * dTap * rinv;
  // ---- force on i; g_i += tp1 del
  if constexpr (ONE) {
    acc.fx += crad * dx - TPQ.x * nix - TPQ.y * njx;
    acc.fy += crad * dy - TPQ.x * niy - TPQ.y * njy;
    acc.fz += crad * dz - TPQ.x * niz - TPQ.y * njz;
    acc.gxa += TPQ.x * dx;
    acc.gya += TPQ.x * dy;
    acc.gza += TPQ.x * dz;
  } else {
    float2 fxy = fma2(p2(crad, crad), dxy, p2(acc.fx, acc.fy));
    fxy = fma2(p2(-TPQ.x, -TPQ.x), p2(nix, niy), fxy);
    fxy = fma2(p2(-TPQ.y, -TPQ.y), p2(njx, njy), fxy);
    acc.fx = fxy.x;
    acc.fy = fxy.y;
    acc.fz += crad * dz - TPQ.x * niz - TPQ.y * njz;
    const float2 gxy = fma2(p2(TPQ.x, TPQ.x), dxy, p2(acc.gxa, acc.gya));
    acc.gxa = gxy.x;
    acc.gya = gxy.y;
    acc.gza += TPQ.x * dz;
  }
  if (EV) {
    acc.evdw += 0.5f * Vvdw * Tap;
    const float eoff = (KC && !c_pot.tap) ? pij.kc_off * wi + pji.kc_off * wj : 0.f;
    acc.erep += 0.5f * (Vsum * Tap - eoff);
    const float cr1 = FS.x * Tap - V.x * dTap * rinv + 0.5f * fsum_v;
    const float kx = cr1 * dx - TPQ.x * nix, ky = cr1 * dy - TPQ.x * niy, kz = cr1 * dz - TPQ.x * niz;
    acc.w0 += dx * kx; acc.w1 += dy * ky; acc.w2 += dz * kz;
    acc.w3 += dx * ky; acc.w4 += dx * kz; acc.w5 += dy * kz;
  }
}

// ---- two list entries at once (single-element path, no energy/virial): FP32x2 lanes
// hold pair A and pair B, so that every quantity of the chain r -> Tap -> vdW ->
// repulsion is naturally a register pair and no operand has to be duplicated.  Same
// formulas as ilp_pair_x2; a pair outside the cutoff (or filtered by molecule or type)
// whose partner is inside is evaluated with Tap = dTap = 0, which zeroes every
// contribution.
// j's compact record: r0 = (hi x, y, z, lo x|y as FP16), r1 = (normal, lo z as FP16).
// The lo parts carry |lo| <= ulp(hi)/2 to ~3e-8 A; i's own lo parts are rounded the same
// way (loi), so that both ends of a pair see the same positions.
template <bool IMG>
__device__ __forceinline__ void disp_x2(const ForceArgs<float> &a, const AtomI<float> &ai, const float3 &loi,
                                        const SysDesc &sdl, uint32_t e, const float4 &r0, const float4 &r1,
                                        float2 &dxy, float &dz) {
  const float2 lj = __half22float2(bits_h2(__float_as_uint(r0.w)));
  const float ljz = __low2float(bits_h2(__float_as_uint(r1.w)));
  float2 hxy = add2(p2(ai.hx, ai.hy), p2(-r0.x, -r0.y));
  float2 lxy = add2(p2(loi.x, loi.y), p2(-lj.x, -lj.y));
  if constexpr (IMG) {
    int j, sx, sy, sz;
    decode_entry(e, a.lc, j, sx, sy, sz);
    const float2 sfx = p2((float)sx, (float)sy);
    hxy = add2(hxy, mul2(sfx, p2(-sdl.Lhi[0], -sdl.Lhi[1])));
    lxy = add2(lxy, mul2(sfx, p2(-sdl.Llo[0], -sdl.Llo[1])));
    dz = ((ai.hz - r0.z) - (float)sz * sdl.Lhi[2]) + ((loi.z - ljz) - (float)sz * sdl.Llo[2]);
  } else {
    dz = (ai.hz - r0.z) + (loi.z - ljz);
  }
  dxy = add2(hxy, lxy);
}

// a per-pair constant pair: element 0's from constant memory (ONE, by value, so that the
// load keeps its constant address space) or the shared-memory row's
template <bool ONE>
__device__ __forceinline__ float2 x2sel(float2 c, const float2 *prow, int k) {
  if constexpr (ONE) return c;
  else return prow[k];
}

// bvalid = false: only pair A exists (B repeats A and contributes nothing).  ONE: the
// constants of element 0 from constant memory; otherwise the (ie, jeA, jeB) row of s_x2m
// (the neighbours' elements travel in the upper half of their record's r1.w).
template <bool ONE, bool IMG>
__device__ __forceinline__ void ilp_pair2(const ForceArgs<float> &a, const AtomI<float> &ai, const float3 &loi,
                                          const SysDesc &sdl, uint32_t eA, const float4 &A0, const float4 &A1,
                                          uint32_t eB, const float4 &B0, const float4 &B1, bool bvalid, float nix,
                                          float niy, float niz, int ie, IlpAcc &acc) {
  const float2 *prow = nullptr;
  if constexpr (!ONE)
    prow = s_x2m + ((ie * MAXELEM + (int)(__float_as_uint(A1.w) >> 16)) * MAXELEM + (int)(__float_as_uint(B1.w) >> 16)) *
                       X2M_N;
#define X2(field, k) x2sel<ONE>(c_x2.field, prow, k)
  float2 dA, dB;
  float dzA, dzB;
  disp_x2<IMG>(a, ai, loi, sdl, eA, A0, A1, dA, dzA);
  disp_x2<IMG>(a, ai, loi, sdl, eB, B0, B1, dB, dzB);
  const float2 sqA = mul2(dA, dA), sqB = mul2(dB, dB);
  const float2 RSQ = p2(fmaf(dzA, dzA, sqA.x + sqA.y), fmaf(dzB, dzB, sqB.x + sqB.y));
  const bool inA = RSQ.x < c_pot.i_cutsq, inB = bvalid && RSQ.y < c_pot.i_cutsq;
  if (!(inA || inB)) return;
  const float2 RINV = p2(rsqrt_ftz(RSQ.x), rsqrt_ftz(RSQ.y));
  const float2 R = mul2(RSQ, RINV);
  // Tap = 1 + x^4 (((20x - 70)x + 84)x - 35), dTap/dr = x^3 (((140x - 420)x + 420)x - 140) / rcut,
  // x = r / rcut, evaluated in r
  float2 TAP = c_x2.one, DTAP = p2(0.f, 0.f);
  if (c_pot.tap) {
    const float2 R2 = mul2(R, R);
    float2 t = fma2(c_x2.ta0, R, c_x2.ta1);
    t = fma2(t, R, c_x2.ta2);
    t = fma2(t, R, c_x2.ta3);
    TAP = fma2(t, mul2(R2, R2), c_x2.one);
    float2 u = fma2(c_x2.td0, R, c_x2.td1);
    u = fma2(u, R, c_x2.td2);
    u = fma2(u, R, c_x2.td3);
    DTAP = mul2(u, mul2(R2, R));
  }
  if (!inA) { TAP.x = 0.f; DTAP.x = 0.f; }
  if (!inB) { TAP.y = 0.f; DTAP.y = 0.f; }
  const float2 DR = mul2(DTAP, RINV);
  // ---- vdW: V = -C6 r^-6 / TS, TS = 1 + e^{-d (r/seff - 1)}
  const float2 R2I = mul2(RINV, RINV);
  const float2 R6I = mul2(mul2(R2I, R2I), R2I);
  const float2 EXA = fma2(R, X2(nts_a, 7), X2(ts_a_seff, 8));
  const float2 EX = p2(ex2_ftz(EXA.x), ex2_ftz(EXA.y));
  const float2 TSV = add2(EX, c_x2.one);
  const float2 TSI = p2(rcp_ftz(TSV.x), rcp_ftz(TSV.y));
  const float2 C6T = mul2(X2(C6, 9), TSI);
  const float2 C6R6 = mul2(C6T, R6I);                       // -V
  const float2 G = fma2(mul2(mul2(EX, TSI), R), X2(d_over_seff, 10), c_x2.m6);
  const float2 FPV = mul2(mul2(C6R6, R2I), G);
  const float2 FSUMV = fma2(FPV, TAP, mul2(C6R6, DR));      // fpv Tap - V dTap / r
  // ---- repulsion, terms (i,j) with n_i and (j,i) with n_j
  const float2 PQI = p2(fmaf(niz, dzA, fmaf(niy, dA.y, nix * dA.x)), fmaf(niz, dzB, fmaf(niy, dB.y, nix * dB.x)));
  const float2 PQJ = p2(fmaf(A1.z, dzA, fmaf(A1.y, dA.y, A1.x * dA.x)), fmaf(B1.z, dzB, fmaf(B1.y, dB.y, B1.x * dB.x)));
  const float2 RHI = fma2(p2(-PQI.x, -PQI.y), PQI, RSQ);
  const float2 RHJ = fma2(p2(-PQJ.x, -PQJ.y), PQJ, RSQ);
  // V_t = E0 (eps/2 + C e^{-rho_t^2/delta^2}), fpair1_t = 2 E0 C e^{...} / delta^2, and the
  // radial factor of both terms together, lambda (V_i + V_j) / r + fpair1_i + fpair1_j
  const float2 E0A = fma2(R, X2(nlam_l2e, 5), X2(lamz0_l2e, 6));
  const float2 E0 = p2(ex2_ftz(E0A.x), ex2_ftz(E0A.y));
  const float2 EIA = fma2(X2(nd2_l2e, 0), RHI, X2(log2C, 1)), EJA = fma2(X2(nd2_l2e, 0), RHJ, X2(log2C, 1));
  const float2 E0FI = mul2(E0, p2(ex2_ftz(EIA.x), ex2_ftz(EIA.y)));
  const float2 E0FJ = mul2(E0, p2(ex2_ftz(EJA.x), ex2_ftz(EJA.y)));
  const float2 S = add2(E0FI, E0FJ);
  const float2 VS = fma2(E0, X2(eps, 2), S);
  const float2 FSS = fma2(mul2(X2(lambda, 4), RINV), VS, mul2(S, X2(d2x2, 3)));
  const float2 TPQI = mul2(mul2(TAP, PQI), mul2(E0FI, X2(d2x2, 3)));
  const float2 TPQJ = mul2(mul2(TAP, PQJ), mul2(E0FJ, X2(d2x2, 3)));
  const float2 CRAD = fma2(p2(-VS.x, -VS.y), DR, fma2(FSS, TAP, FSUMV));
  // ---- force on i and g_i
  // the n_i terms -tp1 n_i of all pairs are applied once, after the loop (acc.tpi)
  acc.tpi += TPQI.x + TPQI.y;
  acc.fx += CRAD.x * dA.x - TPQJ.x * A1.x;
  acc.fy += CRAD.x * dA.y - TPQJ.x * A1.y;
  acc.fz += CRAD.x * dzA - TPQJ.x * A1.z;
  acc.gxa += TPQI.x * dA.x;
  acc.gya += TPQI.x * dA.y;
  acc.gza += TPQI.x * dzA;
  acc.fx += CRAD.y * dB.x - TPQJ.y * B1.x;
  acc.fy += CRAD.y * dB.y - TPQJ.y * B1.y;
  acc.fz += CRAD.y * dzB - TPQJ.y * B1.z;
  acc.gxa += TPQI.y * dB.x;
  acc.gya += TPQI.y * dB.y;
  acc.gza += TPQI.y * dzB;
#undef X2
}
#endif  // LMFF_PACKED_X2

// the pair body of this precision: packed FP32x2 for the mixed path, scalar FP64
template <bool EV, bool ONE, bool KC, bool IMG, bool GH>
__device__ __forceinline__ void pair_body(const ForceArgs<R> &a, const AtomI<R> &ai, const SysDesc &sdl, uint32_t e,
                                          const typename AtomI<R>::J &J, const NrmJ<R> &N, R nix, R niy, R niz, int ie,
                                          long long mi, long long itag, bool check, bool iown, IlpAcc &acc) {
#ifdef LMFF_PACKED_X2
  ilp_pair_x2<EV, ONE, KC, IMG, GH>(a, ai, sdl, e, J, N, nix, niy, niz, ie, mi, itag, check, iown, acc);
#else
  ilp_pair<EV, ONE, KC, IMG, GH>(a, ai, sdl, e, J, N, nix, niy, niz, ie, mi, itag, check, iown, acc);
#endif
}

// FP32: the generic force-only loops at least 5 blocks of 256 threads per SM (48
// registers) -- issue-bound with long-scoreboard stalls on j's data, and 40 resident
// warps hide them better than 36 (measured: -8 % at 2.7M atoms, -16 % at 490k).  The
// two-pair body of the single-element path needs 76 registers without spills; 4 blocks
// (64 registers) measured 3 % faster than 3 blocks at 2.7M atoms.  The energy/virial
// loops with their FP64 flushes: 4 blocks (64 registers), 26 % faster than 5 on the
// 256-replica batch, 12 % on the 331k slab.  FP64 keeps its registers.
template <int TPA, bool EV, bool EATOM, bool ONE, bool GH, bool KC, bool TWO>
constexpr int ilp_min_blocks() {
  return sizeof(R) == 8 ? 1 : (TWO || EV) ? 4 : 5;
}

// TWO: the two-pair loop alone (mixed precision, forces only, interlayer list, C >= 0
// and symmetric element-pair constants: the host checks these), in a kernel of its own
// so that the generic loops do not share its register allocation
// GH: subdomain mode (owned + ghost atoms, see ForceArgs::own_perm)
template <int TPA, bool EV, bool EATOM, bool ONE, bool GH, bool KC, bool TWO>
__global__ void __launch_bounds__(256, (ilp_min_blocks<TPA, EV, EATOM, ONE, GH, KC, TWO>())) k_ilp(ForceArgs<R> a) {
  pdl_enter(a.pdl);
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gtid / TPA;
  const int lane = threadIdx.x & (TPA - 1);
  const bool valid = i < a.n;
  const int ii = valid ? i : a.n - 1;
  const SysDesc &sd = a.A.sys[a.A.sysid[ii]];
  AtomI<R> ai;
  ai.load(a.A, ii);
  const int ti = info_type(ai.info);
  const long long mi = info_mol(ai.info);
  const int ie = c_pot.i_map[ti];
  R nix, niy, niz;
  if constexpr (sizeof(R) == 8) { d4 q = a.nrm64[ii]; nix = q.x; niy = q.y; niz = q.z; }
  else { float4 q = a.nrm32[ii]; nix = q.x; niy = q.y; niz = q.z; }
  const long long itag = (c_pot.vdw_sym && !GH) ? 0 : a.tag[ii];
  const bool iown = !GH || owned(a, ii);
  IlpAcc acc;
  __shared__ double s_tot[ILP_TOT_SPLIT ? LaneTot<TPA, EV, EATOM>::HOLD : 1][256];
  LaneTot<TPA, EV, EATOM> tot;
  if constexpr (ILP_TOT_SPLIT) tot.init(&s_tot[0][0]);
  // a flush after the iteration of lane entry k: every ILP_FLUSH_PAIRS pairs of a lane,
  // when all TPA lanes run that iteration (then the condition is the same for all of
  // them); what is left at the end goes with the final flush
#define ILP_FLUSH_AT(k, step, last)                                                         \
  if constexpr (ILP_TOT_SPLIT)                                                               \
    if ((((k) + (step)) & (TPA * ILP_FLUSH_PAIRS - 1)) < TPA && ((k) | (TPA - 1)) + (last) < cnt) \
      tot.flush(acc, nix, niy, niz);
  SysDesc sdl;  // box of i's system in registers for the image shifts
#pragma unroll
  for (int d = 0; d < 3; d++) {
    sdl.L[d] = sd.L[d];
    sdl.Lhi[d] = sd.Lhi[d];
    sdl.Llo[d] = sd.Llo[d];
  }
  // a list without list_full holds only interlayer pairs of ILP-mapped types (k_list)
  const bool check = a.list_full != 0;
  if constexpr (!ONE) {
#ifdef LMFF_PACKED_X2
    if constexpr (TWO) {
      for (int w = threadIdx.x; w < X2M_ROWS * X2M_N; w += blockDim.x) s_x2m[w] = g_x2m[w];
    } else
#endif
    {
      const int words = (int)(sizeof(c_pot.ilp) / sizeof(int));
      const int *src = reinterpret_cast<const int *>(c_pot.ilp);
      int *dst = reinterpret_cast<int *>(s_ilp);
      for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
  }
  if (valid && ie >= 0) {
    const int64_t b = a.list_off[i];
    const uint32_t *lst = a.list + b;
    const int cnt = (int)(a.list_off[i + 1] - b);
    // atoms whose list holds no periodic-image entry (most of a large box) run the loop
    // without the image decode and shift
    auto run = [&](auto img_t) {
      constexpr bool IMG = decltype(img_t)::value;
#ifdef LMFF_PACKED_X2
      if constexpr (TWO) {
        {
          // two entries (k, k + TPA) per iteration, loaded one iteration ahead, j's data
          // from the compact 32-byte records
          const float3 loi = make_float3(__half2float(__float2half_rn(ai.lx)), __half2float(__float2half_rn(ai.ly)),
                                         __half2float(__float2half_rn(ai.lz)));
          int k = lane;
          uint32_t eA = k < cnt ? __ldg(&lst[k]) : 0u;
          uint32_t eB = k + TPA < cnt ? __ldg(&lst[k + TPA]) : 0u;
          for (; k + TPA < cnt; k += 2 * TPA) {
              const uint32_t ea = eA, eb = eB;
              if (k + 2 * TPA < cnt) eA = __ldg(&lst[k + 2 * TPA]);
              if (k + 3 * TPA < cnt) eB = __ldg(&lst[k + 3 * TPA]);
              const size_t ja = 2 * (size_t)(ea & a.lc.imask), jb = 2 * (size_t)(eb & a.lc.imask);
              ilp_pair2<ONE, IMG>(a, ai, loi, sdl, ea, __ldg(&a.A.jrec2[ja]), __ldg(&a.A.jrec2[ja + 1]), eb,
                                  __ldg(&a.A.jrec2[jb]), __ldg(&a.A.jrec2[jb + 1]), true, nix, niy, niz, ie, acc);
              ILP_FLUSH_AT(k, 2 * TPA, TPA)
          }
          if (k < cnt) {
            const size_t ja = 2 * (size_t)(eA & a.lc.imask);
            const float4 r0 = __ldg(&a.A.jrec2[ja]), r1 = __ldg(&a.A.jrec2[ja + 1]);
            ilp_pair2<ONE, IMG>(a, ai, loi, sdl, eA, r0, r1, eA, r0, r1, false, nix, niy, niz, ie, acc);
          }
          return;
        }
      } else
#endif
      if constexpr (ONE) {
        // the next list entry is loaded one iteration ahead, so that only j's data (not
        // the list read before it) is on the dependence chain of a pair (-9 % on the
        // 2.7M-atom graphite; the multi-element body has no registers to spare for it)
        uint32_t e_next = lane < cnt ? __ldg(&lst[lane]) : 0u;
        for (int k = lane; k < cnt; k += TPA) {
          const uint32_t e = e_next;
          if (k + TPA < cnt) e_next = __ldg(&lst[k + TPA]);
          const int j = (int)(e & a.lc.imask);
          pair_body<EV, ONE, KC, IMG, GH>(a, ai, sdl, e, ai.fetch(a.A, j), NrmJ<R>::load(a, j), nix, niy, niz, ie,
                                          mi, itag, check, iown, acc);
          ILP_FLUSH_AT(k, TPA, 0)
        }
      } else {
        for (int k = lane; k < cnt; k += TPA) {
          const uint32_t e = __ldg(&lst[k]);
          const int j = (int)(e & a.lc.imask);
          pair_body<EV, ONE, KC, IMG, GH>(a, ai, sdl, e, ai.fetch(a.A, j), NrmJ<R>::load(a, j), nix, niy, niz, ie,
                                          mi, itag, check, iown, acc);
          ILP_FLUSH_AT(k, TPA, 0)
        }
      }
    };
    if (a.list_img[i]) run(std::true_type{});
    else run(std::false_type{});
  }
#undef ILP_FLUSH_AT
  if constexpr (ILP_TOT_SPLIT) {
    // final flush (all lanes of atom i reach it), then each primary lane stores the
    // FP64 totals it holds
    tot.flush(acc, nix, niy, niz);
    constexpr int NS = LaneTot<TPA, EV, EATOM>::NS, HOLD = LaneTot<TPA, EV, EATOM>::HOLD;
    if (!valid || (TPA > NS && (lane & (TPA / NS - 1)) != 0)) return;
    const int s0 = rs_slot0<TPA, NS>(lane);
#pragma unroll
    for (int k = 0; k < HOLD; k++) {
      const int sl = s0 + k;
      const double t = tot.get(k);
      if (sl < 3) a.ilp_f[(size_t)sl * a.n + i] = t;
      else if (sl < 6) {
        double *g = reinterpret_cast<double *>(&a.ilp_g[i]);
        g[sl - 3] = t;
        if (sl == 3) g[3] = 0.0;
      } else if (EV && sl < 14) a.stat_ilp[(size_t)(sl - 6) * a.n + i] = t;
      else if (EV && EATOM && sl == 14) a.eatom_ilp[i] = t;
    }
  } else {
    double fx = acc.fx - acc.tpi * nix, fy = acc.fy - acc.tpi * niy, fz = acc.fz - acc.tpi * niz;
    double gxa = acc.gxa, gya = acc.gya, gza = acc.gza;
    double evdw = acc.evdw, erep = acc.erep, w0 = acc.w0, w1 = acc.w1, w2 = acc.w2, w3 = acc.w3, w4 = acc.w4,
           w5 = acc.w5;
    // ---- reduce over the TPA lanes of atom i
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
      fx += __shfl_xor_sync(0xffffffff, fx, o);
      fy += __shfl_xor_sync(0xffffffff, fy, o);
      fz += __shfl_xor_sync(0xffffffff, fz, o);
      gxa += __shfl_xor_sync(0xffffffff, gxa, o);
      gya += __shfl_xor_sync(0xffffffff, gya, o);
      gza += __shfl_xor_sync(0xffffffff, gza, o);
      if (EV) {
        evdw += __shfl_xor_sync(0xffffffff, evdw, o);
        erep += __shfl_xor_sync(0xffffffff, erep, o);
        w0 += __shfl_xor_sync(0xffffffff, w0, o);
        w1 += __shfl_xor_sync(0xffffffff, w1, o);
        w2 += __shfl_xor_sync(0xffffffff, w2, o);
        w3 += __shfl_xor_sync(0xffffffff, w3, o);
        w4 += __shfl_xor_sync(0xffffffff, w4, o);
        w5 += __shfl_xor_sync(0xffffffff, w5, o);
      }
    }
    if (!valid || lane != 0) return;
    a.ilp_f[i] = fx;
    a.ilp_f[a.n + i] = fy;
    a.ilp_f[2 * a.n + i] = fz;
    a.ilp_g[i] = make_d4(gxa, gya, gza, 0.0);
    if (EV) {
      double *st = a.stat_ilp;
      st[i] = evdw;
      st[(size_t)a.n + i] = erep;
      st[(size_t)2 * a.n + i] = w0; st[(size_t)3 * a.n + i] = w1; st[(size_t)4 * a.n + i] = w2;
      st[(size_t)5 * a.n + i] = w3; st[(size_t)6 * a.n + i] = w4; st[(size_t)7 * a.n + i] = w5;
      if (EATOM) a.eatom_ilp[i] = evdw + erep;
    }
  }
}

// ============================================================== k_nderiv =========
// Normal-derivative assembly in FP64, one thread per atom i (calc_normal's dnormdri and
// dnormal, pair_ilp_graphene_hbn.cpp:893-926 / :1043-1067, applied to the reverse-
// accumulated g_i of the pair kernel).  With h = (I - n n^T) g / |n1| the force on
// intralayer neighbour m is -(dn1/dv_m)^T h and on i -(dn1/dx_i)^T h; dn1/dv of a cross
// product is a skew matrix, so each term is one cross product with h.  The neighbour
// forces go to ilp_c slots, gathered by k_finish.
// nderiv_eval: the assembly of atom i without writes -- the neighbour forces c[m] (zero
// past the atom's intralayer count), the force F on i and, with EV, the virial W.
struct NDeriv {
  double c[3][3];
  double F[3];
  double W[6];
};
// The normal frame of atom i: the part of the assembly that does not depend on g_i -- the
// bond vectors to its intralayer neighbours, the unit normal and 1/|n1|.  With a frame
// array (ForceArgs::nframe) k_nframe computes it beside the pair kernel, on the Tersoff
// stream, and k_nderiv only applies g_i to it: about half of the assembly's FP64 work
// leaves the step's critical path.  The arithmetic is that of the assembly done in one
// piece, so the results are the same to the bit.
struct NFrame {
  int cont;   // intralayer neighbours (0 when i is not ILP-mapped)
  bool ok;    // cont >= 2 and |n1| > 0
  double v[MAXILP][3];
  double nx, ny, nz, inn;
};
__device__ __forceinline__ void nframe_eval(const ForceArgs<R> &a, int i, NFrame &fr) {
  const SysDesc &sd = a.A.sys[a.A.sysid[i]];
  const int ie = c_pot.i_map[info_type(__double_as_longlong(a.A.xq[i].w))];
  fr.cont = ie >= 0 ? a.ilp_cnt[i] : 0;
  fr.ok = false;
  fr.nx = fr.ny = fr.nz = fr.inn = 0.0;
#pragma unroll
  for (int m = 0; m < MAXILP; m++) fr.v[m][0] = fr.v[m][1] = fr.v[m][2] = 0.0;
  const int cont = fr.cont;
  if (cont >= 2) {
#pragma unroll
    for (int m = 0; m < MAXILP; m++) {
      if (m >= cont) break;
      int j, sx, sy, sz;
      decode_entry(a.ilp_nb[(size_t)i * MAXILP + m], a.lc, j, sx, sy, sz);
      double ddx, ddy, ddz;
      disp64(a.A.xq, sd, i, j, sx, sy, sz, ddx, ddy, ddz);
      fr.v[m][0] = -ddx; fr.v[m][1] = -ddy; fr.v[m][2] = -ddz;
    }
    // three neighbours: v1 x v2 + v3 x v1 + v2 x v3 = (v2 - v1) x (v3 - v1), one product
    // instead of three.  The reference averages the three products (n1 / 3); the
    // unnormalised sum gives the same n, and h / 3 absorbs the 1/3 of each product's
    // derivative.
    const double ax = cont == 3 ? fr.v[1][0] - fr.v[0][0] : fr.v[0][0];
    const double ay = cont == 3 ? fr.v[1][1] - fr.v[0][1] : fr.v[0][1];
    const double az = cont == 3 ? fr.v[1][2] - fr.v[0][2] : fr.v[0][2];
    const double bx = cont == 3 ? fr.v[2][0] - fr.v[0][0] : fr.v[1][0];
    const double by = cont == 3 ? fr.v[2][1] - fr.v[0][1] : fr.v[1][1];
    const double bz = cont == 3 ? fr.v[2][2] - fr.v[0][2] : fr.v[1][2];
    const double n1x = ay * bz - by * az;
    const double n1y = az * bx - bz * ax;
    const double n1z = ax * by - bx * ay;
    const double nn2 = n1x * n1x + n1y * n1y + n1z * n1z;
    if (nn2 > 0.0) {
      double inn;
      if constexpr (sizeof(R) == 4) inn = nn2 > 1e-30 ? rsqrt_nr(nn2) : 1.0 / sqrt(nn2);
      else inn = 1.0 / sqrt(nn2);
      fr.ok = true;
      fr.inn = inn;
      fr.nx = n1x * inn; fr.ny = n1y * inn; fr.nz = n1z * inn;
    }
  }
}

// g_i applied to the frame: the forces on the intralayer neighbours and on i, and with EV
// their virial
template <bool EV>
__device__ __forceinline__ void nderiv_apply(const NFrame &fr, const d4 &g, NDeriv &o) {
  const double Gx = g.x, Gy = g.y, Gz = g.z;
  double Fx = 0, Fy = 0, Fz = 0;
  double W0 = 0, W1 = 0, W2 = 0, W3 = 0, W4 = 0, W5 = 0;
  double c0x = 0, c0y = 0, c0z = 0, c1x = 0, c1y = 0, c1z = 0, c2x = 0, c2y = 0, c2z = 0;
  const int cont = fr.cont;
  if (fr.ok) {
    const double(&v)[MAXILP][3] = fr.v;
    const double ax = cont == 3 ? v[1][0] - v[0][0] : v[0][0];
    const double ay = cont == 3 ? v[1][1] - v[0][1] : v[0][1];
    const double az = cont == 3 ? v[1][2] - v[0][2] : v[0][2];
    const double bx = cont == 3 ? v[2][0] - v[0][0] : v[1][0];
    const double by = cont == 3 ? v[2][1] - v[0][1] : v[1][1];
    const double bz = cont == 3 ? v[2][2] - v[0][2] : v[1][2];
    const double inn = fr.inn;
    const double nx = fr.nx, ny = fr.ny, nz = fr.nz;
    double ng = nx * Gx + ny * Gy + nz * Gz;
    double hx = (Gx - nx * ng) * inn, hy = (Gy - ny * ng) * inn, hz = (Gz - nz * ng) * inn;
    auto crs = [](double ax, double ay, double az, double bx, double by, double bz, double &ox, double &oy, double &oz) {
      ox = ay * bz - az * by; oy = az * bx - ax * bz; oz = ax * by - ay * bx;
    };
    if (cont == 2) {
      // -(dn1/dv1)^T h = -(v2 x h); -(dn1/dv2)^T h = v1 x h; on i: (v2 - v1) x h
      crs(v[1][0], v[1][1], v[1][2], hx, hy, hz, c0x, c0y, c0z);
      c0x = -c0x; c0y = -c0y; c0z = -c0z;
      crs(v[0][0], v[0][1], v[0][2], hx, hy, hz, c1x, c1y, c1z);
      Fx = -(c0x + c1x); Fy = -(c0y + c1y); Fz = -(c0z + c1z);
    } else {
      // -(dn1/dv_m)^T h for m = 1, 2, 3: (v3 - v2) x h, (v1 - v3) x h, (v2 - v1) x h; the
      // three sum to zero (no force on i), so the first is minus the other two
      crs(-bx, -by, -bz, hx, hy, hz, c1x, c1y, c1z);
      crs(ax, ay, az, hx, hy, hz, c2x, c2y, c2z);
      c0x = -(c1x + c2x); c0y = -(c1y + c2y); c0z = -(c1z + c2z);
    }
    if (EV) {
      // virial of the neighbour forces relative to i (the term's forces sum to zero)
      W0 = v[0][0] * c0x + v[1][0] * c1x; W1 = v[0][1] * c0y + v[1][1] * c1y; W2 = v[0][2] * c0z + v[1][2] * c1z;
      W3 = v[0][0] * c0y + v[1][0] * c1y; W4 = v[0][0] * c0z + v[1][0] * c1z; W5 = v[0][1] * c0z + v[1][1] * c1z;
      if (cont == 3) {
        W0 += v[2][0] * c2x; W1 += v[2][1] * c2y; W2 += v[2][2] * c2z;
        W3 += v[2][0] * c2y; W4 += v[2][0] * c2z; W5 += v[2][1] * c2z;
      }
    }
  }
  o.c[0][0] = c0x; o.c[0][1] = c0y; o.c[0][2] = c0z;
  o.c[1][0] = c1x; o.c[1][1] = c1y; o.c[1][2] = c1z;
  o.c[2][0] = c2x; o.c[2][1] = c2y; o.c[2][2] = c2z;
  o.F[0] = Fx; o.F[1] = Fy; o.F[2] = Fz;
  if (EV) {
    o.W[0] = W0; o.W[1] = W1; o.W[2] = W2; o.W[3] = W3; o.W[4] = W4; o.W[5] = W5;
  }
}

// the assembly of atom i from its stored frame, or in one piece without a frame array
template <bool EV>
__device__ __forceinline__ void nderiv_eval(const ForceArgs<R> &a, int i, NDeriv &o) {
  NFrame fr;
  if (a.nframe) {
    const d4 f0 = a.nframe[4 * (size_t)i], f1 = a.nframe[4 * (size_t)i + 1], f2 = a.nframe[4 * (size_t)i + 2],
             f3 = a.nframe[4 * (size_t)i + 3];
    fr.nx = f0.x; fr.ny = f0.y; fr.nz = f0.z; fr.inn = f0.w;
    fr.v[0][0] = f1.x; fr.v[0][1] = f1.y; fr.v[0][2] = f1.z; fr.cont = (int)f1.w;
    fr.v[1][0] = f2.x; fr.v[1][1] = f2.y; fr.v[1][2] = f2.z; fr.ok = f2.w != 0.0;
    fr.v[2][0] = f3.x; fr.v[2][1] = f3.y; fr.v[2][2] = f3.z;
  } else {
    nframe_eval(a, i, fr);
  }
  nderiv_apply<EV>(fr, a.ilp_g[i], o);
}

__global__ void k_nframe(ForceArgs<R> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  NFrame fr;
  nframe_eval(a, i, fr);
  d4 *q = a.nframe + 4 * (size_t)i;
  q[0] = make_d4(fr.nx, fr.ny, fr.nz, fr.inn);
  q[1] = make_d4(fr.v[0][0], fr.v[0][1], fr.v[0][2], (double)fr.cont);
  q[2] = make_d4(fr.v[1][0], fr.v[1][1], fr.v[1][2], fr.ok ? 1.0 : 0.0);
  q[3] = make_d4(fr.v[2][0], fr.v[2][1], fr.v[2][2], 0.0);
}

template <bool EV>
__global__ void k_nderiv(ForceArgs<R> a) {
  pdl_enter(a.pdl);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  NDeriv o;
  nderiv_eval<EV>(a, i, o);
  d4 *cs = a.ilp_c + (size_t)i * MAXILP;
  cs[0] = make_d4(o.c[0][0], o.c[0][1], o.c[0][2], 0.0);
  cs[1] = make_d4(o.c[1][0], o.c[1][1], o.c[1][2], 0.0);
  cs[2] = make_d4(o.c[2][0], o.c[2][1], o.c[2][2], 0.0);
  a.ilp_f[i] += o.F[0];
  a.ilp_f[a.n + i] += o.F[1];
  a.ilp_f[2 * a.n + i] += o.F[2];
  if (EV) {
    double *st = a.stat_ilp;
    st[(size_t)2 * a.n + i] += o.W[0]; st[(size_t)3 * a.n + i] += o.W[1]; st[(size_t)4 * a.n + i] += o.W[2];
    st[(size_t)5 * a.n + i] += o.W[3]; st[(size_t)6 * a.n + i] += o.W[4]; st[(size_t)7 * a.n + i] += o.W[5];
  }
}

// The gather's velocity half-kick of atom i (k_nve2's arithmetic on the force just
// stored) and, with kick.drift, the next step's first half (k_nve1's: a second
// half-kick on the same force, then the drift).
__device__ __forceinline__ void kick_atom(const KickArgs &kick, const ForceArgs<R> &a, int i, double Fx, double Fy,
                                          double Fz) {
  const double dtfm = kick.dtfm[__double_as_longlong(a.A.xq[i].w) & 255];
  double vx = kick.v[i] + dtfm * Fx;
  double vy = kick.v[a.n + i] + dtfm * Fy;
  double vz = kick.v[2 * a.n + i] + dtfm * Fz;
  if (kick.drift) {
    vx = vx + dtfm * Fx;
    vy = vy + dtfm * Fy;
    vz = vz + dtfm * Fz;
  }
  kick.v[i] = vx;
  kick.v[a.n + i] = vy;
  kick.v[2 * a.n + i] = vz;
  if (kick.drift) {
    const double d2 = nve_drift(i, vx, vy, vz, kick.dtv, kick.xq, kick.xhold, kick.xh, kick.xl, kick.sys, kick.sysid,
                                kick.do_hilo);
    if (d2 > kick.trig2) atomicOr(kick.status, ST_SKIN_TRIP);
  }
}

// ============================================================== k_finish =========
// Per atom a: its own ILP and Tersoff forces + the slots its neighbours left for it:
// Tersoff bond/three-body forces from every j with a in N_ters(j) and ILP normal-
// derivative forces from every j with a in N_ilp(j).  Fixed summation order.
template <bool EATOM, bool KICK>
__global__ void k_finish(ForceArgs<R> a, KickArgs kick) {
  pdl_enter(a.pdl);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double Fx = 0, Fy = 0, Fz = 0, ea = 0;
  if (a.do_ilp) {
    Fx += a.ilp_f[i]; Fy += a.ilp_f[a.n + i]; Fz += a.ilp_f[2 * a.n + i];
  }
  if (a.do_ters) {
    Fx += a.ters_f[i]; Fy += a.ters_f[a.n + i]; Fz += a.ters_f[2 * a.n + i];
    int cnt = a.ters_cnt[i];
    for (int s = 0; s < cnt; s++) {
      int j, sx, sy, sz;
      decode_entry(a.ters_nb[(size_t)i * MAXTERS + s], a.lc, j, sx, sy, sz);
      uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
      int cj = a.ters_cnt[j];
      for (int t = 0; t < cj; t++) {
        if (a.ters_nb[(size_t)j * MAXTERS + t] == want) {
          d4 g = a.ters_g[(size_t)j * MAXTERS + t];
          Fx += g.x; Fy += g.y; Fz += g.z;
          if (EATOM) ea += 0.5 * g.w;
          break;
        }
      }
    }
  }
  if (a.do_ilp) {
    // the atoms j whose intralayer list holds i: with symmetric intralayer cutoffs they
    // are i's own intralayer neighbours (the exact FP64 distance test is symmetric),
    // otherwise any short candidate of the same molecule
    const bool sym = c_pot.ilp_cut_sym != 0;
    const int cnt = sym ? a.ilp_cnt[i] : a.short_cnt[i];
    const uint32_t *cand = sym ? a.ilp_nb + (size_t)i * MAXILP : a.short_nb + (size_t)i * MAXSHORT;
    const long long mi = sym ? 0 : info_mol(__double_as_longlong(a.A.xq[i].w));
    for (int c = 0; c < cnt; c++) {
      int j, sx, sy, sz;
      decode_entry(cand[c], a.lc, j, sx, sy, sz);
      int cj = a.ilp_cnt[j];
      if (cj == 0) continue;
      if (!sym && info_mol(__double_as_longlong(a.A.xq[j].w)) != mi) continue;
      uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
      for (int t = 0; t < cj; t++) {
        if (a.ilp_nb[(size_t)j * MAXILP + t] == want) {
          d4 g = a.ilp_c[(size_t)j * MAXILP + t];
          Fx += g.x; Fy += g.y; Fz += g.z;
          break;
        }
      }
    }
  }
  a.f_out[i] = Fx;
  a.f_out[a.n + i] = Fy;
  a.f_out[2 * a.n + i] = Fz;
  if constexpr (KICK) kick_atom(kick, a, i, Fx, Fy, Fz);
  if (EATOM) {
    // per-atom energy as the reference's ev_tally splits it: the Tersoff own share was
    // written by k_ters_eatom_own, the partners' halves are gathered above
    double e = a.do_ters ? a.eatom_ters[i] + ea : 0.0;
    if (a.do_ilp) e += a.eatom_ilp[i];
    a.eatom_ters[i] = e;
  }
}

// k_finish with FINISH_LANES lanes per atom, for small systems whose few threads cannot
// hide k_finish's chains of dependent loads (the reverse search of each partner's list).
// A block takes FINISH_ATOMS atoms.  The atom's gather items (its Tersoff partners, then
// its intralayer candidates) are dealt out to its lanes, one item per lane and round, and
// staged in shared memory; then one thread per atom -- a full warp for the block's atoms,
// since GB300 issues an FP64 instruction for the whole warp whatever lanes are active --
// adds them in item order and applies the kick, so the forces are the one-lane
// kernel's to the bit.
constexpr int FINISH_LANES = 8;
constexpr int FINISH_ATOMS = 32;
constexpr int FINISH_LANES_MAX_ATOMS = 65536;
template <bool EATOM, bool KICK>
__global__ void __launch_bounds__(FINISH_LANES * FINISH_ATOMS) k_finish_lanes(ForceArgs<R> a, KickArgs kick) {
  pdl_enter(a.pdl);
  constexpr int L = FINISH_LANES, NA = FINISH_ATOMS, NV = EATOM ? 4 : 3;
  __shared__ double sv[NA][L][NV];
  __shared__ int sf[NA][L];
  __shared__ int stot[NA], snt[NA];
  __shared__ int srounds;
  const int t = threadIdx.x, al = t / L, l = t % L;
  const int i = blockIdx.x * NA + al;
  const bool act = i < a.n;
  const bool sym = c_pot.ilp_cut_sym != 0;
  int nt = 0, ni = 0;
  const uint32_t *cand = nullptr;
  long long mi = 0;
  if (act) {
    nt = a.do_ters ? a.ters_cnt[i] : 0;
    ni = a.do_ilp ? (sym ? a.ilp_cnt[i] : a.short_cnt[i]) : 0;
    cand = sym ? a.ilp_nb + (size_t)i * MAXILP : a.short_nb + (size_t)i * MAXSHORT;
    mi = (sym || !a.do_ilp) ? 0 : info_mol(__double_as_longlong(a.A.xq[i].w));
  }
  const int tot = nt + ni;
  if (l == 0) {
    stot[al] = tot;
    snt[al] = nt;
  }
  __syncthreads();
  if (t < 32) {   // the block's rounds: its largest item count
    int m = t < NA ? stot[t] : 0;
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (t == 0) srounds = (m + L - 1) / L;
  }
  // the adding thread of atom i2 (threads t < NA)
  const int i2 = blockIdx.x * NA + t;
  const bool adder = t < NA && i2 < a.n;
  double Fx = 0, Fy = 0, Fz = 0, ea = 0;
  int tot2 = 0, nt2 = 0;
  if (adder) {
    if (a.do_ilp) {
      Fx += a.ilp_f[i2]; Fy += a.ilp_f[a.n + i2]; Fz += a.ilp_f[2 * a.n + i2];
    }
    if (a.do_ters) {
      Fx += a.ters_f[i2]; Fy += a.ters_f[a.n + i2]; Fz += a.ters_f[2 * a.n + i2];
    }
  }
  __syncthreads();
  if (adder) {
    tot2 = stot[t];
    nt2 = snt[t];
  }
  const int rounds = srounds;
  for (int r = 0; r < rounds; r++) {
    const int q = r * L + l;
    int found = 0;
    d4 g = make_d4(0.0, 0.0, 0.0, 0.0);
    if (act && q < nt) {
      int j, sx, sy, sz;
      decode_entry(a.ters_nb[(size_t)i * MAXTERS + q], a.lc, j, sx, sy, sz);
      const uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
      const int cj = a.ters_cnt[j];
      for (int u = 0; u < cj; u++) {
        if (a.ters_nb[(size_t)j * MAXTERS + u] == want) {
          g = a.ters_g[(size_t)j * MAXTERS + u];
          found = 1;
          break;
        }
      }
    } else if (act && q < tot) {
      int j, sx, sy, sz;
      decode_entry(cand[q - nt], a.lc, j, sx, sy, sz);
      const int cj = a.ilp_cnt[j];
      if (cj > 0 && (sym || info_mol(__double_as_longlong(a.A.xq[j].w)) == mi)) {
        const uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
        for (int u = 0; u < cj; u++) {
          if (a.ilp_nb[(size_t)j * MAXILP + u] == want) {
            g = a.ilp_c[(size_t)j * MAXILP + u];
            found = 1;
            break;
          }
        }
      }
    }
    sv[al][l][0] = g.x;
    sv[al][l][1] = g.y;
    sv[al][l][2] = g.z;
    if (EATOM) sv[al][l][NV - 1] = g.w;
    sf[al][l] = found;
    __syncthreads();
    if (adder) {
#pragma unroll
      for (int k = 0; k < L; k++) {
        const int qq = r * L + k;
        if (qq < tot2 && sf[t][k]) {
          Fx += sv[t][k][0]; Fy += sv[t][k][1]; Fz += sv[t][k][2];
          if (EATOM && qq < nt2) ea += 0.5 * sv[t][k][NV - 1];
        }
      }
    }
    __syncthreads();
  }
  if (!adder) return;
  a.f_out[i2] = Fx;
  a.f_out[a.n + i2] = Fy;
  a.f_out[2 * a.n + i2] = Fz;
  if constexpr (KICK) kick_atom(kick, a, i2, Fx, Fy, Fz);
  if (EATOM) {
    double e = a.do_ters ? a.eatom_ters[i2] + ea : 0.0;
    if (a.do_ilp) e += a.eatom_ilp[i2];
    a.eatom_ters[i2] = e;
  }
}

// Tersoff per-atom energy, own share (half of each bond energy centred here and half of
// each repulsion from this end), written before k_finish adds the partners' halves.
__global__ void k_ters_eatom_own(ForceArgs<R> a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double e = 0.0;
  int cnt = a.ters_cnt[i];
  for (int s = 0; s < cnt; s++) e += 0.5 * a.ters_g[(size_t)i * MAXTERS + s].w;
  // stat_ters[i] = sum of bond energies centred at i + half repulsions from this end
  double bonds = 0.0;
  for (int s = 0; s < cnt; s++) bonds += a.ters_g[(size_t)i * MAXTERS + s].w;
  a.eatom_ters[i] = (a.stat_ters[i] - bonds) + e;
}

// Per-atom virial pass, both precision modes: atom i's slots, the halves of its
// normal-derivative tallies that its intralayer neighbours m receive,
// 0.5 (v_m (x) c_m(g_i) + [c_m(G_i row p)]_pb), from its FP64 frame and the sums
// g_i = sum_j c_ij del_ij, G_i = sum_j c_ij del_ij (x) del_ij of the terms it owns
// (c_m(g) = -(dn_i/dx_m)^T g; zero slots when i owns none or has no frame).
__device__ __forceinline__ void va_write_slots(const ForceArgs<R> &a, int i, bool on, const NFrame &fri, double gx,
                                               double gy, double gz, const double G[6]) {
  double s[MAXILP][6];
#pragma unroll
  for (int m = 0; m < MAXILP; m++)
#pragma unroll
    for (int k = 0; k < 6; k++) s[m][k] = 0.0;
  if (on && fri.ok) {
    NDeriv og, o0, o1, o2;
    nderiv_apply<false>(fri, make_d4(gx, gy, gz, 0.0), og);
    nderiv_apply<false>(fri, make_d4(G[0], G[3], G[4], 0.0), o0);   // row x of G
    nderiv_apply<false>(fri, make_d4(G[3], G[1], G[5], 0.0), o1);   // row y
    nderiv_apply<false>(fri, make_d4(G[4], G[5], G[2], 0.0), o2);   // row z
#pragma unroll
    for (int m = 0; m < MAXILP; m++) {
      if (m >= fri.cont) break;
      const double *v = fri.v[m];
      s[m][0] = 0.5 * (v[0] * og.c[m][0] + o0.c[m][0]);
      s[m][1] = 0.5 * (v[1] * og.c[m][1] + o1.c[m][1]);
      s[m][2] = 0.5 * (v[2] * og.c[m][2] + o2.c[m][2]);
      s[m][3] = 0.5 * (v[0] * og.c[m][1] + o0.c[m][1]);
      s[m][4] = 0.5 * (v[0] * og.c[m][2] + o0.c[m][2]);
      s[m][5] = 0.5 * (v[1] * og.c[m][2] + o1.c[m][2]);
    }
  }
#pragma unroll
  for (int m = 0; m < MAXILP; m++)
#pragma unroll
    for (int k = 0; k < 6; k++) a.va_is[((size_t)i * MAXILP + m) * 6 + k] = s[m][k];
}

#ifndef LMFF_PACKED_X2
// ===================================================== per-atom virial (FP64) =====
// Pair::vatom as the reference's tallies split it (pair.cpp ev_tally :913, ev_tally_xyz
// :1060, v_tally3 :1435), run on request after an evaluation in either precision mode:
// FP64 kernels from the FP64 positions, lists and constants.  Deterministic like the
// forces: every atom sums its own shares, and the shares it cannot form itself are left
// in per-slot arrays by the atom that can and gathered in a fixed order.
//
// ILP (pair_ilp_graphene_hbn.cpp:536, :667, :671).  For atom i and each interlayer
// neighbour j (del = x_i - x_j):
//   * vdW: ev_tally of fsum along del, half to each end, once per pair;
//   * the repulsion term with i's normal (i owns it): ev_tally_xyz of its pair force fkc
//     along del, half to i; and its normal-derivative forces fk on i's intralayer
//     neighbours m, tallied against x_m - x_j, half to m and half to j.  j's half is
//     formed by j (below); m's half is summed over j here through
//       sum_j (x_m - x_j) (x) fk_jm = v_m (x) c_m(g_i) + [c_m(G_i row p)]_pb,
//     with v_m = x_m - x_i, c_m(g) = -(dn_i/dx_m)^T g the normal-derivative force for a
//     vector g, g_i = sum_j c_ij del and G_i = sum_j c_ij del (x) del (c_ij = Tap prod
//     fpair1): the first from the whole of g_i, the second from the three rows of the
//     symmetric G_i, four applications of i's frame, written to i's slot of m;
//   * the term with j's normal (i is its partner): half of its pair force's tally, and
//     i's half of its normal-derivative tallies, sum_m (x_m - x_i) (x) fk_m over j's
//     intralayer neighbours m, = W_j + del_ji (x) sum_m c_m from one application of j's
//     frame to g = c_ji del_ji (W_j = sum_m v_m (x) c_m, the assembly's own virial).
// Subdomain mode: vdW when the end the tag-parity half keeps is owned, each repulsion
// term when its normal's atom is owned.

// the frame k_nframe left for atom i and the normal it carries: the reference's (0,0,1)
// for fewer than two intralayer neighbours (calc_normal, pair_ilp_graphene_hbn.cpp:800-806)
__device__ __forceinline__ void va_frame(const ForceArgs<R> &a, int i, NFrame &fr, double &nx, double &ny,
                                         double &nz) {
  const d4 f0 = a.nframe[4 * (size_t)i], f1 = a.nframe[4 * (size_t)i + 1], f2 = a.nframe[4 * (size_t)i + 2],
           f3 = a.nframe[4 * (size_t)i + 3];
  fr.nx = f0.x; fr.ny = f0.y; fr.nz = f0.z; fr.inn = f0.w;
  fr.v[0][0] = f1.x; fr.v[0][1] = f1.y; fr.v[0][2] = f1.z; fr.cont = (int)f1.w;
  fr.v[1][0] = f2.x; fr.v[1][1] = f2.y; fr.v[1][2] = f2.z; fr.ok = f2.w != 0.0;
  fr.v[2][0] = f3.x; fr.v[2][1] = f3.y; fr.v[2][2] = f3.z;
  if (fr.cont >= 2) {
    nx = fr.nx; ny = fr.ny; nz = fr.nz;
  } else {
    nx = 0.0; ny = 0.0; nz = 1.0;
  }
}

// one repulsion term (calc_FRep :609-640, kolmogorov/crespi/full :600-645) with normal n
// along del: its pair force fkc and c = Tap prod fpair1, the weight of its normal-
// derivative forces
template <bool KC>
__device__ __forceinline__ void va_rep(const IlpP<double> &p, double nx, double ny, double nz, double dx, double dy,
                                       double dz, double rsq, double r, double Tap, double dTap, double fkc[3],
                                       double &c) {
  const double prod = nx * dx + ny * dy + nz * dz;
  const double rhosq = rsq - prod * prod;
  const double x = rhosq * p.delta2inv;
  const double exp0 = exp(-p.lambda * (r - p.z0));
  const double exp1 = exp(-x);
  double V, fpair, fpair1;
  if constexpr (KC) {
    const double sumC1 = p.kc_C0 + p.kc_C2 * x + p.kc_C4 * x * x;
    const double sumC11 = (p.kc_C2 + 2.0 * p.kc_C4 * x) * p.delta2inv;
    const double E = p.eps_half + exp1 * sumC1;
    V = exp0 * E;
    fpair = p.lambda * exp0 / r * E;
    fpair1 = 2.0 * exp0 * exp1 * (p.delta2inv * sumC1 - sumC11);
  } else {
    const double frho = exp1 * p.C;
    const double E = p.eps_half + frho;
    V = exp0 * E;
    fpair = p.lambda * exp0 / r * E;
    fpair1 = 2.0 * exp0 * frho * p.delta2inv;
  }
  const double fsum = fpair + fpair1;
  fkc[0] = (dx * fsum - prod * nx * fpair1) * Tap - V * dTap * dx / r;
  fkc[1] = (dy * fsum - prod * ny * fpair1) * Tap - V * dTap * dy / r;
  fkc[2] = (dz * fsum - prod * nz * fpair1) * Tap - V * dTap * dz / r;
  c = Tap * prod * fpair1;
}

// v += s * (d (x) f) in LAMMPS order (ev_tally_xyz's v[6])
__device__ __forceinline__ void va_add_xyz(double v[6], double s, double dx, double dy, double dz, const double f[3]) {
  v[0] += s * (dx * f[0]); v[1] += s * (dy * f[1]); v[2] += s * (dz * f[2]);
  v[3] += s * (dx * f[1]); v[4] += s * (dx * f[2]); v[5] += s * (dy * f[2]);
}

template <bool GH, bool KC>
__global__ void __launch_bounds__(128) k_va_ilp(ForceArgs<R> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double w[6] = {0, 0, 0, 0, 0, 0};
  double gx = 0, gy = 0, gz = 0;
  double G[6] = {0, 0, 0, 0, 0, 0};   // xx yy zz xy xz yz
  const long long iinfo = __double_as_longlong(a.A.xq[i].w);
  const int ie = c_pot.i_map[info_type(iinfo)];
  const bool iown = !GH || owned(a, i);
  NFrame fri;
  double nix, niy, niz;
  va_frame(a, i, fri, nix, niy, niz);
  if (ie >= 0) {
    const SysDesc &sd = a.A.sys[a.A.sysid[i]];
    const long long mi = info_mol(iinfo);
    const long long itag = a.tag[i];
    const double cutsq = c_pot.i_cutsq;
    const int64_t q1 = a.list_off[i + 1];
    for (int64_t q = a.list_off[i]; q < q1; q++) {
      int j, sx, sy, sz;
      decode_entry(a.list[q], a.lc, j, sx, sy, sz);
      const long long jinfo = __double_as_longlong(a.A.xq[j].w);
      if (info_mol(jinfo) == mi) continue;
      const int je = c_pot.i_map[info_type(jinfo)];
      if (je < 0) continue;
      double dx, dy, dz;
      disp64(a.A.xq, sd, i, j, sx, sy, sz, dx, dy, dz);
      const double rsq = rsq_rn(dx, dy, dz);
      if (!(rsq < cutsq)) continue;
      const double r = sqrt(rsq);
      double Tap = 1.0, dTap = 0.0;
      if (c_pot.tap) {
        // Tap = 20x^7 - 70x^6 + 84x^5 - 35x^4 + 1, dTap/dr = 140 x^3 (x - 1)^3 / Rcut
        const double xr = r * c_pot.i_inv_rcut, x2 = xr * xr;
        Tap = (((20.0 * xr - 70.0) * xr + 84.0) * xr - 35.0) * (x2 * x2) + 1.0;
        const double y = x2 - xr;
        dTap = (y * y) * (y * (140.0 * c_pot.i_inv_rcut));
      }
      const bool jown = !GH || owned(a, j);
      const long long jtag = a.tag[j];
      const bool keep = GH ? keep_half_r(itag, jtag, -dx, -dy, -dz) : keep_half(itag, jtag, sx, sy, sz);
      // ---- vdW (calc_FvdW :506-540), the kept end's parameters
      if (!GH || (keep ? iown : jown)) {
        const IlpP<double> &pv = c_pot.ilp[(keep || c_pot.vdw_sym) ? ie * MAXELEM + je : je * MAXELEM + ie];
        const double r2inv = 1.0 / rsq, r6inv = r2inv * r2inv * r2inv, r8inv = r6inv * r2inv;
        double Vv, fpv;
        if constexpr (KC) {
          Vv = -pv.kc_Az06 * r6inv;
          fpv = -6.0 * pv.kc_Az06 * r8inv;
        } else {
          const double TS = 1.0 + exp(-pv.d * (r / pv.seff - 1.0));
          const double TS2inv = 1.0 / (TS * TS);
          Vv = -pv.C6 * r6inv / TS;
          fpv = -6.0 * pv.C6 * r8inv / TS + pv.C6 * pv.d / pv.seff * (TS - 1.0) * TS2inv * r8inv * r;
        }
        const double fs = fpv * Tap - Vv * dTap / r;
        const double f3[3] = {fs * dx, fs * dy, fs * dz};
        va_add_xyz(w, 0.5, dx, dy, dz, f3);
      }
      // ---- the term with i's normal
      if (iown) {
        double fkc[3], c;
        va_rep<KC>(c_pot.ilp[ie * MAXELEM + je], nix, niy, niz, dx, dy, dz, rsq, r, Tap, dTap, fkc, c);
        va_add_xyz(w, 0.5, dx, dy, dz, fkc);
        gx += c * dx; gy += c * dy; gz += c * dz;
        G[0] += c * (dx * dx); G[1] += c * (dy * dy); G[2] += c * (dz * dz);
        G[3] += c * (dx * dy); G[4] += c * (dx * dz); G[5] += c * (dy * dz);
      }
      // ---- the term with j's normal, i its partner: del' = x_j - x_i
      if (jown) {
        NFrame frj;
        double njx, njy, njz;
        va_frame(a, j, frj, njx, njy, njz);
        const double ex = -dx, ey = -dy, ez = -dz;
        double fkc[3], c;
        va_rep<KC>(c_pot.ilp[je * MAXELEM + ie], njx, njy, njz, ex, ey, ez, rsq, r, Tap, dTap, fkc, c);
        va_add_xyz(w, 0.5, ex, ey, ez, fkc);
        if (frj.ok) {
          NDeriv o;
          nderiv_apply<true>(frj, make_d4(c * ex, c * ey, c * ez, 0.0), o);
          const double sc[3] = {o.c[0][0] + o.c[1][0] + o.c[2][0], o.c[0][1] + o.c[1][1] + o.c[2][1],
                                o.c[0][2] + o.c[1][2] + o.c[2][2]};
#pragma unroll
          for (int k = 0; k < 6; k++) w[k] += 0.5 * o.W[k];
          va_add_xyz(w, 0.5, ex, ey, ez, sc);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 6; k++) a.va_i[6 * (size_t)i + k] = w[k];
  va_write_slots(a, i, ie >= 0 && iown, fri, gx, gy, gz, G);
}

// Per atom: its own shares plus the slots its Tersoff bond partners and the atoms whose
// intralayer list holds it left for it (found as k_finish finds its force slots), in a
// fixed order, into out[6 n] (sorted order).
__global__ void __launch_bounds__(128) k_va_gather(ForceArgs<R> a, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double w[6] = {0, 0, 0, 0, 0, 0};
  if (a.do_ters) {
#pragma unroll
    for (int k = 0; k < 6; k++) w[k] += a.va_t[6 * (size_t)i + k];
    const int cnt = a.ters_cnt[i];
    for (int s = 0; s < cnt; s++) {
      int j, sx, sy, sz;
      decode_entry(a.ters_nb[(size_t)i * MAXTERS + s], a.lc, j, sx, sy, sz);
      const uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
      const int cj = a.ters_cnt[j];
      for (int t = 0; t < cj; t++) {
        if (a.ters_nb[(size_t)j * MAXTERS + t] == want) {
          const double *v = a.va_ts + ((size_t)j * MAXTERS + t) * 6;
#pragma unroll
          for (int k = 0; k < 6; k++) w[k] += v[k];
          break;
        }
      }
    }
  }
  if (a.do_ilp) {
#pragma unroll
    for (int k = 0; k < 6; k++) w[k] += a.va_i[6 * (size_t)i + k];
    const bool sym = c_pot.ilp_cut_sym != 0;
    const int cnt = sym ? a.ilp_cnt[i] : a.short_cnt[i];
    const uint32_t *cand = sym ? a.ilp_nb + (size_t)i * MAXILP : a.short_nb + (size_t)i * MAXSHORT;
    const long long mi = sym ? 0 : info_mol(__double_as_longlong(a.A.xq[i].w));
    for (int c = 0; c < cnt; c++) {
      int j, sx, sy, sz;
      decode_entry(cand[c], a.lc, j, sx, sy, sz);
      const int cj = a.ilp_cnt[j];
      if (cj == 0) continue;
      if (!sym && info_mol(__double_as_longlong(a.A.xq[j].w)) != mi) continue;
      const uint32_t want = encode_entry(i, -sx, -sy, -sz, a.lc);
      for (int t = 0; t < cj; t++) {
        if (a.ilp_nb[(size_t)j * MAXILP + t] == want) {
          const double *v = a.va_is + ((size_t)j * MAXILP + t) * 6;
#pragma unroll
          for (int k = 0; k < 6; k++) w[k] += v[k];
          break;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 6; k++) out[6 * (size_t)i + k] = w[k];
}
#else   // LMFF_PACKED_X2: the mixed engines' interlayer per-atom virial
// The same split as k_va_ilp with the pair terms in the pair kernel's FP32 form:
//  * the own share is half of del (x) f_ij over the atom's interlayer pairs, f_ij the
//    per-pair force on i the pair kernel forms (vdW, both repulsion terms' pair forces;
//    the three tallies of a pair sum to exactly this);
//  * the partner j's normal-derivative share, W_j(g) + del_ji (x) sum_m c_m(g) for
//    g = c_ji del_ji = Tap q fpair1(j) del, is linear in g: with the 27 numbers of
//    k_va_tens per atom (A[k][a] = W_j(e_a)[k], B[a][b] = sum_m c_m(e_a)[b]) it is
//    sum_a A[k][a] g_a - del_p(k) sum_a B[a][b(k)] g_a;
//  * g_i, G_i and the shares are summed in FP64, and the slots come from the FP64 frame.

// per atom: A (18, row-major k, a) then B (9, row-major a, b), from three applications
// of the FP64 frame to the unit vectors, stored as FP32 in 7 float4
__global__ void __launch_bounds__(128) k_va_tens(ForceArgs<R> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  NFrame fr;
  nframe_eval(a, i, fr);
  float t[28];
#pragma unroll
  for (int k = 0; k < 28; k++) t[k] = 0.f;
  if (fr.ok) {
#pragma unroll
    for (int e = 0; e < 3; e++) {
      NDeriv o;
      nderiv_apply<true>(fr, make_d4(e == 0 ? 1.0 : 0.0, e == 1 ? 1.0 : 0.0, e == 2 ? 1.0 : 0.0, 0.0), o);
#pragma unroll
      for (int k = 0; k < 6; k++) t[3 * k + e] = (float)o.W[k];
#pragma unroll
      for (int b = 0; b < 3; b++) t[18 + 3 * e + b] = (float)(o.c[0][b] + o.c[1][b] + o.c[2][b]);
    }
  }
  float4 *q = a.va_tens + 7 * (size_t)i;
#pragma unroll
  for (int k = 0; k < 7; k++) q[k] = make_float4(t[4 * k], t[4 * k + 1], t[4 * k + 2], t[4 * k + 3]);
}

template <bool GH, bool KC>
__global__ void __launch_bounds__(128) k_va_ilp32(ForceArgs<R> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double w[6] = {0, 0, 0, 0, 0, 0};
  double gx = 0, gy = 0, gz = 0;
  double G[6] = {0, 0, 0, 0, 0, 0};   // xx yy zz xy xz yz
  AtomI<R> ai;
  ai.load(a.A, i);
  const int ie = c_pot.i_map[info_type(ai.info)];
  const bool iown = !GH || owned(a, i);
  if (ie >= 0) {
    const SysDesc &sd = a.A.sys[a.A.sysid[i]];
    const long long mi = info_mol(ai.info);
    const long long itag = a.tag[i];
    const float4 ni = a.nrm32[i];
    const int64_t q1 = a.list_off[i + 1];
    for (int64_t q = a.list_off[i]; q < q1; q++) {
      int j, sx, sy, sz;
      decode_entry(a.list[q], a.lc, j, sx, sy, sz);
      R dx, dy, dz;
      long long jinfo;
      ai.disp(a.A, sd, j, sx, sy, sz, dx, dy, dz, jinfo);
      if (info_mol(jinfo) == mi) continue;
      const int je = c_pot.i_map[info_type(jinfo)];
      if (je < 0) continue;
      const R rsq = dx * dx + dy * dy + dz * dz;
      if (!(rsq < c_pot.i_cutsq)) continue;
      const R rinv = rsqrt_ftz(rsq), r = rsq * rinv;
      R Tap = 1, dTap = 0;
      if (c_pot.tap) {
        const R x = r * c_pot.i_inv_rcut, x2 = x * x;
        Tap = ((R(20) * x + R(-70)) * x + R(84)) * x + R(-35);
        Tap = Tap * (x2 * x2) + R(1);
        const R y = x2 - x;
        dTap = (y * y) * (y * (R(140) * c_pot.i_inv_rcut));
      }
      const bool jown = !GH || owned(a, j);
      const bool keep = GH ? keep_half_r(itag, a.tag[j], -dx, -dy, -dz)
                           : (c_pot.vdw_sym || keep_half(itag, a.tag[j], sx, sy, sz));
      const R wi = iown ? R(1) : R(0), wj = jown ? R(1) : R(0);
      const R wv = GH ? ((keep ? iown : jown) ? R(1) : R(0)) : R(1);
      const IlpP<R> &pij = c_pot.ilp[ie * MAXELEM + je];
      const IlpP<R> &pji = c_pot.ilp[je * MAXELEM + ie];
      const IlpP<R> &pv = (c_pot.vdw_sym || keep) ? pij : pji;
      const R r2inv = rinv * rinv, r6inv = r2inv * r2inv * r2inv, r8inv = r6inv * r2inv;
      R Vv, fpv;
      if constexpr (KC) {
        Vv = -pv.kc_Az06 * r6inv;
        fpv = R(-6) * pv.kc_Az06 * r8inv;
      } else {
        const R TS = R(1) + Math<R>::exp_ts(pv, r), TSinv = Math<R>::rcp(TS);
        Vv = -pv.C6 * r6inv * TSinv;
        fpv = pv.C6 * r8inv * TSinv * (R(-6) + pv.d_over_seff * (TS - R(1)) * TSinv * r);
      }
      const R fsum_v = (fpv * Tap - Vv * dTap * rinv) * wv;
      const float4 nj = a.nrm32[j];
      const R p = ni.x * dx + ni.y * dy + ni.z * dz;
      const R qq = nj.x * dx + nj.y * dy + nj.z * dz;
      R V, fpair1, fsum, V2, fpair1b, fsum2;
      const R exp0 = Math<R>::exp_rep0(pij, r);
      rep_term<KC>(pij, exp0, Math<R>::exp_rep1(pij, rsq - p * p), rsq - p * p, rinv, V, fpair1, fsum);
      const R exp0b = pji.same_as_swapped ? exp0 : Math<R>::exp_rep0(pji, r);
      rep_term<KC>(pji, exp0b, Math<R>::exp_rep1(pji, rsq - qq * qq), rsq - qq * qq, rinv, V2, fpair1b, fsum2);
      V *= wi; fpair1 *= wi; fsum *= wi;
      V2 *= wj; fpair1b *= wj; fsum2 *= wj;
      const R crad = fsum_v + (fsum + fsum2) * Tap - (V + V2) * dTap * rinv;
      const R tp1 = Tap * p * fpair1, tq1 = Tap * qq * fpair1b;
      const R fx = crad * dx - tp1 * ni.x - tq1 * nj.x;
      const R fy = crad * dy - tp1 * ni.y - tq1 * nj.y;
      const R fz = crad * dz - tp1 * ni.z - tq1 * nj.z;
      w[0] += 0.5 * (double)(dx * fx); w[1] += 0.5 * (double)(dy * fy); w[2] += 0.5 * (double)(dz * fz);
      w[3] += 0.5 * (double)(dx * fy); w[4] += 0.5 * (double)(dx * fz); w[5] += 0.5 * (double)(dy * fz);
      gx += (double)(tp1 * dx); gy += (double)(tp1 * dy); gz += (double)(tp1 * dz);
      G[0] += (double)(tp1 * (dx * dx)); G[1] += (double)(tp1 * (dy * dy)); G[2] += (double)(tp1 * (dz * dz));
      G[3] += (double)(tp1 * (dx * dy)); G[4] += (double)(tp1 * (dx * dz)); G[5] += (double)(tp1 * (dy * dz));
      if (tq1 != R(0)) {
        // the partner's normal-derivative share, g = tq1 del
        const R g0 = tq1 * dx, g1 = tq1 * dy, g2 = tq1 * dz;
        const float4 *tt = a.va_tens + 7 * (size_t)j;
        const float4 t0 = tt[0], t1 = tt[1], t2 = tt[2], t3 = tt[3], t4 = tt[4], t5 = tt[5], t6 = tt[6];
        // A[k][e] = t[3k + e], B[e][b] = t[18 + 3e + b]
        const R A0 = t0.x * g0 + t0.y * g1 + t0.z * g2;   // k = 0 (xx)
        const R A1 = t0.w * g0 + t1.x * g1 + t1.y * g2;   // k = 1 (yy)
        const R A2 = t1.z * g0 + t1.w * g1 + t2.x * g2;   // k = 2 (zz)
        const R A3 = t2.y * g0 + t2.z * g1 + t2.w * g2;   // k = 3 (xy)
        const R A4 = t3.x * g0 + t3.y * g1 + t3.z * g2;   // k = 4 (xz)
        const R A5 = t3.w * g0 + t4.x * g1 + t4.y * g2;   // k = 5 (yz)
        const R s0 = t4.z * g0 + t5.y * g1 + t6.x * g2;   // sum_e B[e][0] g_e
        const R s1 = t4.w * g0 + t5.z * g1 + t6.y * g2;   // b = 1
        const R s2 = t5.x * g0 + t5.w * g1 + t6.z * g2;   // b = 2
        w[0] += 0.5 * (double)(A0 - dx * s0); w[1] += 0.5 * (double)(A1 - dy * s1);
        w[2] += 0.5 * (double)(A2 - dz * s2); w[3] += 0.5 * (double)(A3 - dx * s1);
        w[4] += 0.5 * (double)(A4 - dx * s2); w[5] += 0.5 * (double)(A5 - dy * s2);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 6; k++) a.va_i[6 * (size_t)i + k] = w[k];
  NFrame fri;
  nframe_eval(a, i, fri);
  va_write_slots(a, i, ie >= 0 && iown, fri, gx, gy, gz, G);
}
#endif  // LMFF_PACKED_X2

// ============================================================ host launchers ======

void upload_pot(const PotConst<R> &p, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_pot, &p, sizeof(p), 0, cudaMemcpyHostToDevice, s);
  if (sizeof(R) == 8) k_fill_exp2_f64<<<1, EXP2_F64_N, 0, s>>>();
#ifdef LMFF_PACKED_X2
  {
    static PairX2Const x2;   // static: the asynchronous copy reads it after return
    const IlpP<float> &q = p.ilp[0];
    x2.tap0 = make_float2(20.f, 140.f);
    x2.tap1 = make_float2(-70.f, -420.f);
    x2.tap2 = make_float2(84.f, 420.f);
    x2.tap3 = make_float2(-35.f, -140.f);
    x2.nd2_l2e = make_float2(q.nd2_l2e, q.nd2_l2e);
    x2.C = make_float2(q.C, q.C);
    x2.eps_half = make_float2(q.eps_half, q.eps_half);
    x2.d2x2 = make_float2(2.f * q.delta2inv, 2.f * q.delta2inv);
    x2.lambda = make_float2(q.lambda, q.lambda);
    const double irc = (double)p.i_inv_rcut, i4 = irc * irc * irc * irc;
    auto dup = [](double v) { return make_float2((float)v, (float)v); };
    x2.ta0 = dup(20.0 * i4 * irc * irc * irc);
    x2.ta1 = dup(-70.0 * i4 * irc * irc);
    x2.ta2 = dup(84.0 * i4 * irc);
    x2.ta3 = dup(-35.0 * i4);
    x2.td0 = dup(140.0 * i4 * irc * irc * irc);
    x2.td1 = dup(-420.0 * i4 * irc * irc);
    x2.td2 = dup(420.0 * i4 * irc);
    x2.td3 = dup(-140.0 * i4);
    x2.one = make_float2(1.f, 1.f);
    x2.nts_a = make_float2(-q.ts_a, -q.ts_a);
    x2.ts_a_seff = make_float2(q.ts_a * q.seff, q.ts_a * q.seff);
    x2.C6 = make_float2(q.C6, q.C6);
    x2.d_over_seff = make_float2(q.d_over_seff, q.d_over_seff);
    x2.m6 = make_float2(-6.f, -6.f);
    x2.nlam_l2e = make_float2(-q.lam_l2e, -q.lam_l2e);
    x2.lamz0_l2e = make_float2(q.lamz0_l2e, q.lamz0_l2e);
    // the two-pair body runs only for C >= 0 (log2 0 = -inf gives 2^-inf = 0)
    const float l2c = q.C > 0.f ? (float)std::log2((double)q.C) : -INFINITY;
    x2.log2C = make_float2(l2c, l2c);
    x2.eps = make_float2(2.f * q.eps_half, 2.f * q.eps_half);
    cudaMemcpyToSymbolAsync(c_x2, &x2, sizeof(x2), 0, cudaMemcpyHostToDevice, s);
    // kept out of PotConst: growing c_pot changes the single-element pair kernel's
    // register allocation (measured: a spill and -2 %)
    static int p2m;
    p2m = (p.i_enabled && !p.kc && p.vdw_sym) ? 1 : 0;
    for (int ea = 0; ea < p.i_ne; ea++)
      for (int eb = 0; eb < p.i_ne; eb++) {
        const IlpP<float> &o = p.ilp[ea * MAXELEM + eb];
        if (!o.same_as_swapped || !(o.C >= 0.f)) p2m = 0;
      }
    h_two_multi = p2m;
    h_two_one = (p.i_enabled && !p.kc && p.ilp[0].C >= 0.f) ? 1 : 0;
    if (p2m) {
      static float2 tab[X2M_ROWS * X2M_N];
      for (int ea = 0; ea < MAXELEM; ea++)
        for (int eb = 0; eb < MAXELEM; eb++)
          for (int ec = 0; ec < MAXELEM; ec++) {
            const IlpP<float> &u = p.ilp[ea * MAXELEM + eb], &v = p.ilp[ea * MAXELEM + ec];
            auto two = [](float x, float y) { return make_float2(x, y); };
            auto l2c = [](float c) { return c > 0.f ? (float)std::log2((double)c) : -INFINITY; };
            float2 *t = tab + ((ea * MAXELEM + eb) * MAXELEM + ec) * X2M_N;
            t[0] = two(u.nd2_l2e, v.nd2_l2e);
            t[1] = two(l2c(u.C), l2c(v.C));
            t[2] = two(2.f * u.eps_half, 2.f * v.eps_half);
            t[3] = two(2.f * u.delta2inv, 2.f * v.delta2inv);
            t[4] = two(u.lambda, v.lambda);
            t[5] = two(-u.lam_l2e, -v.lam_l2e);
            t[6] = two(u.lamz0_l2e, v.lamz0_l2e);
            t[7] = two(-u.ts_a, -v.ts_a);
            t[8] = two(u.ts_a * u.seff, v.ts_a * v.seff);
            t[9] = two(u.C6, v.C6);
            t[10] = two(u.d_over_seff, v.d_over_seff);
          }
      cudaMemcpyToSymbolAsync(g_x2m, tab, sizeof(tab), 0, cudaMemcpyHostToDevice, s);
    }
  }
#endif
  if (sizeof(R) == 4) k_fill_exptab<<<EXP_TAB_N / 256, 256, 0, s>>>();
}

void launch_short(const ForceArgs<R> &a, const double *cutILPsq64, double tcutmaxsq64, cudaStream_t s) {
  if (a.n == 0) return;
  const bool p = (a.pdl & PDL_SHORT) != 0;
  if (a.no_small)
    launch_pdl(p, k_short<1>, (a.n + 127) / 128, 128, s, a, cutILPsq64, tcutmaxsq64);
  else if (a.n <= SHORT_SG16_MAX_ATOMS)
    launch_pdl(p, k_short<16>, (int)(((long long)a.n * 16 + 127) / 128), 128, s, a, cutILPsq64, tcutmaxsq64);
  else if (a.n <= SHORT_SG_MAX_ATOMS)
    launch_pdl(p, k_short<4>, (int)(((long long)a.n * 4 + 127) / 128), 128, s, a, cutILPsq64, tcutmaxsq64);
  else launch_pdl(p, k_short<1>, (a.n + 127) / 128, 128, s, a, cutILPsq64, tcutmaxsq64);
}

void launch_tersoff(const ForceArgs<R> &a, bool ev, bool eatom, cudaStream_t s) {
  if (a.n == 0) return;
  const int b = per_atom_block(a.n);
  const int g = (a.n + b - 1) / b;
  if (a.own_perm) {
    if (ev) k_tersoff<true, false, true><<<g, b, 0, s>>>(a);
    else k_tersoff<false, false, true><<<g, b, 0, s>>>(a);
  } else if (ev) {
    k_tersoff<true, false, false><<<g, b, 0, s>>>(a);
  } else if (a.ters_alone && a.n <= TERS_LANES_MAX_ATOMS && !a.no_small) {
    k_tersoff_lanes<<<(int)(((long long)a.n * TERS_LANES + 127) / 128), 128, 0, s>>>(a);
  } else {
    k_tersoff<false, false, false><<<g, b, 0, s>>>(a);
  }
  if (ev && eatom) k_ters_eatom_own<<<g, b, 0, s>>>(a);
}

template <int TPA, bool ONE>
static void launch_ilp_t(const ForceArgs<R> &a, bool ev, bool eatom, int block, cudaStream_t s) {
  long long threads = (long long)a.n * TPA;
  int g = (int)((threads + block - 1) / block);
  const bool p = (a.pdl & PDL_ILP) != 0;
  if (a.kc) {
    if (ev && eatom) launch_pdl(p, k_ilp<TPA, true, true, ONE, false, true, false>, g, block, s, a);
    else if (ev) launch_pdl(p, k_ilp<TPA, true, false, ONE, false, true, false>, g, block, s, a);
    else launch_pdl(p, k_ilp<TPA, false, false, ONE, false, true, false>, g, block, s, a);
    return;
  }
  if (ev && eatom) launch_pdl(p, k_ilp<TPA, true, true, ONE, false, false, false>, g, block, s, a);
  else if (ev) launch_pdl(p, k_ilp<TPA, true, false, ONE, false, false, false>, g, block, s, a);
  else if (TWO_PAIR_BODY && !a.list_full && a.pair_tile != 1 && (ONE ? h_two_one : h_two_multi))
    launch_pdl(p, k_ilp<TPA, false, false, ONE, false, false, TWO_PAIR_BODY>, g, block, s, a);
  else launch_pdl(p, k_ilp<TPA, false, false, ONE, false, false, false>, g, block, s, a);
}

template <bool ONE>
static void launch_ilp_one(const ForceArgs<R> &a, bool ev, bool eatom, int tpa, int block, cudaStream_t s) {
  switch (tpa) {
    case 4: launch_ilp_t<4, ONE>(a, ev, eatom, block, s); break;
    case 8: launch_ilp_t<8, ONE>(a, ev, eatom, block, s); break;
    case 16: launch_ilp_t<16, ONE>(a, ev, eatom, block, s); break;
    default: launch_ilp_t<32, ONE>(a, ev, eatom, block, s); break;
  }
}

// subdomain mode: the generic loops at 8 lanes per atom
template <bool ONE>
static void launch_ilp_ghost(const ForceArgs<R> &a, bool ev, bool eatom, int block, cudaStream_t s) {
  constexpr int TPA = 8;
  long long threads = (long long)a.n * TPA;
  int g = (int)((threads + block - 1) / block);
  if (a.kc) {
    if (ev && eatom) k_ilp<TPA, true, true, ONE, true, true, false><<<g, block, 0, s>>>(a);
    else if (ev) k_ilp<TPA, true, false, ONE, true, true, false><<<g, block, 0, s>>>(a);
    else k_ilp<TPA, false, false, ONE, true, true, false><<<g, block, 0, s>>>(a);
  } else if (ev && eatom) {
    k_ilp<TPA, true, true, ONE, true, false, false><<<g, block, 0, s>>>(a);
  } else if (ev) {
    k_ilp<TPA, true, false, ONE, true, false, false><<<g, block, 0, s>>>(a);
  } else {
    k_ilp<TPA, false, false, ONE, true, false, false><<<g, block, 0, s>>>(a);
  }
}

void launch_ilp(const ForceArgs<R> &a, bool ev, bool eatom, int tpa, int block, bool one_element, cudaStream_t s) {
  if (a.n == 0) return;
  if (a.own_perm) {
    if (one_element) launch_ilp_ghost<true>(a, ev, eatom, block, s);
    else launch_ilp_ghost<false>(a, ev, eatom, block, s);
    return;
  }
  if (one_element) launch_ilp_one<true>(a, ev, eatom, tpa, block, s);
  else launch_ilp_one<false>(a, ev, eatom, tpa, block, s);
}

void launch_nframe(const ForceArgs<R> &a, cudaStream_t s) {
  if (a.n == 0 || !a.nframe) return;
  const int b = per_atom_block(a.n);
  k_nframe<<<(a.n + b - 1) / b, b, 0, s>>>(a);
}

void launch_nderiv(const ForceArgs<R> &a, bool ev, cudaStream_t s) {
  if (a.n == 0) return;
  const int b = per_atom_block(a.n);
  const int g = (a.n + b - 1) / b;
  const bool p = (a.pdl & PDL_NDERIV) != 0;
  if (ev) launch_pdl(p, k_nderiv<true>, g, b, s, a);
  else launch_pdl(p, k_nderiv<false>, g, b, s, a);
}

void launch_finish(const ForceArgs<R> &a, bool eatom, const KickArgs *kick, cudaStream_t s) {
  if (a.n == 0) return;
  int g = (a.n + 127) / 128;
  KickArgs k{};
  if (kick) k = *kick;
  // early launch only behind the normal-derivative kernel (an evaluation without ILP, or
  // one that clears the Tersoff per-atom energies, puts a memset there)
  const bool p = (a.pdl & PDL_FINISH) && a.do_ilp && !(eatom && !a.do_ters);
  if (a.n <= FINISH_LANES_MAX_ATOMS && !a.no_small) {
    const int gl = (a.n + FINISH_ATOMS - 1) / FINISH_ATOMS, bl = FINISH_LANES * FINISH_ATOMS;
    if (kick && !eatom) launch_pdl(p, k_finish_lanes<false, true>, gl, bl, s, a, k);
    else if (kick) launch_pdl(p, k_finish_lanes<true, true>, gl, bl, s, a, k);
    else if (eatom) launch_pdl(p, k_finish_lanes<true, false>, gl, bl, s, a, k);
    else launch_pdl(p, k_finish_lanes<false, false>, gl, bl, s, a, k);
    return;
  }
  if (kick && !eatom) launch_pdl(p, k_finish<false, true>, g, 128, s, a, k);
  else if (kick) launch_pdl(p, k_finish<true, true>, g, 128, s, a, k);
  else if (eatom) launch_pdl(p, k_finish<true, false>, g, 128, s, a, k);
  else launch_pdl(p, k_finish<false, false>, g, 128, s, a, k);
}

#ifndef LMFF_PACKED_X2
// The per-atom virial pass on the lists and positions of the last evaluation: Tersoff's
// shares (the one-thread routine with VA; it also rewrites the force scratch arrays,
// which the evaluation has already gathered), the FP64 normal frames, ILP's shares, and
// the gather into out[6 n] (sorted order).  a.do_ters / a.do_ilp select the styles.
// ilp = false leaves the interlayer shares to the mixed pass (launch_vatom_ilp of the
// FP32 unit), which runs between this and launch_vatom_gather.
void launch_vatom_terms(const ForceArgs<R> &a, bool ilp, cudaStream_t s) {
  if (a.n == 0) return;
  const int g = (a.n + 127) / 128;
  const bool gh = a.own_perm != nullptr;
  if (a.do_ters) {
    if (gh) k_tersoff<false, false, true, true><<<g, 128, 0, s>>>(a);
    else k_tersoff<false, false, false, true><<<g, 128, 0, s>>>(a);
  }
  if (a.do_ilp && ilp) {
    k_nframe<<<g, 128, 0, s>>>(a);
    if (gh && a.kc) k_va_ilp<true, true><<<g, 128, 0, s>>>(a);
    else if (gh) k_va_ilp<true, false><<<g, 128, 0, s>>>(a);
    else if (a.kc) k_va_ilp<false, true><<<g, 128, 0, s>>>(a);
    else k_va_ilp<false, false><<<g, 128, 0, s>>>(a);
  }
}

void launch_vatom_gather(const ForceArgs<R> &a, double *out, cudaStream_t s) {
  if (a.n == 0) return;
  k_va_gather<<<(a.n + 127) / 128, 128, 0, s>>>(a, out);
}
#else
// The mixed engines' interlayer per-atom virial: the per-atom frame tensors, then the
// FP32 pass over the pair list.
void launch_vatom_ilp(const ForceArgs<R> &a, cudaStream_t s) {
  if (a.n == 0 || !a.do_ilp) return;
  const int g = (a.n + 127) / 128;
  const bool gh = a.own_perm != nullptr;
  k_va_tens<<<g, 128, 0, s>>>(a);
  if (gh && a.kc) k_va_ilp32<true, true><<<g, 128, 0, s>>>(a);
  else if (gh) k_va_ilp32<true, false><<<g, 128, 0, s>>>(a);
  else if (a.kc) k_va_ilp32<false, true><<<g, 128, 0, s>>>(a);
  else k_va_ilp32<false, false><<<g, 128, 0, s>>>(a);
}
#endif

}  // namespace LMFF_NS
}  // namespace lmff
