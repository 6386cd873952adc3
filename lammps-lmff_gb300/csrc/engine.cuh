// Internal declarations of the GB300 Tersoff + ILP engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "lmff_gb300.h"

namespace lmff {

// 32-byte aligned four-double vector: one 256-bit access per atom record
typedef double4_32a d4;
__host__ __device__ inline d4 make_d4(double x, double y, double z, double w) { return make_double4_32a(x, y, z, w); }

constexpr int MAXELEM = 4;     // elements per style held in constant memory (B, N, C, H)
constexpr int MAXTYPE = 16;    // LAMMPS atom types
constexpr int MAXILP = 3;      // intralayer neighbours per atom (pair_ilp_graphene_hbn.cpp:739)
constexpr int MAXTERS = 12;    // Tersoff short-list slots per atom
constexpr int MAXSHORT = 64;   // short candidates per atom (Tersoff + ILP intralayer, + skin)
constexpr int NSTAT = 8;       // reduction slots: e_vdw, e_rep | e_ters, then 6 virial

// status bits raised by kernels; the host maps them to LMFF_E* codes and messages
enum : int {
  ST_TOO_MANY_ILP = 1,
  ST_ZERO_NORMAL = 2,
  ST_TERS_OVERFLOW = 4,
  ST_SHORT_OVERFLOW = 8,
  ST_LIST_OVERFLOW = 16,
  ST_NONFINITE = 32,
  ST_STRIDE_OVERFLOW = 64,   // internal: an atom's list outgrew the strided build's stride
  ST_SKIN_TRIP = 128,        // internal: an atom moved more than skin/2 between rebuild checks
};

// ILP parameters of one ordered element pair (pair_ilp_graphene_hbn.h:53-57 after
// read_file scaling), with the constants the kernels need precomputed.
template <class R>
struct IlpP {
  R z0, lambda, eps_half, C, delta2inv, d, seff, C6;
  R d_over_seff;       // d / seff
  R lam_l2e, lamz0_l2e; // exp(-lambda (r - z0)) = exp2(lamz0_l2e - lam_l2e r)
  R nd2_l2e;           // exp(-rho^2 delta2inv) = exp2(nd2_l2e rho^2)
  R ts_a, ts_b;        // exp(-d (r/seff - 1)) = exp2(ts_b - ts_a r)
  int same_as_swapped; // params of (i,j) equal those of (j,i)
  int pad;
  // kolmogorov/crespi/full: f(rho) = exp(-x) (C0 + C2 x + C4 x^2), x = rho^2/delta^2,
  // vdW -A z0^6 / r^6; kc_off = -A (z0/cut)^6, the energy offset without the taper
  R kc_C0, kc_C2, kc_C4, kc_Az06, kc_off;
};

// Tersoff parameters of one element triplet (pair_tersoff.h:38-53) plus derived values.
template <class R>
struct TersP {
  R lam1, lam2, lam3, c2, d2, h, gamma, powern, beta, biga, bigb, bigr, bigd, cutsq;
  R c1, c2t, c3, c4;          // ters_bij branch thresholds (setup_params :569-572)
  R cd2;                      // c^2 / d^2
  R inv2n;                    // 1 / (2 n)
  R pi2_over_D;               // (pi/2) / D
  R pi4_over_D;               // (pi/4) / D
  R rlo, rhi;                 // R - D, R + D
  // FP64 copies of the radial constants: the bond's repulsion and attraction are
  // evaluated in FP64 in both precision modes
  double A64, B64, lam1_64, lam2_64, R64, D64, rlo64, rhi64, pi4D64, cutsq64;
  double nl1x32, nl2x32;       // -32 lam1, -32 lam2 (argument scale of the table exp)
  double h64;                 // h in FP64
  float hhi, hlo;             // h as an FP32 pair (FP32 mode: u = h - cos(theta) in double-float)
  double Al1_64, Bl2_64;      // A lam1, B lam2
  float nl1h, nl1l, nl2h, nl2l;  // -32 lam1, -32 lam2 as FP32 pairs (hi + lo)
  int powermint;
  int pad;
};

template <class R>
struct PotConst {
  int ntypes;
  int t_enabled, i_enabled;
  int t_ne, i_ne;
  int t_map[MAXTYPE + 1];
  int i_map[MAXTYPE + 1];
  int tap;
  int kc;                     // interlayer style is kolmogorov/crespi/full
  int vdw_sym;                // vdW constants symmetric in (i,j) for every pair
  int rep_sym;                // Tersoff repulsion constants of (i,j,j) equal those of (j,i,i)
  int ilp_cut_sym;            // intralayer cutoffs symmetric in the element pair: j in N_ilp(i) <=> i in N_ilp(j)
  unsigned ilp_typemask;      // bit t set when atom type t is mapped to an ILP element
  R t_cutmaxsq;
  R i_cutsq;                  // cut_global^2
  R i_inv_rcut;               // 1 / cut_global
  R i_cutILPsq[MAXELEM * MAXELEM];
  IlpP<R> ilp[MAXELEM * MAXELEM];
  TersP<R> ters[MAXELEM * MAXELEM * MAXELEM];
};

// Per-system geometry (one entry per independent system of a batch).
struct SysDesc {
  int atom_begin, atom_end;   // range in the sorted atom arrays
  int bin_begin;              // first global bin of this system
  int nb[3];                  // bins per dim
  int reach[3];               // stencil half-width in bins
  int per[3];
  double lo[3], L[3];         // box origin and lengths
  double binv[3];             // 1 / bin size
  double base;                // double-float offset (x - lo + 32 + base in [base, 2 base))
  float Lhi[3], Llo[3];       // L split into two floats
  float prefilt_sq;           // list build: a candidate whose hi-part distance squared
                              // exceeds this is beyond every cutoff (rounding margin in)
};

// list entry: neighbour index in the low IBITS, image code above (3 fields of W bits)
struct ListCode {
  int ibits, w, R;
  unsigned imask, wmask;
};

__host__ __device__ inline void decode_entry(uint32_t e, const ListCode &lc, int &j, int &sx, int &sy, int &sz) {
  j = (int)(e & lc.imask);
  uint32_t c = e >> lc.ibits;
  sx = (int)(c & lc.wmask) - lc.R;
  sy = (int)((c >> lc.w) & lc.wmask) - lc.R;
  sz = (int)((c >> (2 * lc.w)) & lc.wmask) - lc.R;
}

__host__ __device__ inline uint32_t encode_entry(int j, int sx, int sy, int sz, const ListCode &lc) {
  uint32_t c = (uint32_t)(sx + lc.R) | ((uint32_t)(sy + lc.R) << lc.w) | ((uint32_t)(sz + lc.R) << (2 * lc.w));
  return (uint32_t)j | (c << lc.ibits);
}

// Device buffers of the current system/batch in sorted order.
struct DevState {
  int n = 0;                  // atoms
  int nsys = 0;
  // positions and identity (sorted order)
  d4 *xq = nullptr;      // x, y, z, w = bits of (mol_dense << 8 | type)
  float4 *xh = nullptr;       // double-float hi parts, w = bits of int32 info
  float4 *xl = nullptr;       // lo parts
  double *v = nullptr;        // 3*n SoA (vx | vy | vz)
  double *f = nullptr;        // 3*n SoA
  double *xhold = nullptr;    // 3*n positions at the last build (AoS)
  int64_t *tag = nullptr;     // sorted tags
  int *perm = nullptr;        // sorted index -> input index
  int *sysid = nullptr;       // system of each atom
  double *mass = nullptr;     // per atom (sorted)
  // normals, per-step lists and gather slots
  d4 *nrm64 = nullptr;   // FP64 path normals
  float4 *nrm32 = nullptr;    // mixed path normals
  float4 *jrec = nullptr;     // 5 per atom: mixed pair kernel's j data, 3 (hi+info, lo, normal)
                              // for atom i at 3i, then the 2-float4 compact records from 3*cap
  int *ilp_cnt = nullptr;
  uint32_t *ilp_nb = nullptr; // n * MAXILP
  int *ters_cnt = nullptr;
  uint32_t *ters_nb = nullptr; // n * MAXTERS
  d4 *ters_g = nullptr;  // n * MAXTERS: force on slot atom from bonds centred here (+ bond energy)
  double *ters_f = nullptr;   // 3*n: Tersoff force on the centre atom
  double *ilp_f = nullptr;    // 3*n: ILP direct force (+ normal term on the atom itself)
  d4 *ilp_c = nullptr;   // n * MAXILP: normal-derivative force on each intralayer neighbour
  d4 *ilp_g = nullptr;   // n: dE/dn_i accumulated by the pair kernel
  d4 *nframe = nullptr;  // 4n: normal frames (k_nframe -> k_nderiv)
  double *eatom = nullptr;    // per-atom energy (when requested)
  double *ters_eatom = nullptr;
  // lists
  int64_t *list_off = nullptr; // n+1
  uint32_t *list = nullptr;
  int64_t list_cap = 0;
  // single-pass build: atom i's entries at list_tmp[i*stride ...] before the compaction
  uint32_t *list_tmp = nullptr;
  int64_t tmp_cap = 0;
  int *nin_tmp = nullptr;     // entries inside the force cutoff per atom
  uint8_t *list_img = nullptr;   // per atom: 1 when its pair list holds periodic-image entries
  int *short_cnt = nullptr;
  uint32_t *short_nb = nullptr; // n * MAXSHORT
  // binning
  uint32_t *bin_key = nullptr;
  uint32_t *bin_key2 = nullptr;
  int *idx = nullptr, *idx2 = nullptr;
  int *bin_start = nullptr, *bin_end = nullptr;
  int *rowocc = nullptr;       // per bin: 1 at the first bin of an occupied bin row
  int nbins = 0, nbins_cap = 0;
  void *cub_tmp = nullptr;
  size_t cub_tmp_bytes = 0;
  int64_t *cnt_tmp = nullptr; // n+1 per-atom pair-list counts (scanned into list_off)
  // systems
  SysDesc *sys = nullptr;
  // reductions
  double *partials = nullptr; // blocks * NSTAT * 2
  int partials_cap = 0;
  double *red_out = nullptr;  // NSTAT * 2 * nsys
  int *status = nullptr;      // device status word
  unsigned long long *maxdisp = nullptr;  // max squared displacement since build (as bits)
  int cap = 0;
};

}  // namespace lmff
