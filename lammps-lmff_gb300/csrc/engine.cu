// Engine orchestration and the C ABI (include/lmff_gb300.h).
//
// One engine = one device + one stream.  Atoms live on the device in bin-sorted order;
// perm maps sorted positions back to the caller's order.  A call runs, in order:
//   [rebuild when atoms moved > skin/2 since the last build, or identity/box changed]
//     k_wrap_bin -> radix sort by bin -> k_permute -> k_bin_ranges -> k_hilo
//     -> k_list (count + short lists) -> exclusive scan -> k_list (fill)
//   k_short (intralayer ILP list, Tersoff short list, normals)
//   k_tersoff (bonds centred at each atom)   k_ilp (interlayer pairs, normal derivatives)
//   k_finish (gather) -> [k_reduce energies/virials]
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <mutex>
#include <shared_mutex>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.cuh"
#include "forces.cuh"
#include "lmff_gb300.h"
#include "neighbor.cuh"
#include "potentials.h"

namespace lmff {

#define LMFF_FORCE_API(NS, R)                                                                              \
  namespace NS {                                                                                           \
  void upload_pot(const PotConst<R> &p, cudaStream_t s);                                                   \
  void launch_short(const ForceArgs<R> &a, const double *cutILPsq64, double tcutmaxsq64, cudaStream_t s); \
  void launch_tersoff(const ForceArgs<R> &a, bool ev, bool eatom, cudaStream_t s);                        \
  void launch_ilp(const ForceArgs<R> &a, bool ev, bool eatom, int tpa, int block, bool one_element,       \
                  cudaStream_t s);                                                                         \
  void launch_nframe(const ForceArgs<R> &a, cudaStream_t s);                                               \
  void launch_nderiv(const ForceArgs<R> &a, bool ev, cudaStream_t s);                                      \
  void launch_finish(const ForceArgs<R> &a, bool eatom, const KickArgs *kick, cudaStream_t s);             \
  }
LMFF_FORCE_API(f64, double)
LMFF_FORCE_API(f32, float)
namespace f64 {
void launch_vatom_terms(const ForceArgs<double> &a, bool ilp, cudaStream_t s);
void launch_vatom_gather(const ForceArgs<double> &a, double *out, cudaStream_t s);
}
namespace f32 {
void launch_vatom_ilp(const ForceArgs<float> &a, cudaStream_t s);
}

static const double LOG2E = 1.4426950408889634;
static const double FTM2V = 1.0 / 1.0364269e-4;  // units metal (update.cpp)
static const double MVV2E = 1.0364269e-4;
static const double BOLTZ = 8.617343e-5;

// ------------------------------------------------------------------ small kernels

__global__ void k_load(int n, const double *x, const int *type, const int64_t *mol, const int64_t *tag, const double *v,
                       const double *mass_t, const int *sysid_in, d4 *xq, int64_t *tag_s, int *perm, int *sysid,
                       double *vs, double *mass) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  long long info = ((long long)mol[p] << 8) | (long long)type[p];
  xq[p] = make_d4(x[3 * p], x[3 * p + 1], x[3 * p + 2], __longlong_as_double(info));
  tag_s[p] = tag ? tag[p] : (int64_t)(p + 1);
  perm[p] = p;
  sysid[p] = sysid_in ? sysid_in[p] : 0;
  vs[p] = v ? v[3 * p] : 0.0;
  vs[n + p] = v ? v[3 * p + 1] : 0.0;
  vs[2 * n + p] = v ? v[3 * p + 2] : 0.0;
  mass[p] = mass_t ? mass_t[type[p] - 1] : 1.0;
}

// per-atom tag (1-based within its system) and system id of a flattened batch, from the
// systems' atom offsets off[0..nsys]
__global__ void k_batch_ids(int n, const int *off, int nsys, int64_t *tag, int *sysid) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int lo = 0, hi = nsys;   // off[lo] <= q < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= q) lo = mid;
    else hi = mid;
  }
  tag[q] = (int64_t)(q - off[lo] + 1);
  sysid[q] = lo;
}

// identity check of the caller's arrays against the resident state
__global__ void k_check_ident(int n, const int *perm, const int *type, const int64_t *mol, const int64_t *tag,
                              const d4 *xq, const int64_t *tag_s, int *flag) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  long long info = ((long long)mol[o] << 8) | (long long)type[o];
  bool bad = info != __double_as_longlong(xq[q].w);
  if (tag && tag[o] != tag_s[q]) bad = true;
  if (bad) atomicOr(flag, 1);
}

// Largest squared displacement of the block into *maxdisp (non-negative doubles order as
// their bit patterns): one atomic per block on the shared word, not one per warp.  Every
// thread of the block calls it.
__device__ __forceinline__ void block_max_disp(double d2, unsigned long long *maxdisp) {
  for (int o = 16; o > 0; o >>= 1) d2 = fmax(d2, __shfl_xor_sync(0xffffffff, d2, o));
  __shared__ double wmax[32];
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = d2;
  __syncthreads();
  if (threadIdx.x < 32) {
    d2 = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) d2 = fmax(d2, __shfl_xor_sync(0xffffffff, d2, o));
    if (threadIdx.x == 0 && d2 > 0.0) atomicMax(maxdisp, (unsigned long long)__double_as_longlong(d2));
  }
}

// new caller positions into sorted order + max squared displacement since the build
// New caller positions into the resident state.  On periodic dimensions a position is
// taken in the periodic image nearest the one the list was built with (the caller may
// hand unwrapped coordinates, or coordinates it just wrapped): the list's image codes
// stay valid and an atom that crossed the box edge is not a displacement.
__global__ void k_update_x(int n, const int *perm, const double *x, d4 *xq, const double *xhold,
                           unsigned long long *maxdisp, const SysDesc *sys, const int *sysid) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  double d2 = 0.0;
  if (q < n) {
    int o = perm[q];
    d4 w = xq[q];
    double a = x[3 * o], b = x[3 * o + 1], c = x[3 * o + 2];
    const SysDesc &sd = sys[sysid[q]];
    if (sd.per[0]) a -= sd.L[0] * rint((a - xhold[3 * q]) / sd.L[0]);
    if (sd.per[1]) b -= sd.L[1] * rint((b - xhold[3 * q + 1]) / sd.L[1]);
    if (sd.per[2]) c -= sd.L[2] * rint((c - xhold[3 * q + 2]) / sd.L[2]);
    xq[q] = make_d4(a, b, c, w.w);
    double dx = a - xhold[3 * q], dy = b - xhold[3 * q + 1], dz = c - xhold[3 * q + 2];
    d2 = dx * dx + dy * dy + dz * dz;
  }
  block_max_disp(d2, maxdisp);
}

__global__ void k_scatter_add(int n, const int *perm, const double *fs, double *fin, int overwrite) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  for (int c = 0; c < 3; c++) {
    double v = fs[(size_t)c * n + q];
    fin[3 * o + c] = overwrite ? v : fin[3 * o + c] + v;
  }
}

// fout = fin + fs in the caller's order (fout = fs without fin): k_scatter_add's sums into
// a separate output, so that fin stays the caller's input
__global__ void k_scatter_sum(int n, const int *perm, const double *fs, const double *fin, double *fout) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  for (int c = 0; c < 3; c++) {
    double v = fs[(size_t)c * n + q];
    fout[3 * o + c] = fin ? fin[3 * o + c] + v : v;
  }
}

// per-atom rows of 6 (the per-atom virial), sorted order -> the caller's
__global__ void k_scatter_add6(int n, const int *perm, const double *vs, double *vin, int overwrite) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  for (int c = 0; c < 6; c++) {
    double v = vs[6 * (size_t)q + c];
    vin[6 * (size_t)o + c] = overwrite ? v : vin[6 * (size_t)o + c] + v;
  }
}

__global__ void k_scatter_add1(int n, const int *perm, const double *es, double *ein, int overwrite) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  ein[o] = overwrite ? es[q] : ein[o] + es[q];
}

__global__ void k_unpermute_state(int n, const int *perm, const d4 *xq, const double *v, const double *f, double *xo,
                                  double *vo, double *fo) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  d4 w = xq[q];
  xo[3 * o] = w.x; xo[3 * o + 1] = w.y; xo[3 * o + 2] = w.z;
  for (int c = 0; c < 3; c++) {
    vo[3 * o + c] = v[(size_t)c * n + q];
    fo[3 * o + c] = f[(size_t)c * n + q];
  }
}

// deterministic per-system reduction of the per-atom stat arrays: block (s, q) sums
// quantity q of system s in a fixed order
__global__ void k_reduce(int n, int nq, const double *const *arrs, const SysDesc *sys, double *out) {
  int s = blockIdx.x / nq, q = blockIdx.x % nq;
  const double *a = arrs[q / 8] + (size_t)(q % 8) * n;
  int b = sys[s].atom_begin, e = sys[s].atom_end;
  double acc = 0.0;
  for (int p = b + threadIdx.x; p < e; p += blockDim.x) acc += a[p];
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// interlayer pairs of the list within the ILP cutoff (same test as the pair kernel)
__global__ void k_count_pairs(int n, const d4 *xq, const SysDesc *sys, const int *sysid, const int64_t *off,
                              const uint32_t *list, ListCode lc, double cutsq, unsigned long long *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (i < n) {
    const SysDesc &sd = sys[sysid[i]];
    d4 a = xq[i];
    long long mi = __double_as_longlong(a.w) >> 8;
    for (int64_t k = off[i]; k < off[i + 1]; k++) {
      int j, sx, sy, sz;
      decode_entry(list[k], lc, j, sx, sy, sz);
      d4 b = xq[j];
      if ((__double_as_longlong(b.w) >> 8) == mi) continue;
      double dx = a.x - (b.x + sx * sd.L[0]), dy = a.y - (b.y + sy * sd.L[1]), dz = a.z - (b.z + sz * sd.L[2]);
      if (dx * dx + dy * dy + dz * dz < cutsq) c++;
    }
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffff, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// dtf / mass per atom type, computed on the host: the same FP64 quotient fix_nve.cpp
// forms per atom (dtfm = dtf / mass[type[i]], :64-84), without a division per atom (FP64
// division is a long sequence on a GPU whose FP64 rate is 1/64 of FP32)
struct DtfmTab {
  double v[MAXTYPE + 1];
};

// The rebuild test of a step when the list is checked only every k-th step (small
// systems, where a step costs a few tens of microseconds and the test's conditional graph
// node a sizeable part of it).  A check step looks ahead: it rebuilds when any atom may
// move more than skin/2 from its position at the last build before the next check,
// taking the reach as d + hv |v| + ha dtfm |f| (d: displacement so far; the velocity and
// acceleration terms of k-1 steps with a 25 % margin) into *pred.  A step between checks
// raises ST_SKIN_TRIP into *status when an atom did move more than skin/2 (the list may
// then miss a pair: the host redoes the chunk with a test at every step of it).
struct Lookahead {
  unsigned long long *pred;
  double hv, ha;
  int *status;
  double trig2;
};

// velocity Verlet halves (fix_nve.cpp:64-111); the first also moves x, refreshes the
// double-float split and tracks the displacement since the last build
__global__ void k_nve1(int n, d4 *xq, double *v, const double *f, DtfmTab tab, double dtv,
                       const double *xhold, unsigned long long *maxdisp, const SysDesc *sys, const int *sysid,
                       float4 *xh, float4 *xl, int do_hilo, cudaGraphConditionalHandle h = 0, double trig2 = 0.0,
                       unsigned *ticket = nullptr, Lookahead la = Lookahead{}) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  double d2 = 0.0, p2 = 0.0;
  if (q < n) {
    d4 w = xq[q];
    double dtfm = tab.v[__double_as_longlong(w.w) & 255];
    const double fx = f[q], fy = f[n + q], fz = f[2 * n + q];
    double vx = v[q] + dtfm * fx;
    double vy = v[n + q] + dtfm * fy;
    double vz = v[2 * n + q] + dtfm * fz;
    v[q] = vx; v[n + q] = vy; v[2 * n + q] = vz;
    d2 = nve_drift(q, vx, vy, vz, dtv, xq, xhold, xh, xl, sys, sysid, do_hilo);
    if (la.pred) {
      const double p = sqrt(d2) + la.hv * sqrt(vx * vx + vy * vy + vz * vz) +
                       la.ha * fabs(dtfm) * sqrt(fx * fx + fy * fy + fz * fz);
      p2 = p * p;
    }
    if (la.status && d2 > la.trig2) atomicOr(la.status, ST_SKIN_TRIP);
  }
  block_max_disp(d2, maxdisp);
  if (la.pred) {
    __syncthreads();   // block_max_disp's shared words are reused
    block_max_disp(p2, la.pred);
  }
  if (ticket) {
    // in the step graph: the last block to finish sets the rebuild condition, any atom
    // moved more than skin/2 since the last build (neighbor.cpp:1947-1976 check_distance),
    // or may before the next check
    __shared__ bool last;
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
      *ticket = 0;
      double dmax = __longlong_as_double((long long)atomicMax(maxdisp, 0ull));
      if (la.pred) dmax = fmax(dmax, __longlong_as_double((long long)atomicExch(la.pred, 0ull)));
      cudaGraphSetConditional(h, dmax > trig2 ? 1u : 0u);
    }
  }
}

__global__ void k_nve2(int n, double *v, const double *f, const d4 *xq, const double *mass, DtfmTab tab, double *ke) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const long long info = *reinterpret_cast<const long long *>(&xq[q].w);
  double dtfm = tab.v[info & 255];
  double vx = v[q] + dtfm * f[q];
  double vy = v[n + q] + dtfm * f[n + q];
  double vz = v[2 * n + q] + dtfm * f[2 * n + q];
  v[q] = vx; v[n + q] = vy; v[2 * n + q] = vz;
  if (ke) ke[q] = 0.5 * MVV2E * mass[q] * (vx * vx + vy * vy + vz * vz);
}

// largest |v| and dtfm |f| over the atoms (squared, into out[0], out[1]): the motion
// bound the look-ahead rebuild test sizes its check interval with
__global__ void k_motion_max(int n, const double *v, const double *f, const d4 *xq, DtfmTab tab,
                             unsigned long long *out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  double v2 = 0.0, a2 = 0.0;
  if (q < n) {
    const double dtfm = tab.v[__double_as_longlong(xq[q].w) & 255];
    v2 = v[q] * v[q] + v[n + q] * v[n + q] + v[2 * n + q] * v[2 * n + q];
    a2 = dtfm * dtfm * (f[q] * f[q] + f[n + q] * f[n + q] + f[2 * n + q] * f[2 * n + q]);
  }
  block_max_disp(v2, out);
  __syncthreads();
  block_max_disp(a2, out + 1);
}

// ---------------------------------------------------------------- minimiser kernels
// Conjugate-gradient vectors live in the caller's atom order (index o = perm[q]), so
// list rebuilds, which re-sort the resident atoms, leave them in place.  SoA: [c*n + o].

// fix setforce 0 0 0 on the atoms whose mask is 0 (fix_setforce.cpp min_post_force)
__global__ void k_min_mask(int n, const int *perm, const int *mask, double *f) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n || mask[perm[q]]) return;
  f[q] = 0.0;
  f[n + q] = 0.0;
  f[2 * n + q] = 0.0;
}

// mode 0: h = g = f; 1: g = f, h = g + beta h; 2: h = g; 3: x0 = x
__global__ void k_min_vec(int mode, int n, const int *perm, const double *f, const d4 *xq, double *g, double *h,
                          double *x0, double beta) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  if (mode == 3) {
    d4 w = xq[q];
    x0[o] = w.x;
    x0[n + o] = w.y;
    x0[2 * n + o] = w.z;
    return;
  }
  for (int c = 0; c < 3; c++) {
    size_t k = (size_t)c * n + o;
    if (mode == 0) {
      double v = f[(size_t)c * n + q];
      g[k] = v;
      h[k] = v;
    } else if (mode == 1) {
      double v = f[(size_t)c * n + q];
      g[k] = v;
      h[k] = v + beta * h[k];
    } else {
      h[k] = g[k];
    }
  }
}

// per-block partials of f.f, f.g, f.h, g.h (sums) and max|h|, max|f| (per component)
constexpr int MIN_NQ = 6;
__global__ void k_min_dots(int n, const int *perm, const double *f, const double *g, const double *h,
                           double *part) {
  double acc[MIN_NQ] = {0, 0, 0, 0, 0, 0};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int o = perm[q];
    for (int c = 0; c < 3; c++) {
      double fv = f[(size_t)c * n + q], gv = g[(size_t)c * n + o], hv = h[(size_t)c * n + o];
      acc[0] += fv * fv;
      acc[1] += fv * gv;
      acc[2] += fv * hv;
      acc[3] += gv * hv;
      acc[4] = fmax(acc[4], fabs(hv));
      acc[5] = fmax(acc[5], fabs(fv));
    }
  }
  __shared__ double sh[MIN_NQ][256];
  for (int k = 0; k < MIN_NQ; k++) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < MIN_NQ; k++)
        sh[k][threadIdx.x] = k < 4 ? sh[k][threadIdx.x] + sh[k][threadIdx.x + s]
                                   : fmax(sh[k][threadIdx.x], sh[k][threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x < MIN_NQ) part[blockIdx.x * MIN_NQ + threadIdx.x] = sh[threadIdx.x][0];
}

// x = x0 + alpha h (min_linesearch.cpp alpha_step), with the displacement since the
// last build for the rebuild test
__global__ void k_min_step(int n, const int *perm, const double *x0, const double *h, double alpha, d4 *xq,
                           const double *xhold, unsigned long long *maxdisp) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  double d2 = 0.0;
  if (q < n) {
    int o = perm[q];
    d4 w = xq[q];
    double a = x0[o], b = x0[n + o], c = x0[2 * n + o];
    if (alpha > 0.0) {
      a += alpha * h[o];
      b += alpha * h[n + o];
      c += alpha * h[2 * n + o];
    }
    xq[q] = make_d4(a, b, c, w.w);
    double dx = a - xhold[3 * q], dy = b - xhold[3 * q + 1], dz = c - xhold[3 * q + 2];
    d2 = dx * dx + dy * dy + dz * dz;
  }
  block_max_disp(d2, maxdisp);
}

// after a rebuild wrapped atoms into the box: x0 = x + minimum_image(x0 - x)
// (fix_minimize.cpp reset_coords with domain.cpp minimum_image)
__global__ void k_min_reset(int n, const int *perm, const d4 *xq, const SysDesc *sys, const int *sysid, double *x0) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = perm[q];
  const SysDesc &sd = sys[sysid[q]];
  d4 w = xq[q];
  double x[3] = {w.x, w.y, w.z};
  for (int c = 0; c < 3; c++) {
    double d = x0[(size_t)c * n + o] - x[c];
    if (sd.per[c] && fabs(d) > 0.5 * sd.L[c]) d += d < 0.0 ? sd.L[c] : -sd.L[c];
    x0[(size_t)c * n + o] = x[c] + d;
  }
}

// Pair-list offsets past the capacity the step graph was captured with: clamp them so
// that fill and the force kernels stay inside the array, and flag the overflow (the
// host then redoes the chunk on the eager path, which grows the list).
__global__ void k_clamp_off(int n, int64_t *off, int64_t cap, int *status, unsigned long long *rebuilds) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == 0) atomicAdd(rebuilds, 1ull);
  int64_t o = off[i];
  if (o > cap) {
    off[i] = cap;
    atomicOr(status, ST_LIST_OVERFLOW);
  }
}

// ------------------------------------------------------------------ engine

// The potential tables live in __constant__ memory, one copy per device and module,
// shared by every engine of the process.  Each device records the content hash of the
// tables it holds.  Every device-touching API call holds the device's lock in shared
// mode for its whole duration (all calls finish their GPU work before returning);
// an engine whose tables differ from the device's takes the lock exclusively, waits for
// the device to drain and uploads.  Engines with identical tables (e.g. serving slots)
// therefore run concurrently on their own streams; engines with different tables (the
// two LAMMPS sub-styles) alternate safely.
static std::shared_mutex g_dev_rw[64];
static uint64_t g_dev_tables[64] = {0};

template <class T>
static cudaError_t dalloc(T *&p, size_t count) {
  if (p) cudaFree(p);
  p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)&p, count * sizeof(T));
}

// Binning and double-float geometry of one orthogonal box (lo, L, periodicity): bins
// of at least (cutneigh/2)*1.0001 so that any pair within cutneigh is at most `reach`
// bins apart whatever the rounding of the bin index; R = periodic images needed.
static void sys_geometry(SysDesc &sd, const double lo[3], const double L[3], const int per[3], double cutneigh_max,
                         int &R) {
  double target = 0.5 * cutneigh_max * 1.0001, maxL = 0.0;
  for (int k = 0; k < 3; k++) {
    sd.lo[k] = lo[k];
    sd.L[k] = L[k];
    sd.per[k] = per[k] != 0;
    int nb = std::max(1, (int)std::floor(sd.L[k] / target));
    if (nb > 4096) nb = 4096;
    double bs = sd.L[k] / nb;
    sd.nb[k] = nb;
    sd.binv[k] = 1.0 / bs;
    sd.reach[k] = (int)std::ceil(cutneigh_max / bs * (1.0 + 1e-12));
    // images needed: |s| <= ceil(reach / nb) for a stencil of +-reach bins
    if (sd.per[k]) R = std::max(R, (sd.reach[k] + nb - 1) / nb);
    sd.Lhi[k] = (float)sd.L[k];
    sd.Llo[k] = (float)(sd.L[k] - (double)sd.Lhi[k]);
    maxL = std::max(maxL, sd.L[k]);
  }
  sd.base = std::ldexp(1.0, (int)std::ceil(std::log2(maxL + 64.0)));
  // hi parts alone differ from the displacement by the lo parts, the lo part of the
  // image shift and one rounding: a few ulp of 2*base per component
  double e = 4.0 * std::ldexp(2.0 * sd.base, -23);
  double r = cutneigh_max + 2.0 * e;
  sd.prefilt_sq = (float)(r * r * (1.0 + 1e-5));
}

struct Engine {
  uint64_t table_hash = 0;  // content hash of the constant tables (pot64, pot32, nbc, cutILPsq)
  int device = 0;
  cudaStream_t stream = nullptr;
  int precision = LMFF_FP64;
  int tpa = 16, block = 128;
  int list_full = 0;
  // subdomain mode (lmff_compute_ghost): the number of owned atoms among the caller's
  // nall (owned first, then ghosts); -1 for the ordinary periodic-system mode
  int ghost_nlocal = -1;
  int pair_tile = 2;   // option "pair_tile": list entries per pair-loop iteration (1 or 2)
  bool small_variants = true;   // option "small_variants": the small-system kernel variants
  // option "pdl": a PDL_* mask of the step's chain kernels launched with programmatic
  // dependent launch, for systems of at most PDL_MAX_ATOMS atoms; pdl_short: the capture
  // of a step graph sets it for the steps after the first, whose intralayer-list kernel
  // follows the previous step's gather.  Default: the normal-derivative kernel, the
  // gather and the intralayer lists, dependents scheduled as blocks exit (7,200-atom
  // bilayer, step graphs: 38.2 -> 37.4 us per step).  The pair kernel is left out: launched
  // early its blocks fill the SMs before Tersoff and the normal frames, which start
  // beside it on other streams (45 us per step), and so is the early trigger (+0.8 us).
  static constexpr int PDL_MAX_ATOMS = 65536;
  int pdl_mask = PDL_NDERIV | PDL_FINISH | PDL_SHORT;
  bool pdl_short = false;
  double skin = 2.0;
  int ntypes = 0;
  HostTersoff ht;
  HostIlp hi;
  bool t_on = false, i_on = false;
  bool i_one = false;  // ILP maps every type to one element
  double cut_global = 16.0;
  int tap = 1;
  PotConst<double> pot64;
  PotConst<float> pot32;
  NbConst nbc;
  double *d_cutILPsq = nullptr;
  double rshort = 0.0, cutneigh_max = 0.0;
  bool pot_dirty = true;
  // geometry
  double blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};
  int bper[3] = {0, 0, 0};
  bool have_box = false;
  // triclinic box (lmff_set_box with a tilt): lmff_compute evaluates the owned atoms and
  // their periodic images, made on the host, through the subdomain form; tri_owner[a] is
  // the owned atom of each of the last call's atoms (owned first, then images)
  bool tri = false;
  double tlo[3] = {0, 0, 0}, thi[3] = {0, 0, 0}, tilt[3] = {0, 0, 0};   // tilt: xy xz yz
  int tper[3] = {0, 0, 0};
  std::vector<int> tri_owner;
  int tri_n = -1;
  // state
  DevState d;
  std::vector<SysDesc> hsys;
  ListCode lc{};
  bool loaded = false, built = false, forces_valid = false;
  int n = 0;
  // staging (caller order)
  double *d_xin = nullptr, *d_fin = nullptr, *d_vin = nullptr, *d_ein = nullptr;
  double *d_fo = nullptr;   // lmff_compute's force output, d_fin keeping the caller's input
  // pinned words the device writes back without a host wait: [0] status, [1] largest
  // squared displacement since the build
  unsigned long long *h_words = nullptr;
  cudaEvent_t pend_e0 = nullptr, pend_e1 = nullptr;   // a force evaluation not waited for
  int *d_tin = nullptr, *d_sysin = nullptr;
  int64_t *d_min = nullptr, *d_gin = nullptr;
  double *d_massT = nullptr;
  // spares for permutation
  d4 *xq2 = nullptr;
  double *v2 = nullptr, *mass2 = nullptr;
  int64_t *tag2 = nullptr;
  int *perm2 = nullptr, *sysid2 = nullptr;
  double *stat_ilp = nullptr, *stat_ters = nullptr, *eatom_ilp = nullptr, *eatom_ters = nullptr, *ke = nullptr;
  double **d_arrs = nullptr;
  double **d_karrs = nullptr;
  double *d_kout = nullptr;
  // per-atom virial pass (lmff_compute_vatom): own shares, slots, the sorted result, the
  // result in the caller's order and the mixed pass's frame tensors (7 float4), VA_DOUBLES
  // per atom of capacity va_cap
  static constexpr int VA_DOUBLES = 6 * (2 + MAXTERS + MAXILP + 2) + 14;
  double *d_va = nullptr;
  int va_cap = 0;
  // device calls on this engine (counted by DeviceCall) and the one whose evaluation
  // lmff_compute_vatom may still use
  uint64_t calls = 0, va_call = 0;
  // single-pass list build: stride of the scratch slices (0: two passes), only grown, so
  // that a captured rebuild keeps working; largest per-atom count of the last build
  int stride = 0;
  int *d_maxcnt = nullptr;
  cudaStream_t stream2 = nullptr;   // Tersoff beside the pair kernel
  cudaStream_t stream3 = nullptr;   // the normal frames beside both
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_frame = nullptr;
  bool ters_concurrent = true;      // option "ters_concurrent"
  double *h_pinned = nullptr;   // batch staging (lmff_batch_set)
  size_t h_pinned_bytes = 0;
  int *d_boff = nullptr;        // batch system offsets on the device
  int boff_cap = 0;
  std::vector<double> mass_type;
  // per-system energies and virials of the last evaluation that computed them
  std::vector<lmff_result> last_res;
  bool last_res_valid = false;
  // stats
  int64_t rebuilds = 0, steps = 0, list_total = 0, short_total = 0;
  double ms_build = 0, ms_forces = 0, ms_run = 0;
  int64_t pairs_in_cut = 0;
  // per-kernel device timing (option "kernel_timing"): events around each launch
  bool ktiming = false;
  double kms[7] = {0, 0, 0, 0, 0, 0, 0};
  int64_t klaunch[7] = {0, 0, 0, 0, 0, 0, 0};
  struct Pend {
    cudaEvent_t a, b;
    int k;
  };
  std::vector<Pend> pend;
  std::vector<cudaEvent_t> evpool;
  cudaEvent_t ev_get() {
    if (evpool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = evpool.back();
    evpool.pop_back();
    return e;
  }
  template <class F>
  void timed(int k, F &&f) {
    if (!ktiming) {
      f();
      return;
    }
    Pend p{ev_get(), ev_get(), k};
    cudaEventRecord(p.a, stream);
    f();
    cudaEventRecord(p.b, stream);
    pend.push_back(p);
  }
  // after a stream synchronisation: fold finished events into the per-kernel sums
  void harvest() {
    for (auto &p : pend) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
        kms[p.k] += ms;
        klaunch[p.k]++;
      }
      evpool.push_back(p.a);
      evpool.push_back(p.b);
    }
    pend.clear();
  }
  std::string err;
  int64_t nbit_bins = 1;

  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char *where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return LMFF_ECUDA;
  }
#define CK2(expr)                                                  \
  do {                                                             \
    cudaError_t _e = (expr);                                       \
    if (_e != cudaSuccess) return g.cuda_fail(_e, #expr);          \
  } while (0)
#define CK(expr)                                    \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
  } while (0)

  ~Engine() { release(); }

  void release() {
    if (device >= 0) cudaSetDevice(device);
    void *ptrs[] = {d.xq, d.xh, d.xl, d.v, d.f, d.xhold, d.tag, d.perm, d.sysid, d.mass, d.nrm64, d.nrm32, d.jrec, d.ilp_cnt,
                    d.ilp_nb, d.ters_cnt, d.ters_nb, d.ters_g, d.ters_f, d.ilp_f, d.ilp_c, d.ilp_g, d.nframe, d.list_off, d.list,
                    d.short_cnt, d.short_nb, d.list_img, d.nin_tmp, d.list_tmp, d.bin_key, d.bin_key2, d.idx, d.idx2, d.bin_start, d.bin_end, d.rowocc, d.cub_tmp,
                    d.cnt_tmp, d.sys, d.red_out, d.status, d.maxdisp, d_xin, d_fin, d_fo, d_vin, d_ein, d_tin, d_sysin,
                    d_min, d_gin, d_massT, xq2, v2, mass2, tag2, perm2, sysid2, stat_ilp, stat_ters, eatom_ilp,
                    eatom_ters, ke, d_arrs, d_karrs, d_kout, d_cutILPsq, d_maxpred, d_va};
    for (void *p : ptrs)
      if (p) cudaFree(p);
    d = DevState();
    d_xin = d_fin = d_fo = d_vin = d_ein = nullptr;
    if (h_words) cudaFreeHost(h_words);
    h_words = nullptr;
    d_tin = d_sysin = nullptr;
    d_min = d_gin = nullptr;
    d_massT = nullptr;
    xq2 = nullptr;
    v2 = mass2 = nullptr;
    tag2 = nullptr;
    perm2 = sysid2 = nullptr;
    stat_ilp = stat_ters = eatom_ilp = eatom_ters = ke = nullptr;
    d_arrs = nullptr;
    d_karrs = nullptr;
    d_kout = nullptr;
    d_cutILPsq = nullptr;
    d_maxpred = nullptr;
    d_va = nullptr;
    va_cap = 0;
    if (h_pinned) cudaFreeHost(h_pinned);
    h_pinned = nullptr;
    h_pinned_bytes = 0;
    if (d_boff) cudaFree(d_boff);
    d_boff = nullptr;
    boff_cap = 0;
    if (d_maxcnt) cudaFree(d_maxcnt);
    d_maxcnt = nullptr;
    stride = 0;
    drop_graph();
    void *bks[] = {bk_xq, bk_v, bk_f, bk_mass, bk_tag, bk_perm, bk_sysid};
    for (void *b : bks)
      if (b) cudaFree(b);
    bk_xq = nullptr;
    bk_v = bk_f = bk_mass = nullptr;
    bk_tag = nullptr;
    bk_perm = bk_sysid = nullptr;
    bk_cap = 0;
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cap_stream = nullptr;
    if (d_graph_rebuilds) cudaFree(d_graph_rebuilds);
    d_graph_rebuilds = nullptr;
    if (d_cond_ticket) cudaFree(d_cond_ticket);
    d_cond_ticket = nullptr;
    void *mins[] = {m_x0, m_g, m_h, m_part, m_mask};
    for (void *b : mins)
      if (b) cudaFree(b);
    m_x0 = m_g = m_h = m_part = nullptr;
    m_mask = nullptr;
    m_cap = 0;
    if (stream2) cudaStreamDestroy(stream2);
    stream2 = nullptr;
    if (stream3) cudaStreamDestroy(stream3);
    stream3 = nullptr;
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_frame) cudaEventDestroy(ev_frame);
    ev_fork = ev_join = ev_frame = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }

  // ---------------------------------------------------------------- parameters
  int set_params(const lmff_params *p) {
    if (!p || p->ntypes < 1 || p->ntypes > MAXTYPE) return fail(LMFF_EINVAL, "ntypes must be in 1..16");
    ntypes = p->ntypes;
    t_on = p->tersoff_nparams > 0;
    i_on = p->ilp_nparams > 0;
    if (!t_on && !i_on) return fail(LMFF_EINVAL, "neither tersoff nor ilp/graphene/hbn parameters given");
    ht = HostTersoff();
    hi = HostIlp();
    if (t_on) {
      int ne = p->tersoff_nelements;
      if (ne < 1 || ne > MAXELEM) return fail(LMFF_EUNSUPPORTED, "tersoff: at most 4 elements are supported");
      ht.params.assign(p->tersoff_params, p->tersoff_params + p->tersoff_nparams);
      ht.elem2param.assign(p->tersoff_elem2param, p->tersoff_elem2param + ne * ne * ne);
      ht.map.assign(p->tersoff_map, p->tersoff_map + ntypes + 1);
      ht.elements.resize(ne);
      ht.cutmax = p->tersoff_cutmax;
    }
    if (i_on) {
      int ne = p->ilp_nelements;
      if (ne < 1 || ne > MAXELEM) return fail(LMFF_EUNSUPPORTED, "ilp: at most 4 elements are supported");
      if (p->interlayer_model == LMFF_INTERLAYER_KC) {
        if (!p->kc_params) return fail(LMFF_EINVAL, "kolmogorov/crespi/full: kc_params missing");
        hi.model = LMFF_INTERLAYER_KC;
        hi.kc.assign(p->kc_params, p->kc_params + p->ilp_nparams);
      } else {
        if (!p->ilp_params) return fail(LMFF_EINVAL, "ilp/graphene/hbn: ilp_params missing");
        hi.params.assign(p->ilp_params, p->ilp_params + p->ilp_nparams);
      }
      hi.elem2param.assign(p->ilp_elem2param, p->ilp_elem2param + ne * ne);
      hi.map.assign(p->ilp_map, p->ilp_map + ntypes + 1);
      hi.cutILPsq.assign(p->ilp_cutILPsq, p->ilp_cutILPsq + ne * ne);
      hi.elements.resize(ne);
    }
    i_one = i_on && p->ilp_nelements == 1;
    cut_global = p->ilp_cut_global;
    tap = p->ilp_tap_flag;
    skin = p->skin;
    return build_consts();
  }

  template <class R>
  void fill_pot(PotConst<R> &P) {
    memset(&P, 0, sizeof P);
    P.ntypes = ntypes;
    P.t_enabled = t_on;
    P.i_enabled = i_on;
    P.t_ne = t_on ? (int)ht.elements.size() : 0;
    P.i_ne = i_on ? (int)hi.elements.size() : 0;
    for (int t = 0; t <= MAXTYPE; t++) {
      P.t_map[t] = (t_on && t >= 1 && t <= ntypes) ? ht.map[t] : -1;
      P.i_map[t] = (i_on && t >= 1 && t <= ntypes) ? hi.map[t] : -1;
    }
    P.tap = tap;
    P.kc = i_on && hi.model == LMFF_INTERLAYER_KC;
    P.ilp_typemask = 0;
    for (int t = 1; t <= ntypes && t < 32; t++)
      if (P.i_map[t] >= 0) P.ilp_typemask |= 1u << t;
    P.vdw_sym = 1;
    P.rep_sym = 1;
    P.ilp_cut_sym = 1;
    P.t_cutmaxsq = (R)(ht.cutmax * ht.cutmax);
    P.i_cutsq = (R)(cut_global * cut_global);
    P.i_inv_rcut = (R)(1.0 / cut_global);
    if (i_on) {
      int ne = P.i_ne;
      for (int a = 0; a < ne; a++)
        for (int b = 0; b < ne; b++) {
          if (P.kc) {
            const lmff_kc_param &q = hi.kc[hi.elem2param[a * ne + b]];
            const lmff_kc_param &s = hi.kc[hi.elem2param[b * ne + a]];
            IlpP<R> &o = P.ilp[a * MAXELEM + b];
            o.z0 = (R)q.z0;
            o.lambda = (R)q.lambda;
            o.eps_half = (R)(0.5 * q.C);
            o.C = (R)q.C;
            o.delta2inv = (R)q.delta2inv;
            o.lam_l2e = (R)(q.lambda * LOG2E);
            o.lamz0_l2e = (R)(q.lambda * q.z0 * LOG2E);
            o.nd2_l2e = (R)(-q.delta2inv * LOG2E);
            o.kc_C0 = (R)q.C0;
            o.kc_C2 = (R)q.C2;
            o.kc_C4 = (R)q.C4;
            o.kc_Az06 = (R)(q.A * q.z06);
            o.kc_off = (R)(-q.A * std::pow(q.z0 / cut_global, 6.0));
            o.same_as_swapped = (q.z0 == s.z0 && q.lambda == s.lambda && q.C == s.C && q.delta2inv == s.delta2inv &&
                                 q.C0 == s.C0 && q.C2 == s.C2 && q.C4 == s.C4);
            if (!(q.A * q.z06 == s.A * s.z06)) P.vdw_sym = 0;
            P.i_cutILPsq[a * MAXELEM + b] = (R)hi.cutILPsq[a * ne + b];
            continue;
          }
          const lmff_ilp_param &q = hi.params[hi.elem2param[a * ne + b]];
          const lmff_ilp_param &s = hi.params[hi.elem2param[b * ne + a]];
          IlpP<R> &o = P.ilp[a * MAXELEM + b];
          o.z0 = (R)q.z0;
          o.lambda = (R)q.lambda;
          o.eps_half = (R)(0.5 * q.epsilon);
          o.C = (R)q.C;
          o.delta2inv = (R)q.delta2inv;
          o.d = (R)q.d;
          o.seff = (R)q.seff;
          o.C6 = (R)q.C6;
          o.d_over_seff = (R)(q.d / q.seff);
          o.lam_l2e = (R)(q.lambda * LOG2E);
          o.lamz0_l2e = (R)(q.lambda * q.z0 * LOG2E);
          o.nd2_l2e = (R)(-q.delta2inv * LOG2E);
          o.ts_a = (R)(q.d / q.seff * LOG2E);
          o.ts_b = (R)(q.d * LOG2E);
          o.same_as_swapped = (q.z0 == s.z0 && q.lambda == s.lambda && q.epsilon == s.epsilon && q.C == s.C &&
                               q.delta2inv == s.delta2inv);
          if (!(q.C6 == s.C6 && q.d == s.d && q.seff == s.seff)) P.vdw_sym = 0;
          P.i_cutILPsq[a * MAXELEM + b] = (R)hi.cutILPsq[a * ne + b];
        }
      for (int a = 0; a < ne; a++)
        for (int b = 0; b < ne; b++)
          if (!(hi.cutILPsq[a * ne + b] == hi.cutILPsq[b * ne + a])) P.ilp_cut_sym = 0;
    }
    if (t_on) {
      int ne = P.t_ne;
      for (int a = 0; a < ne; a++)
        for (int b = 0; b < ne; b++)
          for (int c = 0; c < ne; c++) {
            const lmff_tersoff_param &q = ht.params[ht.elem2param[(a * ne + b) * ne + c]];
            TersP<R> &o = P.ters[(a * MAXELEM + b) * MAXELEM + c];
            o.lam1 = (R)q.lam1;
            o.lam2 = (R)q.lam2;
            o.lam3 = (R)q.lam3;
            o.c2 = (R)(q.c * q.c);
            o.d2 = (R)(q.d * q.d);
            o.h = (R)q.h;
            o.gamma = (R)q.gamma;
            o.powern = (R)q.powern;
            o.beta = (R)q.beta;
            o.biga = (R)q.biga;
            o.bigb = (R)q.bigb;
            o.bigr = (R)q.bigr;
            o.bigd = (R)q.bigd;
            o.cutsq = (R)q.cutsq;
            o.c1 = (R)q.c1;
            o.c2t = (R)q.c2;
            o.c3 = (R)q.c3;
            o.c4 = (R)q.c4;
            o.cd2 = (R)((q.c * q.c) / (q.d * q.d));
            o.inv2n = (R)(1.0 / (2.0 * q.powern));
            o.pi2_over_D = (R)(1.57079632679489661923 / q.bigd);
            o.pi4_over_D = (R)(0.78539816339744830962 / q.bigd);
            o.rlo = (R)(q.bigr - q.bigd);
            o.rhi = (R)(q.bigr + q.bigd);
            o.A64 = q.biga;
            o.B64 = q.bigb;
            o.lam1_64 = q.lam1;
            o.lam2_64 = q.lam2;
            o.R64 = q.bigr;
            o.D64 = q.bigd;
            o.rlo64 = q.bigr - q.bigd;
            o.rhi64 = q.bigr + q.bigd;
            o.pi4D64 = 0.78539816339744830962 / q.bigd;
            o.cutsq64 = q.cutsq;
            o.nl1x32 = -32.0 * q.lam1;
            o.nl2x32 = -32.0 * q.lam2;
            o.h64 = q.h;
            o.hhi = (float)q.h;
            o.hlo = (float)(q.h - (double)o.hhi);
            o.Al1_64 = q.biga * q.lam1;
            o.Bl2_64 = q.bigb * q.lam2;
            o.nl1h = (float)o.nl1x32;
            o.nl1l = (float)(o.nl1x32 - (double)o.nl1h);
            o.nl2h = (float)o.nl2x32;
            o.nl2l = (float)(o.nl2x32 - (double)o.nl2h);
            o.powermint = q.powermint;
          }
      for (int a = 0; a < ne; a++)
        for (int b = 0; b < ne; b++) {
          const lmff_tersoff_param &q = ht.params[ht.elem2param[(a * ne + b) * ne + b]];
          const lmff_tersoff_param &s = ht.params[ht.elem2param[(b * ne + a) * ne + a]];
          if (!(q.lam1 == s.lam1 && q.biga == s.biga && q.bigr == s.bigr && q.bigd == s.bigd)) P.rep_sym = 0;
        }
    }
  }

  int build_consts() {
    fill_pot(pot64);
    fill_pot(pot32);
    memset(&nbc, 0, sizeof nbc);
    cutneigh_max = 0.0;
    double rmaxilp = 0.0;
    for (int a = 0; a <= MAXTYPE; a++) nbc.ilp_mapped[a] = (i_on && a >= 1 && a <= ntypes && hi.map[a] >= 0) ? 1 : 0;
    for (int a = 0; a <= MAXTYPE; a++)
      for (int b = 0; b <= MAXTYPE; b++) {
        double cut = 0.0;
        if (a >= 1 && b >= 1 && a <= ntypes && b <= ntypes) {
          if (i_on && hi.map[a] >= 0 && hi.map[b] >= 0) cut = std::max(cut, cut_global);
          if (t_on && ht.map[a] >= 0 && ht.map[b] >= 0) cut = std::max(cut, ht.cutmax);
        }
        double cn = cut > 0.0 ? cut + skin : -1.0;
        nbc.cutnsq_d[a * (MAXTYPE + 1) + b] = cn > 0 ? cn * cn : -1.0;
        nbc.cutnsq_f[a * (MAXTYPE + 1) + b] = cn > 0 ? (float)(cn * cn) : -1.0f;
        cutneigh_max = std::max(cutneigh_max, cn);
      }
    if (i_on)
      for (double c : hi.cutILPsq) rmaxilp = std::max(rmaxilp, std::sqrt(c));
    rshort = std::max(rmaxilp, t_on ? ht.cutmax : 0.0) + skin;
    nbc.rshortsq_d = rshort * rshort;
    nbc.rshortsq_f = (float)(rshort * rshort);
    nbc.innersq_f = (float)(cut_global * cut_global);
    hash_tables();
    pot_dirty = true;
    built = false;
    return LMFF_OK;
  }

  // same parameters and tunables as o, fresh device state
  int clone_from(const Engine &o) {
    ntypes = o.ntypes;
    ht = o.ht;
    hi = o.hi;
    t_on = o.t_on;
    i_on = o.i_on;
    i_one = o.i_one;
    cut_global = o.cut_global;
    tap = o.tap;
    skin = o.skin;
    precision = o.precision;
    tpa = o.tpa;
    block = o.block;
    list_full = o.list_full;
    use_graphs = o.use_graphs;
    pdl_mask = o.pdl_mask;
    mass_type = o.mass_type;
    int rc = build_consts();
    if (rc) return rc;
    return init_device(o.device);
  }

  int init_device(int dev) {
    int cnt = 0;
    if (cudaGetDeviceCount(&cnt) != cudaSuccess || cnt == 0) return fail(LMFF_ENODEV, "no CUDA device");
    if (dev < 0 || dev >= cnt) return fail(LMFF_EINVAL, "device index out of range");
    device = dev;
    // LMFF_GB300_GRAPHS=0 turns the step graphs off (profilers cannot look inside a
    // graph with conditional nodes); the option "graphs" does the same per engine
    const char *eg = getenv("LMFF_GB300_GRAPHS");
    if (eg && eg[0] == '0') use_graphs = false;
    CK(cudaSetDevice(dev));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaMalloc(&d.status, sizeof(int)));
    CK(cudaMalloc(&d.maxdisp, sizeof(unsigned long long)));
    CK(cudaMallocHost(&h_words, 8 * sizeof(unsigned long long)));
    CK(cudaMalloc(&d_maxpred, 3 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(d_maxpred, 0, 3 * sizeof(unsigned long long), stream));
    CK(cudaMalloc(&d_cutILPsq, sizeof(double) * MAXELEM * MAXELEM));
    CK(cudaMalloc(&d_arrs, sizeof(double *) * 2));
    CK(cudaMalloc(&d_karrs, sizeof(double *) * 2));
    CK(cudaMalloc(&d_kout, sizeof(double)));
    CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
    return LMFF_OK;
  }

  // The device's constant tables are this engine's (guaranteed by DeviceCall); only the
  // engine-owned copy of the intralayer cutoffs may still need refreshing.
  int push_consts() {
    if (!pot_dirty) return LMFF_OK;
    double c[MAXELEM * MAXELEM] = {0};
    if (i_on) {
      int ne = (int)hi.elements.size();
      for (int a = 0; a < ne; a++)
        for (int b = 0; b < ne; b++) c[a * MAXELEM + b] = hi.cutILPsq[a * ne + b];
    }
    CK(cudaMemcpyAsync(d_cutILPsq, c, sizeof c, cudaMemcpyHostToDevice, stream));
    CK(cudaGetLastError());
    pot_dirty = false;
    return LMFF_OK;
  }

  // Upload the constant tables to the device (caller holds the device lock exclusively
  // and the device is idle); synchronous so that other streams see them complete.
  int upload_tables() {
    f64::upload_pot(pot64, stream);
    f32::upload_pot(pot32, stream);
    nb_upload_const(nbc, stream);
    CK(cudaStreamSynchronize(stream));
    CK(cudaGetLastError());
    return LMFF_OK;
  }

  static uint64_t fnv(const void *p, size_t n, uint64_t h) {
    const unsigned char *b = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    return h;
  }
  void hash_tables() {
    uint64_t h = 1469598103934665603ull;
    h = fnv(&pot64, sizeof pot64, h);
    h = fnv(&pot32, sizeof pot32, h);
    h = fnv(&nbc, sizeof nbc, h);
    table_hash = h ? h : 1;
  }

  // ---------------------------------------------------------------- capacity
  int cap_n = 0, cap_sys = 0;

  int ensure_atoms(int nn) {
    if (nn <= cap_n) return LMFF_OK;
    int c = nn + nn / 8 + 64;
    CK(cudaStreamSynchronize(stream));
    drop_graph();
    CK(dalloc(d.xq, c)); CK(dalloc(xq2, c)); CK(dalloc(d.xh, c)); CK(dalloc(d.xl, c));
    CK(dalloc(d.v, 3 * (size_t)c)); CK(dalloc(v2, 3 * (size_t)c)); CK(dalloc(d.f, 3 * (size_t)c));
    CK(dalloc(d.xhold, 3 * (size_t)c));
    CK(dalloc(d.tag, c)); CK(dalloc(tag2, c)); CK(dalloc(d.perm, c)); CK(dalloc(perm2, c));
    CK(dalloc(d.sysid, c)); CK(dalloc(sysid2, c)); CK(dalloc(d.mass, c)); CK(dalloc(mass2, c));
    CK(dalloc(d.nrm64, c)); CK(dalloc(d.nrm32, c)); CK(dalloc(d.jrec, 5 * (size_t)c));
    CK(dalloc(d.ilp_cnt, c)); CK(dalloc(d.ilp_nb, (size_t)c * MAXILP));
    CK(dalloc(d.ters_cnt, c)); CK(dalloc(d.ters_nb, (size_t)c * MAXTERS));
    CK(dalloc(d.ters_g, (size_t)c * MAXTERS)); CK(dalloc(d.ters_f, 3 * (size_t)c));
    CK(dalloc(d.ilp_f, 3 * (size_t)c)); CK(dalloc(d.ilp_c, (size_t)c * MAXILP)); CK(dalloc(d.ilp_g, c));
    CK(dalloc(d.nframe, 4 * (size_t)c));
    CK(dalloc(stat_ilp, 8 * (size_t)c)); CK(dalloc(stat_ters, 8 * (size_t)c));
    CK(dalloc(eatom_ilp, c)); CK(dalloc(eatom_ters, c)); CK(dalloc(ke, c));
    CK(dalloc(d.list_off, (size_t)c + 1)); CK(dalloc(d.short_cnt, c)); CK(dalloc(d.short_nb, (size_t)c * MAXSHORT));
    CK(dalloc(d.list_img, c)); CK(dalloc(d.nin_tmp, c));
    CK(dalloc(d.bin_key, c)); CK(dalloc(d.bin_key2, c)); CK(dalloc(d.idx, c)); CK(dalloc(d.idx2, c));
    CK(dalloc(d.cnt_tmp, (size_t)c + 1));
    CK(dalloc(d_xin, 3 * (size_t)c)); CK(dalloc(d_fin, 3 * (size_t)c)); CK(dalloc(d_vin, 3 * (size_t)c));
    CK(dalloc(d_fo, 3 * (size_t)c));
    CK(dalloc(d_ein, c)); CK(dalloc(d_tin, c)); CK(dalloc(d_sysin, c)); CK(dalloc(d_min, c)); CK(dalloc(d_gin, c));
    // CUB temporary storage for the sort (32 key bits) and the scan
    size_t tb = nb_sort_tmp_bytes(c, 32);
    if (d.cub_tmp) cudaFree(d.cub_tmp);
    d.cub_tmp = nullptr;
    CK(cudaMalloc(&d.cub_tmp, tb));
    d.cub_tmp_bytes = tb;
    cap_n = c;
    const double *arrs[2] = {stat_ilp, stat_ters};
    CK(cudaMemcpy(d_arrs, arrs, sizeof arrs, cudaMemcpyHostToDevice));
    const double *karrs[2] = {ke, ke};
    CK(cudaMemcpy(d_karrs, karrs, sizeof karrs, cudaMemcpyHostToDevice));
    return LMFF_OK;
  }

  // device bytes this engine holds (the arrays of ensure_atoms, the pair list, bins,
  // sort workspace and the step graph's checkpoint)
  double per_atom_bytes() const {
    double per_atom = 2 * sizeof(*d.xq) + sizeof(*d.xh) + sizeof(*d.xl) + 3 * (3 * sizeof(double)) +
                      3 * sizeof(double) + 2 * sizeof(*d.tag) + 4 * sizeof(int) + 2 * sizeof(double) +
                      sizeof(*d.nrm64) + sizeof(*d.nrm32) + 5 * sizeof(*d.jrec) + sizeof(*d.ilp_cnt) + MAXILP * sizeof(*d.ilp_nb) +
                      sizeof(*d.ters_cnt) + MAXTERS * (sizeof(*d.ters_nb) + sizeof(*d.ters_g)) +
                      2 * 3 * sizeof(double) + MAXILP * sizeof(*d.ilp_c) + sizeof(*d.ilp_g) + 16 * sizeof(double) +
                      3 * sizeof(double) + sizeof(*d.list_off) + sizeof(*d.list_img) + sizeof(*d.nin_tmp) + sizeof(*d.short_cnt) + MAXSHORT * sizeof(*d.short_nb) +
                      2 * sizeof(*d.bin_key) + 2 * sizeof(*d.idx) + sizeof(*d.cnt_tmp) + 3 * 3 * sizeof(double) +
                      sizeof(double) + 2 * sizeof(int) + 2 * sizeof(int64_t);
    if (bk_cap) per_atom += sizeof(d4) + 7 * sizeof(double) + sizeof(int64_t) + 2 * sizeof(int);
    return per_atom;
  }
  double device_bytes() const {
    return (double)cap_n * per_atom_bytes() + (double)(d.list_cap + d.tmp_cap) * sizeof(uint32_t) +
           (double)d.cub_tmp_bytes + (double)d.nbins_cap * 3 * sizeof(int) + (double)va_cap * VA_DOUBLES * sizeof(double);
  }
  // device bytes per atom a batch like the current one needs: the per-atom arrays with
  // their growth margin, the pair list at the current density with the step graph's
  // headroom, and the sort workspace
  double bytes_per_atom_need() const {
    if (n <= 0) return 0.0;
    double list_pa = (double)list_total / n;
    return 1.125 * per_atom_bytes() + 1.25 * 4.0 * list_pa + 4.0 * stride +
           (double)d.cub_tmp_bytes / std::max(cap_n, 1);
  }

  // stride for the next builds from the last build's largest count (1/8 + 32 headroom);
  // off when the scratch would exceed twice the list itself or does not fit
  void update_stride(int maxcnt) {
    int want = ((maxcnt + maxcnt / 8 + 32) + 31) & ~31;
    if (want <= stride && stride > 0) return;
    const int64_t need = (int64_t)cap_n * want;
    if (need > 2 * std::max<int64_t>(d.list_cap, 1024)) {
      stride = 0;
      return;
    }
    if (need > d.tmp_cap) {
      drop_graph();   // a captured rebuild holds the old scratch pointer and stride
      if (d.list_tmp) cudaFree(d.list_tmp);
      d.list_tmp = nullptr;
      d.tmp_cap = 0;
      if (cudaMalloc(&d.list_tmp, sizeof(uint32_t) * need) != cudaSuccess) {
        cudaGetLastError();
        stride = 0;
        return;
      }
      d.tmp_cap = need;
    } else {
      drop_graph();
    }
    stride = want;
  }

  int ensure_stream2() {
    if (stream2) return LMFF_OK;
    CK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&stream3, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_frame, cudaEventDisableTiming));
    return LMFF_OK;
  }

  int ensure_pinned(size_t bytes) {
    if (bytes <= h_pinned_bytes) return LMFF_OK;
    if (h_pinned) cudaFreeHost(h_pinned);
    h_pinned = nullptr;
    CK(cudaMallocHost(&h_pinned, bytes));
    h_pinned_bytes = bytes;
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- geometry
  // One SysDesc per system: bins of at least (cutneigh/2)*1.0001 so that any pair
  // within cutneigh is at most `reach` bins apart whatever the rounding of the bin index.
  int make_sys(std::vector<SysDesc> &out, const std::vector<std::array<double, 9>> &boxes) {
    out.clear();
    int bin_begin = 0;
    int R = 0;
    for (size_t s = 0; s < boxes.size(); s++) {
      const auto &b = boxes[s];
      SysDesc sd;
      memset(&sd, 0, sizeof sd);
      double lo[3], L[3];
      int per[3];
      for (int k = 0; k < 3; k++) {
        lo[k] = b[k];
        L[k] = b[3 + k] - b[k];
        per[k] = b[6 + k] != 0.0;
        if (!(L[k] > 0.0)) return fail(LMFF_EINVAL, "box length must be positive");
      }
      sys_geometry(sd, lo, L, per, cutneigh_max, R);
      sd.bin_begin = bin_begin;
      long long nbins = (long long)sd.nb[0] * sd.nb[1] * sd.nb[2];
      if (bin_begin + nbins > MAX_GLOBAL_BINS) return fail(LMFF_EOVERFLOW, "too many bins");
      bin_begin += (int)nbins;
      out.push_back(sd);
    }
    d.nbins = bin_begin;
    int w = 1;
    while ((1 << w) < 2 * R + 1) w++;
    lc.R = R;
    lc.w = w;
    lc.ibits = 32 - 3 * w;
    lc.imask = (lc.ibits >= 32) ? 0xffffffffu : ((1u << lc.ibits) - 1u);
    lc.wmask = (1u << w) - 1u;
    nbit_bins = 1;
    while ((1LL << nbit_bins) < d.nbins) nbit_bins++;
    return LMFF_OK;
  }

  int upload_sys() {
    drop_graph();   // bins, image code and sort width are frozen in a captured step
    if ((int)hsys.size() > cap_sys) {
      CK(dalloc(d.sys, hsys.size()));
      CK(dalloc(d.red_out, hsys.size() * 16));
      cap_sys = (int)hsys.size();
    }
    CK(cudaMemcpyAsync(d.sys, hsys.data(), sizeof(SysDesc) * hsys.size(), cudaMemcpyHostToDevice, stream));
    if (d.nbins > d.nbins_cap) {
      CK(dalloc(d.bin_start, d.nbins));
      CK(dalloc(d.bin_end, d.nbins));
      CK(dalloc(d.rowocc, d.nbins));
      d.nbins_cap = d.nbins;
    }
    d.nsys = (int)hsys.size();
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- load / rebuild
  int load_from_staging(int nn, bool have_v, bool have_sysid) {
    drop_graph();
    n = nn;
    d.n = nn;
    if ((int64_t)n >= (1LL << lc.ibits))
      return fail(LMFF_EOVERFLOW, "too many atoms for the 32-bit neighbour-list code of this box");
    int g = (n + 255) / 256;
    if (n) {
      k_load<<<g, 256, 0, stream>>>(n, d_xin, d_tin, d_min, d_gin, have_v ? d_vin : nullptr, d_massT,
                                    have_sysid ? d_sysin : nullptr, d.xq, d.tag, d.perm, d.sysid, d.v, d.mass);
      CK(cudaGetLastError());
    }
    loaded = true;
    built = false;
    forces_valid = false;
    last_res_valid = false;
    return rebuild();
  }

  // the sorted copies back into the primary arrays, so device pointers stay fixed
  // across rebuilds (a captured step graph holds them)
  cudaError_t copy_back_permuted(cudaStream_t s) {
    cudaMemcpyAsync(d.xq, xq2, sizeof(d4) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d.v, v2, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d.tag, tag2, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d.perm, perm2, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d.sysid, sysid2, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    return cudaMemcpyAsync(d.mass, mass2, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  }

  int rebuild() {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, stream);
    int rc = push_consts();
    if (rc) return rc;
    if (n == 0) {
      built = true;
      return LMFF_OK;
    }
    int g = (n + 255) / 256;
    nb_wrap_bin(n, d.xq, d.sys, d.sysid, d.bin_key, d.idx, stream);
    CK(nb_sort(d.cub_tmp, d.cub_tmp_bytes, d.bin_key, d.bin_key2, d.idx, d.idx2, n, (int)nbit_bins, stream));
    nb_permute(n, d.idx2, d.xq, xq2, d.v, v2, d.tag, tag2, d.perm, perm2, d.sysid, sysid2, d.mass, mass2, stream);
    CK(copy_back_permuted(stream));
    CK(cudaMemsetAsync(d.bin_start, 0, sizeof(int) * d.nbins, stream));
    CK(cudaMemsetAsync(d.bin_end, 0, sizeof(int) * d.nbins, stream));
    CK(cudaMemsetAsync(d.rowocc, 0, sizeof(int) * d.nbins, stream));
    nb_bin_ranges(n, d.bin_key2, d.bin_start, d.bin_end, stream, d.sys, d.sysid, d.rowocc);
    // atoms' systems are contiguous after the sort: atom ranges per system
    CK(cudaGetLastError());
    hilo_all();
    NbArgs a;
    memset(&a, 0, sizeof a);
    a.n = n;
    a.no_small = !small_variants;
    a.xq = d.xq;
    a.xh = d.xh;
    a.xl = d.xl;
    a.sys = d.sys;
    a.sysid = d.sysid;
    a.bin_start = d.bin_start;
    a.bin_end = d.bin_end;
    a.rowocc = d.rowocc;
    a.nbins = d.nbins;
    a.bin_key = d.bin_key2;
    a.list_off = d.list_off;
    a.list = d.list;
    a.list_cap = d.list_cap;
    a.cnt = d.cnt_tmp;
    a.short_cnt = d.short_cnt;
    a.short_nb = d.short_nb;
    a.img = d.list_img;
    a.lc = lc;
    a.full = list_full;
    a.status = d.status;
    if (!d_maxcnt) CK(cudaMalloc(&d_maxcnt, sizeof(int)));
    bool strided = stride > 0 && d.list_tmp && (int64_t)n * stride <= d.tmp_cap;
    a.tmp = d.list_tmp;
    a.stride = strided ? stride : 0;
    a.nin = d.nin_tmp;
    a.maxcnt = d_maxcnt;
    CK(cudaMemsetAsync(d_maxcnt, 0, sizeof(int), stream));
    CK(cudaMemsetAsync(d.cnt_tmp + n, 0, sizeof(int64_t), stream));
    nb_list(a, strided ? 2 : 0, stream);
    CK(nb_scan(d.cub_tmp, d.cub_tmp_bytes, d.cnt_tmp, d.list_off, n, stream));
    int64_t total = 0;
    int st0 = 0, maxcnt = 0;
    CK(cudaMemcpyAsync(&total, d.list_off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&st0, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&maxcnt, d_maxcnt, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (strided && (st0 & ST_STRIDE_OVERFLOW)) {   // an atom outgrew the stride: fill pass instead
      strided = false;
      st0 &= ~(ST_STRIDE_OVERFLOW | ST_LIST_OVERFLOW);
      CK(cudaMemcpyAsync(d.status, &st0, sizeof(int), cudaMemcpyHostToDevice, stream));
    }
    if (total < 0 || total > (int64_t)n * 65536)
      return fail(LMFF_EOVERFLOW, "pair-list count out of range (" + std::to_string(total) + ")");
    if (total > d.list_cap) {
      int64_t cap = total + total / 8 + 1024;
      drop_graph();
      if (d.list) cudaFree(d.list);
      d.list = nullptr;
      cudaError_t e = cudaMalloc(&d.list, sizeof(uint32_t) * cap);
      if (e != cudaSuccess) {
        d.list_cap = 0;
        return fail(LMFF_ENOMEM, "pair list of " + std::to_string(total) + " entries does not fit on the device");
      }
      d.list_cap = cap;
    }
    a.list = d.list;
    a.list_cap = d.list_cap;
    if (strided) nb_compact(a, d.list_cap, stream);
    else nb_list(a, 1, stream);
    nb_copy_hold(n, d.xq, d.xhold, stream);
    CK(cudaGetLastError());
    // atoms of one system stay contiguous after the sort (bins of system s precede
    // those of s+1), so the ranges follow from the per-system atom counts
    if (batch_offsets.size() == hsys.size() + 1) {
      for (size_t s = 0; s < hsys.size(); s++) {
        hsys[s].atom_begin = batch_offsets[s];
        hsys[s].atom_end = batch_offsets[s + 1];
      }
    } else {
      hsys[0].atom_begin = 0;
      hsys[0].atom_end = n;
    }
    CK(cudaMemcpyAsync(d.sys, hsys.data(), sizeof(SysDesc) * hsys.size(), cudaMemcpyHostToDevice, stream));
    int st = 0;
    CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemsetAsync(d.maxdisp, 0, sizeof(unsigned long long), stream));
    cudaEventRecord(e1, stream);
    CK(cudaStreamSynchronize(stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ms_build = ms;
    if (ktiming) {
      kms[5] += ms;
      klaunch[5]++;
    }
    list_total = total;
    if (st) return status_error(st);
    update_stride(maxcnt);
    built = true;
    forces_valid = false;
    rebuilds++;
    return LMFF_OK;
  }

  void hilo_all(cudaStream_t s = nullptr) { nb_hilo(n, d.xq, d.sys, d.sysid, d.xh, d.xl, s ? s : stream); }

  int status_error(int st) {
    CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
    if (st & ST_TOO_MANY_ILP)
      return fail(LMFF_ETOO_MANY_ILP_NEIGH,
                  "There are too many neighbors for some atoms, please check your configuration");
    if (st & ST_ZERO_NORMAL) return fail(LMFF_EZERO_NORMAL, "The magnitude of the normal vector is zero");
    if (st & ST_TERS_OVERFLOW) return fail(LMFF_EOVERFLOW, "more than 12 Tersoff neighbours within cutmax for an atom");
    if (st & ST_SHORT_OVERFLOW) return fail(LMFF_EOVERFLOW, "more than 64 short-range candidates for an atom");
    if (st & ST_LIST_OVERFLOW) return fail(LMFF_EOVERFLOW, "Neighbor list overflow");
    return fail(LMFF_ECUDA, "kernel status " + std::to_string(st));
  }

  // rebuild when any atom moved more than skin/2 since the last build; ahead: also when
  // one may before the next check (the look-ahead reach k_nve1 left in d_maxpred)
  int maybe_rebuild(bool ahead = false) {
    unsigned long long bits[2] = {0, 0};
    CK(cudaMemcpyAsync(&bits[0], d.maxdisp, sizeof bits[0], cudaMemcpyDeviceToHost, stream));
    if (ahead) {
      CK(cudaMemcpyAsync(&bits[1], d_maxpred, sizeof bits[1], cudaMemcpyDeviceToHost, stream));
      CK(cudaMemsetAsync(d_maxpred, 0, sizeof bits[1], stream));
    }
    CK(cudaStreamSynchronize(stream));
    double d2[2];
    memcpy(d2, bits, sizeof d2);
    if (!built || d2[0] > 0.25 * skin * skin || (ahead && d2[1] > 0.25 * skin * skin)) return rebuild();
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- rebuild checks
  // The list is tested every ck-th step of an NVE run (steps whose index is a multiple of
  // ck) with the look-ahead; ck = 1 tests every step for displacement alone, as LAMMPS's
  // neigh_modify every 1 delay 0 check yes.  Forces do not depend on when the list is
  // rebuilt (the cutoff tests are exact), only the order of some sums does.
  static constexpr int LOOKAHEAD_MAX_ATOMS = 65536;
  static constexpr int LOOKAHEAD_MAX_EVERY = 8;
  int check_every_opt = 0;   // option "check_every": 0 = chosen per run, k >= 1 = every k steps
  int ck = 1;                // the interval of the current run
  unsigned long long *d_maxpred = nullptr;   // [0] look-ahead reach, [1..2] motion bound

  bool check_step(int64_t step) const { return ck <= 1 || step % ck == 0; }
  Lookahead lookahead_for(bool check, bool graph, double dt) const {
    Lookahead la{};
    if (ck <= 1) return la;
    if (check) {
      la.pred = d_maxpred;
      la.hv = 1.25 * (ck - 1) * dt;
      la.ha = 1.25 * (double)(ck - 1) * (ck - 1) * dt;
    } else if (graph) {
      la.status = d.status;
      la.trig2 = 0.25 * skin * skin;
    }
    return la;
  }
  // the run's check interval: the largest of 8, 4, 2 whose look-ahead reach from the
  // current motion stays within skin/4 (half the margin, so that a check rarely finds
  // a rebuild needed right after the last one), else 1
  int choose_check_every(double dt) {
    ck = 1;
    if (check_every_opt >= 1) {
      ck = check_every_opt;
      return LMFF_OK;
    }
    if (n == 0 || n > LOOKAHEAD_MAX_ATOMS || !(skin > 0.0)) return LMFF_OK;
    CK(cudaMemsetAsync(d_maxpred + 1, 0, 2 * sizeof(unsigned long long), stream));
    k_motion_max<<<(n + 255) / 256, 256, 0, stream>>>(n, d.v, d.f, d.xq, dtfm_table(0.5 * dt * FTM2V), d_maxpred + 1);
    CK(cudaGetLastError());
    unsigned long long bits[2] = {0, 0};
    CK(cudaMemcpyAsync(bits, d_maxpred + 1, sizeof bits, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    double m2[2];
    memcpy(m2, bits, sizeof m2);
    const double vmax = sqrt(m2[0]), amax = sqrt(m2[1]);
    for (int k = LOOKAHEAD_MAX_EVERY; k >= 2; k /= 2) {
      if (1.25 * ((k - 1) * dt * vmax + (double)(k - 1) * (k - 1) * dt * amax) <= 0.25 * skin) {
        ck = k;
        break;
      }
    }
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- forces
  template <class R>
  ForceArgs<R> args() {
    ForceArgs<R> a;
    memset(&a, 0, sizeof a);
    a.A.xq = d.xq;
    a.A.xh = d.xh;
    a.A.xl = d.xl;
    a.A.jrec = d.jrec;
    a.A.jrec2 = d.jrec + 3 * (size_t)cap_n;
    a.A.sys = d.sys;
    a.A.sysid = d.sysid;
    a.lc = lc;
    a.n = n;
    a.tag = d.tag;
    a.list_off = d.list_off;
    a.list = d.list;
    a.list_img = d.list_img;
    a.short_cnt = d.short_cnt;
    a.short_nb = d.short_nb;
    a.ilp_cnt = d.ilp_cnt;
    a.ilp_nb = d.ilp_nb;
    a.ters_cnt = d.ters_cnt;
    a.ters_nb = d.ters_nb;
    a.nrm64 = d.nrm64;
    a.nrm32 = d.nrm32;
    a.jrec = d.jrec;
    a.jrec2 = d.jrec + 3 * (size_t)cap_n;
    a.ters_g = d.ters_g;
    a.ters_f = d.ters_f;
    a.ilp_f = d.ilp_f;
    a.ilp_c = d.ilp_c;
    a.ilp_g = d.ilp_g;
    a.nframe = d.nframe;
    a.stat_ilp = stat_ilp;
    a.stat_ters = stat_ters;
    a.eatom_ilp = eatom_ilp;
    a.eatom_ters = eatom_ters;
    a.f_out = d.f;
    a.status = d.status;
    a.list_full = list_full;
    a.own_perm = ghost_nlocal >= 0 ? d.perm : nullptr;
    a.nown = ghost_nlocal;
    a.pair_tile = pair_tile;
    a.no_small = !small_variants;
    a.kc = i_on && hi.model == LMFF_INTERLAYER_KC;
    // not while kernels are timed one by one (events between the launches)
    if (!ktiming && n <= PDL_MAX_ATOMS) a.pdl = pdl_short ? pdl_mask : (pdl_mask & ~PDL_SHORT);
    return a;
  }

  template <class R, class NS_SHORT, class NS_TERS, class NS_ILP, class NS_FR, class NS_ND, class NS_FIN>
  void run_kernels(ForceArgs<R> a, int which, bool ev, bool eatom, NS_SHORT fs, NS_TERS ft, NS_ILP fi, NS_FR fr,
                   NS_ND fn, NS_FIN ff) {
    a.do_ters = t_on && (which & LMFF_TERSOFF);
    a.do_ilp = i_on && (which & LMFF_ILP);
    timed(2, [&] { fs(a, d_cutILPsq, ht.cutmax * ht.cutmax, stream); });
    // Tersoff (FP64-pipe bound) on a second stream beside the pair kernel (FP32 bound):
    // the two share the SMs and overlap; joined before the gather.  Serial when the
    // kernels are timed one by one.
    const bool fork = a.do_ters && a.do_ilp && ters_concurrent && !ktiming && ensure_stream2() == LMFF_OK;
    a.ters_alone = !fork;
    // the normal frames (the g-independent part of the normal-derivative assembly) on a
    // third stream, beside both
    if (fork) {
      cudaEventRecord(ev_fork, stream);
      cudaStreamWaitEvent(stream2, ev_fork, 0);
      cudaStreamWaitEvent(stream3, ev_fork, 0);
      fr(a, stream3);
      cudaEventRecord(ev_frame, stream3);
      ft(a, ev, eatom, stream2);
      cudaEventRecord(ev_join, stream2);
    } else if (a.do_ters) {
      timed(1, [&] { ft(a, ev, eatom, stream); });
    } else if (ev) {
      cudaMemsetAsync(stat_ters, 0, sizeof(double) * 8 * (size_t)n, stream);
    }
    if (a.do_ilp) {
      if (!fork) timed(6, [&] { fr(a, stream); });
      timed(0, [&] { fi(a, ev, eatom, tpa, block, i_one, stream); });
      if (fork) cudaStreamWaitEvent(stream, ev_frame, 0);
      timed(6, [&] { fn(a, ev, stream); });
    }
    else if (ev) cudaMemsetAsync(stat_ilp, 0, sizeof(double) * 8 * (size_t)n, stream);
    if (eatom && !a.do_ters) cudaMemsetAsync(eatom_ters, 0, sizeof(double) * (size_t)n, stream);
    if (fork) cudaStreamWaitEvent(stream, ev_join, 0);
    timed(3, [&] { ff(a, eatom, kick_on ? &kick_args : nullptr, stream); });
  }

  // forces (+ energies/virials per system into hres when ev) on the resident state
  // wait = false (force-only evaluations): the status word comes back into a pinned word
  // and the caller waits once for everything it queued, then calls forces_done
  int forces(int which, bool ev, bool eatom, std::vector<lmff_result> *hres, bool wait = true) {
    int rc = push_consts();
    if (rc) return rc;
    if (!built) {
      rc = rebuild();
      if (rc) return rc;
    }
    if (eatom) ev = true;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, stream);
    if (n > 0) {
      if (precision == LMFF_MIXED && !hilo_fresh) hilo_all();
      const bool cap = use_graphs && !ktiming && !kick_on;
      std::vector<unsigned char> key;
      if (cap) {
        if (ters_concurrent && ensure_stream2() != LMFF_OK) return LMFF_ECUDA;   // before any capture
        key = force_key(which, ev, eatom);
      }
      if (cap && fexec && key == fkey) {
        CK(cudaGraphLaunch(fexec, stream));
      } else {
        if (cap) {
          drop_fgraph();
          CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        }
        if (precision == LMFF_FP64) {
          run_kernels(args<double>(), which, ev, eatom, f64::launch_short, f64::launch_tersoff, f64::launch_ilp,
                      f64::launch_nframe, f64::launch_nderiv, f64::launch_finish);
        } else {
          run_kernels(args<float>(), which, ev, eatom, f32::launch_short, f32::launch_tersoff, f32::launch_ilp,
                      f32::launch_nframe, f32::launch_nderiv, f32::launch_finish);
        }
        if (ev) k_reduce<<<(int)hsys.size() * 16, 256, 0, stream>>>(n, 16, (const double *const *)d_arrs, d.sys, d.red_out);
        if (cap) {
          cudaGraph_t g = nullptr;
          cudaError_t e = cudaStreamEndCapture(stream, &g);
          if (e == cudaSuccess) e = cudaGraphInstantiate(&fexec, g, 0);
          if (g) cudaGraphDestroy(g);
          if (e != cudaSuccess) {
            fexec = nullptr;
            return fail(LMFF_ECUDA, std::string("force graph: ") + cudaGetErrorString(e));
          }
          fkey = key;
          CK(cudaGraphLaunch(fexec, stream));
        }
      }
      CK(cudaGetLastError());
    }
    cudaEventRecord(e1, stream);
    if (!wait && !ev && !hres) {
      pend_e0 = e0;
      pend_e1 = e1;
      CK(cudaMemcpyAsync(h_words, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
      return LMFF_OK;
    }
    int st = 0;
    CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    std::vector<double> red;
    if (ev && n > 0) {
      red.resize(hsys.size() * 16);
      CK(cudaMemcpyAsync(red.data(), d.red_out, sizeof(double) * red.size(), cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaStreamSynchronize(stream));
    harvest();
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ms_forces = ms;
    if (st) return status_error(st);
    forces_valid = true;
    if (ev && hres) last_res_valid = true;
    if (hres) {
      hres->assign(hsys.size(), lmff_result());
      for (size_t s = 0; s < hsys.size(); s++) {
        lmff_result &r = (*hres)[s];
        memset(&r, 0, sizeof r);
        if (!ev || n == 0) continue;
        const double *q = &red[s * 16];
        r.pvector[0] = q[0];
        r.pvector[1] = q[1];
        r.e_ilp = q[0] + q[1];
        for (int k = 0; k < 6; k++) r.virial_ilp[k] = q[2 + k];
        r.e_tersoff = q[8];
        for (int k = 0; k < 6; k++) r.virial_tersoff[k] = q[10 + k];
      }
      if (ev) last_res = *hres;
    }
    return LMFF_OK;
  }
  // the end of a force evaluation queued with wait = false, after the caller's wait
  int forces_done() {
    harvest();
    float ms = 0;
    cudaEventElapsedTime(&ms, pend_e0, pend_e1);
    cudaEventDestroy(pend_e0);
    cudaEventDestroy(pend_e1);
    pend_e0 = pend_e1 = nullptr;
    ms_forces = ms;
    const int st = (int)*reinterpret_cast<const int *>(h_words);
    if (st) return status_error(st);
    forces_valid = true;
    return LMFF_OK;
  }
  bool hilo_fresh = false;

  // ---------------------------------------------------------------- API paths
  int set_single_box() {
    if (!have_box) return fail(LMFF_EINVAL, "lmff_set_box must be called first");
    std::vector<std::array<double, 9>> boxes(1);
    for (int k = 0; k < 3; k++) {
      boxes[0][k] = blo[k];
      boxes[0][3 + k] = bhi[k];
      boxes[0][6 + k] = bper[k];
    }
    int rc = make_sys(hsys, boxes);
    if (rc) return rc;
    return upload_sys();
  }

  // the checks of check_mol without the error message (thread-safe)
  bool ids_ok(int nn, const int64_t *mol, const int *type) const {
    for (int p = 0; p < nn; p++) {
      if (mol && (mol[p] < 0 || mol[p] >= (1LL << 23))) return false;
      if (type[p] < 1 || type[p] > ntypes) return false;
    }
    return true;
  }

  int check_mol(int nn, const int64_t *mol, const int *type) {
    for (int p = 0; p < nn; p++) {
      if (mol && (mol[p] < 0 || mol[p] >= (1LL << 23)))
        return fail(LMFF_EUNSUPPORTED, "molecule ids must lie in [0, 2^23)");
      if (type[p] < 1 || type[p] > ntypes) return fail(LMFF_EINVAL, "atom type out of range");
    }
    return LMFF_OK;
  }

  // stage caller host arrays; returns whether the identity must be (re)loaded
  int stage_host(int nn, const double *x, const int *type, const int64_t *mol, const int64_t *tag, bool same_atoms,
                 bool &reload) {
    int rc = ensure_atoms(nn);
    if (rc) return rc;
    CK(cudaMemcpyAsync(d_xin, x, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, stream));
    reload = !loaded || nn != n || !built;
    if (!same_atoms || reload) {
      rc = check_mol(nn, mol, type);
      if (rc) return rc;
      CK(cudaMemcpyAsync(d_tin, type, sizeof(int) * nn, cudaMemcpyHostToDevice, stream));
      if (mol) CK(cudaMemcpyAsync(d_min, mol, sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
      else CK(cudaMemsetAsync(d_min, 0, sizeof(int64_t) * nn, stream));
      if (tag) CK(cudaMemcpyAsync(d_gin, tag, sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
      if (!reload && nn > 0) {
        CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
        k_check_ident<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d_tin, d_min, tag ? d_gin : nullptr, d.xq, d.tag,
                                                            d.status);
        int flag = 0;
        CK(cudaMemcpyAsync(&flag, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
        CK(cudaStreamSynchronize(stream));
        if (flag) reload = true;
      }
      if (!tag && reload) {
        // default tags 1..n
        std::vector<int64_t> t(nn);
        for (int p = 0; p < nn; p++) t[p] = p + 1;
        CK(cudaMemcpyAsync(d_gin, t.data(), sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
      }
    }
    return LMFF_OK;
  }

  // test: rebuild now if an atom moved more than skin/2 (else the caller tests later)
  int apply_positions(int nn, bool reload, bool test = true) {
    if (reload) {
      if (!mass_type.empty()) {
        if (!d_massT) CK(cudaMalloc(&d_massT, sizeof(double) * (MAXTYPE + 1)));
        CK(cudaMemcpyAsync(d_massT, mass_type.data(), sizeof(double) * mass_type.size(), cudaMemcpyHostToDevice, stream));
      }
      batch_offsets.clear();
      int rc = set_single_box();
      if (rc) return rc;
      return load_from_staging(nn, false, false);
    }
    if (nn > 0) {
      k_update_x<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d_xin, d.xq, d.xhold, d.maxdisp, d.sys, d.sysid);
      CK(cudaGetLastError());
    }
    hilo_fresh = false;
    if (precision == LMFF_MIXED) {
      hilo_all();
      hilo_fresh = true;
    }
    return test ? maybe_rebuild() : LMFF_OK;
  }

  int compute_host(int nn, const double *x, const int *type, const int64_t *mol, const int64_t *tag, int which,
                   int eflag, int vflag, double *f, double *eatom, lmff_result *res) {
    bool reload = false;
    int rc = stage_host(nn, x, type, mol, tag, (which & LMFF_SAME_ATOMS) != 0, reload);
    if (rc) return rc;
    if (!reload && nn > 0 && f && !eatom && !eflag && !vflag) return compute_forces_one_wait(nn, which, f, res);
    rc = apply_positions(nn, reload);
    if (rc) return rc;
    std::vector<lmff_result> hr;
    bool ev = eflag || vflag || eatom;
    rc = forces(which, ev, eatom != nullptr, &hr);
    if (rc) return rc;
    if (res) *res = hr.empty() ? lmff_result() : hr[0];
    bool overwrite = (which & LMFF_OVERWRITE) != 0;
    if (nn > 0 && f) {
      if (!overwrite) CK(cudaMemcpyAsync(d_fin, f, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, stream));
      k_scatter_add<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d.f, d_fin, overwrite);
      CK(cudaMemcpyAsync(f, d_fin, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, stream));
    }
    if (nn > 0 && eatom) {
      if (!overwrite) CK(cudaMemcpyAsync(d_ein, eatom, sizeof(double) * nn, cudaMemcpyHostToDevice, stream));
      k_scatter_add1<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, eatom_ters, d_ein, overwrite);
      CK(cudaMemcpyAsync(eatom, d_ein, sizeof(double) * nn, cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaStreamSynchronize(stream));
    return LMFF_OK;
  }

  // Forces only, on loaded atoms (a pair style's call on most steps), with one host wait.
  // The list test comes after the evaluation: the forces run on the current list at once
  // and the largest displacement since the build comes back with them.  In the rare call
  // where an atom moved more than skin/2 the list is rebuilt and the evaluation repeated
  // (the first result is discarded; the caller's input forces stay in d_fin meanwhile).
  int compute_forces_one_wait(int nn, int which, double *f, lmff_result *res) {
    int rc = apply_positions(nn, false, false);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h_words + 1, d.maxdisp, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    rc = forces(which, false, false, nullptr, false);
    if (rc) return rc;
    const bool overwrite = (which & LMFF_OVERWRITE) != 0;
    if (!overwrite) CK(cudaMemcpyAsync(d_fin, f, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, stream));
    k_scatter_sum<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d.f, overwrite ? nullptr : d_fin, d_fo);
    CK(cudaMemcpyAsync(f, d_fo, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    double d2;
    memcpy(&d2, h_words + 1, sizeof d2);
    if (!(d2 > 0.25 * skin * skin)) {
      rc = forces_done();
      if (rc) return rc;
    } else {
      // the list did not cover these positions: the evaluation (and any status it
      // raised) is discarded
      harvest();
      cudaEventDestroy(pend_e0);
      cudaEventDestroy(pend_e1);
      pend_e0 = pend_e1 = nullptr;
      CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
      rc = rebuild();
      if (rc) return rc;
      rc = forces(which, false, false, nullptr);
      if (rc) return rc;
      k_scatter_sum<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d.f, overwrite ? nullptr : d_fin, d_fo);
      CK(cudaMemcpyAsync(f, d_fo, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, stream));
      CK(cudaStreamSynchronize(stream));
    }
    if (res) memset(res, 0, sizeof *res);
    return LMFF_OK;
  }

  // Subdomain mode: x[nall*3] holds the caller's owned atoms [0, nlocal) followed by
  // ghost atoms, in a box the engine chooses itself (non-periodic, around all nall atoms
  // with room for the skin; the ghosts carry the periodic images).  Only interactions
  // owned by owned atoms are evaluated; every atom receives its share of their forces
  // (f[nall*3]) and per-atom energy, and the energies and virial are those of the owned
  // interactions, so that summing over subdomains after the ghost forces are folded back
  // gives the whole system's.
  int compute_ghost(int nlocal, int nall, const double *x, const int *type, const int64_t *mol, const int64_t *tag,
                    int which, int eflag, int vflag, double *f, double *eatom, lmff_result *res) {
    if (nlocal < 0 || nall < nlocal) return fail(LMFF_EINVAL, "lmff_compute_ghost: need 0 <= nlocal <= nall");
    const bool same = (which & LMFF_SAME_ATOMS) && ghost_nlocal == nlocal && have_box && loaded && built && n == nall;
    if (!same) {
      double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {1.0, 1.0, 1.0};
      for (int p = 0; p < nall; p++)
        for (int k = 0; k < 3; k++) {
          const double c = x[3 * p + k];
          if (!std::isfinite(c)) return fail(LMFF_EINVAL, "lmff_compute_ghost: non-finite coordinate");
          if (p == 0 || c < lo[k]) lo[k] = c;
          if (p == 0 || c > hi[k]) hi[k] = c;
        }
      const double pad = skin + 1.0;
      for (int k = 0; k < 3; k++) {
        blo[k] = lo[k] - pad;
        bhi[k] = hi[k] + pad;
        bper[k] = 0;
      }
      have_box = true;
      loaded = false;
      built = false;
      which &= ~LMFF_SAME_ATOMS;
    }
    ghost_nlocal = nlocal;
    return compute_host(nall, x, type, mol, tag, which, eflag, vflag, f, eatom, res);
  }

  // A triclinic periodic box (domain.cpp: h = [[lx, xy, xz], [0, ly, yz], [0, 0, lz]],
  // lamda = h^-1 (x - lo)): the owned atoms are wrapped into the box by whole lattice
  // vectors (an atom inside keeps its coordinates to the bit), then every periodic image
  // whose lamda lies within the ghost cutoff of the box, cutneigh in each direction
  // (lamda_d within cutneigh |row d of h^-1| of [0, 1), the distance between the box's
  // faces of constant lamda_d being 1 / |row d|), is added as a ghost carrying its
  // owner's type, molecule and tag -- the atoms a LAMMPS rank holds (comm_brick.cpp
  // borders, domain.cpp pbc) -- and the subdomain form evaluates them.  The images'
  // forces and per-atom energies are folded into their owners.
  int compute_tri(int nn, const double *x, const int *type, const int64_t *mol, const int64_t *tag, int which,
                  int eflag, int vflag, double *f, double *eatom, lmff_result *res) {
    const double lx = thi[0] - tlo[0], ly = thi[1] - tlo[1], lz = thi[2] - tlo[2];
    const double xy = tilt[0], xz = tilt[1], yz = tilt[2];
    const double col[3][3] = {{lx, 0.0, 0.0}, {xy, ly, 0.0}, {xz, yz, lz}};
    // rows of h^-1 (domain.cpp h_inv)
    const double r0[3] = {1.0 / lx, -xy / (lx * ly), (xy * yz - ly * xz) / (lx * ly * lz)};
    const double r1[3] = {0.0, 1.0 / ly, -yz / (ly * lz)};
    const double r2[3] = {0.0, 0.0, 1.0 / lz};
    const double *row[3] = {r0, r1, r2};
    const double cg = cutneigh_max > 0.0 ? cutneigh_max : skin;
    double cl[3];
    int K[3];
    for (int d = 0; d < 3; d++) {
      cl[d] = cg * std::sqrt(row[d][0] * row[d][0] + row[d][1] * row[d][1] + row[d][2] * row[d][2]);
      K[d] = tper[d] ? (int)std::ceil(cl[d]) : 0;
    }
    std::vector<double> xw(3 * (size_t)nn), lam(3 * (size_t)nn);
    for (int p = 0; p < nn; p++) {
      const double q[3] = {x[3 * p] - tlo[0], x[3 * p + 1] - tlo[1], x[3 * p + 2] - tlo[2]};
      double l[3], s[3];
      for (int d = 0; d < 3; d++) {
        l[d] = row[d][0] * q[0] + row[d][1] * q[1] + row[d][2] * q[2];
        if (!std::isfinite(l[d])) return fail(LMFF_EINVAL, "lmff_compute: non-finite coordinate");
        s[d] = tper[d] ? std::floor(l[d]) : 0.0;
      }
      for (int c = 0; c < 3; c++) {
        const double sh = s[0] * col[0][c] + s[1] * col[1][c] + s[2] * col[2][c];
        xw[3 * p + c] = sh != 0.0 ? x[3 * p + c] - sh : x[3 * p + c];
      }
      for (int d = 0; d < 3; d++) lam[3 * p + d] = l[d] - s[d];
    }
    std::vector<double> xs(xw);
    std::vector<int> ts(type, type + nn), own(nn);
    std::vector<int64_t> ms(nn), gs(nn);
    for (int p = 0; p < nn; p++) {
      own[p] = p;
      ms[p] = mol ? mol[p] : 0;
      gs[p] = tag ? tag[p] : (int64_t)(p + 1);
    }
    for (int a = -K[0]; a <= K[0]; a++)
      for (int b = -K[1]; b <= K[1]; b++)
        for (int c = -K[2]; c <= K[2]; c++) {
          if (a == 0 && b == 0 && c == 0) continue;
          const int sh[3] = {a, b, c};
          double dv[3];
          for (int k = 0; k < 3; k++) dv[k] = a * col[0][k] + b * col[1][k] + c * col[2][k];
          for (int p = 0; p < nn; p++) {
            bool in = true;
            for (int d = 0; d < 3 && in; d++) {
              if (!tper[d]) continue;   // no images along a non-periodic direction
              const double l = lam[3 * p + d] + sh[d];
              in = l >= -cl[d] && l < 1.0 + cl[d];
            }
            if (!in) continue;
            for (int k = 0; k < 3; k++) xs.push_back(xw[3 * p + k] + dv[k]);
            ts.push_back(type[p]);
            ms.push_back(ms[p]);
            gs.push_back(gs[p]);
            own.push_back(p);
          }
        }
    if (xs.size() / 3 > (size_t)INT32_MAX / 2) return fail(LMFF_EOVERFLOW, "lmff_compute: too many periodic images");
    const int nall = (int)own.size();
    std::vector<double> fa(3 * (size_t)nall, 0.0), ea(eatom ? (size_t)nall : 0, 0.0);
    int rc = compute_ghost(nn, nall, xs.data(), ts.data(), ms.data(), gs.data(), which & (LMFF_TERSOFF | LMFF_ILP),
                           eflag, vflag, fa.data(), eatom ? ea.data() : nullptr, res);
    if (rc) return rc;
    const bool overwrite = (which & LMFF_OVERWRITE) != 0;
    if (f && overwrite) memset(f, 0, sizeof(double) * 3 * (size_t)nn);
    if (eatom && overwrite) memset(eatom, 0, sizeof(double) * (size_t)nn);
    for (int a = 0; a < nall; a++) {
      const int o = own[a];
      if (f)
        for (int c = 0; c < 3; c++) f[3 * (size_t)o + c] += fa[3 * (size_t)a + c];
      if (eatom) eatom[o] += ea[a];
    }
    tri_owner.swap(own);
    tri_n = nn;
    return LMFF_OK;
  }

  int compute_device(int nn, const double *dx, const int *dtype, const int64_t *dmol, const int64_t *dtag, int which,
                     int eflag, int vflag, double *df, lmff_result *res) {
    int rc = ensure_atoms(nn);
    if (rc) return rc;
    CK(cudaMemcpyAsync(d_xin, dx, sizeof(double) * 3 * nn, cudaMemcpyDeviceToDevice, stream));
    bool reload = !loaded || nn != n || !built;
    if (!(which & LMFF_SAME_ATOMS) || reload) {
      CK(cudaMemcpyAsync(d_tin, dtype, sizeof(int) * nn, cudaMemcpyDeviceToDevice, stream));
      if (dmol) CK(cudaMemcpyAsync(d_min, dmol, sizeof(int64_t) * nn, cudaMemcpyDeviceToDevice, stream));
      else CK(cudaMemsetAsync(d_min, 0, sizeof(int64_t) * nn, stream));
      if (dtag) CK(cudaMemcpyAsync(d_gin, dtag, sizeof(int64_t) * nn, cudaMemcpyDeviceToDevice, stream));
      else {
        std::vector<int64_t> t(nn);
        for (int p = 0; p < nn; p++) t[p] = p + 1;
        CK(cudaMemcpyAsync(d_gin, t.data(), sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
      }
      if (!reload && nn > 0) {
        k_check_ident<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d_tin, d_min, d_gin, d.xq, d.tag, d.status);
        int flag = 0;
        CK(cudaMemcpyAsync(&flag, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
        CK(cudaStreamSynchronize(stream));
        if (flag) reload = true;
      }
    }
    rc = apply_positions(nn, reload);
    if (rc) return rc;
    std::vector<lmff_result> hr;
    rc = forces(which, eflag || vflag, false, &hr);
    if (rc) return rc;
    if (res) *res = hr.empty() ? lmff_result() : hr[0];
    if (nn > 0 && df) {
      k_scatter_add<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, d.f, df, (which & LMFF_OVERWRITE) != 0);
      CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(stream));
    return LMFF_OK;
  }

  // Per-atom virial of the last evaluation (lmff_compute_vatom): the FP64 pass of
  // launch_vatom on that evaluation's lists and positions, in either precision mode,
  // added into out[6 nn] in the caller's atom order.
  int vatom(int which, int nn, double *out) {
    if (tri && tri_n >= 0) {   // the last evaluation was a triclinic lmff_compute: fold the images
      if (nn != tri_n) return fail(LMFF_EINVAL, "lmff_compute_vatom: natoms is not the atom count of the last evaluation");
      std::vector<double> va(6 * (size_t)n, 0.0);
      tri_n = -1;   // the inner call evaluates the n = owned + image atoms
      int rc = vatom((which & (LMFF_TERSOFF | LMFF_ILP)) | LMFF_OVERWRITE, n, va.data());
      tri_n = nn;
      if (rc) return rc;
      if (which & LMFF_OVERWRITE) memset(out, 0, sizeof(double) * 6 * (size_t)nn);
      for (int a = 0; a < n; a++)
        for (int c = 0; c < 6; c++) out[6 * (size_t)tri_owner[a] + c] += va[6 * (size_t)a + c];
      return LMFF_OK;
    }
    if (nn != n) return fail(LMFF_EINVAL, "lmff_compute_vatom: natoms is not the atom count of the last evaluation");
    if (hsys.size() > 1) return fail(LMFF_EUNSUPPORTED, "lmff_compute_vatom: batches are not supported");
    if (n == 0) return LMFF_OK;
    if (va_cap < cap_n) {
      if (d_va) cudaFree(d_va);
      d_va = nullptr;
      va_cap = 0;
      CK(cudaMalloc(&d_va, sizeof(double) * VA_DOUBLES * (size_t)cap_n));
      va_cap = cap_n;
    }
    ForceArgs<double> a = args<double>();
    a.do_ters = t_on && (which & LMFF_TERSOFF);
    a.do_ilp = i_on && (which & LMFF_ILP);
    const size_t c6 = 6 * (size_t)va_cap;
    a.va_t = d_va;
    a.va_i = d_va + c6;
    a.va_ts = d_va + 2 * c6;
    a.va_is = a.va_ts + MAXTERS * c6;
    double *sorted = a.va_is + MAXILP * c6;
    double *inorder = sorted + c6;
    a.va_tens = reinterpret_cast<float4 *>(inorder + c6);   // 16-byte aligned: 912 B per atom before it
    // the interlayer shares in the precision of the evaluation: FP64, or the mixed
    // engines' FP32 pair form with FP64 sums
    const bool mixed_ilp = precision == LMFF_MIXED && a.do_ilp;
    f64::launch_vatom_terms(a, !mixed_ilp, stream);
    if (mixed_ilp) {
      ForceArgs<float> b = args<float>();
      b.do_ters = a.do_ters;
      b.do_ilp = a.do_ilp;
      b.va_t = a.va_t;
      b.va_i = a.va_i;
      b.va_ts = a.va_ts;
      b.va_is = a.va_is;
      b.va_tens = a.va_tens;
      f32::launch_vatom_ilp(b, stream);
    }
    f64::launch_vatom_gather(a, sorted, stream);
    CK(cudaGetLastError());
    const bool overwrite = (which & LMFF_OVERWRITE) != 0;
    if (!overwrite) CK(cudaMemcpyAsync(inorder, out, sizeof(double) * 6 * (size_t)nn, cudaMemcpyHostToDevice, stream));
    k_scatter_add6<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d.perm, sorted, inorder, overwrite);
    CK(cudaMemcpyAsync(out, inorder, sizeof(double) * 6 * (size_t)nn, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return LMFF_OK;
  }

  int upload(int nn, const double *x, const double *v, const int *type, const int64_t *mol, const int64_t *tag,
             const double *mass) {
    int rc = ensure_atoms(nn);
    if (rc) return rc;
    rc = check_mol(nn, mol, type);
    if (rc) return rc;
    mass_type.assign(MAXTYPE + 1, 1.0);
    if (mass)
      for (int t = 0; t < ntypes; t++) mass_type[t] = mass[t];
    if (!d_massT) CK(cudaMalloc(&d_massT, sizeof(double) * (MAXTYPE + 1)));
    CK(cudaMemcpyAsync(d_massT, mass_type.data(), sizeof(double) * (MAXTYPE + 1), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_xin, x, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, stream));
    if (v) CK(cudaMemcpyAsync(d_vin, v, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tin, type, sizeof(int) * nn, cudaMemcpyHostToDevice, stream));
    if (mol) CK(cudaMemcpyAsync(d_min, mol, sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
    else CK(cudaMemsetAsync(d_min, 0, sizeof(int64_t) * nn, stream));
    std::vector<int64_t> t;
    if (!tag) {
      t.resize(nn);
      for (int p = 0; p < nn; p++) t[p] = p + 1;
      tag = t.data();
    }
    CK(cudaMemcpyAsync(d_gin, tag, sizeof(int64_t) * nn, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    batch_offsets.clear();
    rc = set_single_box();
    if (rc) return rc;
    return load_from_staging(nn, v != nullptr, false);
  }

  // ---------------------------------------------------------------- step graph
  // One velocity-Verlet step as a CUDA graph: k_nve1 (whose last block sets the rebuild
  // condition) -> IF(rebuild) -> forces -> k_nve2, replayed with no host synchronisation
  // between steps.  Kernel
  // arguments are frozen at capture, so the graph's rebuild permutes into the spare
  // arrays and copies back, and the pair list keeps the capacity it had at capture
  // (an overflow raises ST_LIST_OVERFLOW; the chunk is then redone on the eager path
  // from a checkpoint of its first step, equal to the uninterrupted run up to the
  // summation order of a list built at a different step).
  // With a check interval ck > 1 there are three graphs: a check step, a step between
  // checks, and ck steps from a check step on (one launch, one conditional node).
  bool use_graphs = true;
  cudaGraphExec_t step_exec = nullptr, between_exec = nullptr, block_exec = nullptr;
  cudaStream_t cap_stream = nullptr;
  struct StepKey {
    int n, prec, tpa, block, full, ck;
    double dt, skin;
    const void *list, *xq;
    int64_t cap;
    bool operator==(const StepKey &o) const { return memcmp(this, &o, sizeof o) == 0; }
  } step_key;
  // chunk-start checkpoint for the overflow redo
  d4 *bk_xq = nullptr;
  double *bk_v = nullptr, *bk_f = nullptr, *bk_mass = nullptr;
  int64_t *bk_tag = nullptr;
  int *bk_perm = nullptr, *bk_sysid = nullptr;
  int bk_cap = 0;
  int64_t graph_steps = 0, graph_redos = 0;
  unsigned long long *d_graph_rebuilds = nullptr;
  unsigned *d_cond_ticket = nullptr;   // k_nve1's block count for the rebuild condition
  int64_t graph_cap = 0;           // pair-list capacity the step graph's rebuild fills up to
  int64_t graph_cap_limit = 0;     // > 0: lower it to this (exercises the overflow redo)

  cudaError_t enqueue_rebuild_fixed(cudaStream_t s) {
    nb_wrap_bin(n, d.xq, d.sys, d.sysid, d.bin_key, d.idx, s);
    cudaError_t e = nb_sort(d.cub_tmp, d.cub_tmp_bytes, d.bin_key, d.bin_key2, d.idx, d.idx2, n, (int)nbit_bins, s);
    if (e != cudaSuccess) return e;
    nb_permute(n, d.idx2, d.xq, xq2, d.v, v2, d.tag, tag2, d.perm, perm2, d.sysid, sysid2, d.mass, mass2, s);
    copy_back_permuted(s);
    cudaMemsetAsync(d.bin_start, 0, sizeof(int) * d.nbins, s);
    cudaMemsetAsync(d.bin_end, 0, sizeof(int) * d.nbins, s);
    cudaMemsetAsync(d.rowocc, 0, sizeof(int) * d.nbins, s);
    nb_bin_ranges(n, d.bin_key2, d.bin_start, d.bin_end, s, d.sys, d.sysid, d.rowocc);
    hilo_all(s);
    NbArgs a;
    memset(&a, 0, sizeof a);
    a.n = n;
    a.no_small = !small_variants;
    a.xq = d.xq;
    a.xh = d.xh;
    a.xl = d.xl;
    a.sys = d.sys;
    a.sysid = d.sysid;
    a.bin_start = d.bin_start;
    a.bin_end = d.bin_end;
    a.rowocc = d.rowocc;
    a.nbins = d.nbins;
    a.bin_key = d.bin_key2;
    a.list_off = d.list_off;
    a.list = d.list;
    a.list_cap = graph_cap;
    a.cnt = d.cnt_tmp;
    a.short_cnt = d.short_cnt;
    a.short_nb = d.short_nb;
    a.img = d.list_img;
    a.lc = lc;
    a.full = list_full;
    a.status = d.status;
    // single pass when the scratch holds the current stride (an atom outgrowing it
    // raises the list-overflow status: the chunk is redone host-driven, which grows it)
    const bool strided = stride > 0 && d.list_tmp && (int64_t)n * stride <= d.tmp_cap;
    a.tmp = d.list_tmp;
    a.stride = strided ? stride : 0;
    a.nin = d.nin_tmp;
    a.maxcnt = nullptr;
    cudaMemsetAsync(d.cnt_tmp + n, 0, sizeof(int64_t), s);
    nb_list(a, strided ? 2 : 0, s);
    e = nb_scan(d.cub_tmp, d.cub_tmp_bytes, d.cnt_tmp, d.list_off, n, s);
    if (e != cudaSuccess) return e;
    k_clamp_off<<<(n + 256) / 256, 256, 0, s>>>(n, d.list_off, graph_cap, d.status, d_graph_rebuilds);
    if (strided) nb_compact(a, graph_cap, s);
    else nb_list(a, 1, s);
    nb_copy_hold(n, d.xq, d.xhold, s);
    cudaMemsetAsync(d.maxdisp, 0, sizeof(unsigned long long), s);
    return cudaGetLastError();
  }

  void drop_graph() {
    if (step_exec) cudaGraphExecDestroy(step_exec);
    if (between_exec) cudaGraphExecDestroy(between_exec);
    if (block_exec) cudaGraphExecDestroy(block_exec);
    step_exec = between_exec = block_exec = nullptr;
    drop_fgraph();
  }

  // One force evaluation's device work (the kernels of run_kernels and the reduction)
  // as a CUDA graph, replayed while its arguments and launch shapes stay the same:
  // repeated single points, batch re-evaluations, the LAMMPS styles' per-step calls.
  cudaGraphExec_t fexec = nullptr;
  std::vector<unsigned char> fkey;
  void drop_fgraph() {
    if (fexec) cudaGraphExecDestroy(fexec);
    fexec = nullptr;
    fkey.clear();
  }
  template <class T>
  static void key_put(std::vector<unsigned char> &k, const T &v) {
    const unsigned char *b = reinterpret_cast<const unsigned char *>(&v);
    k.insert(k.end(), b, b + sizeof(T));
  }
  std::vector<unsigned char> force_key(int which, bool ev, bool eatom) {
    std::vector<unsigned char> k;
    if (precision == LMFF_FP64) key_put(k, args<double>());
    else key_put(k, args<float>());
    const int ints[] = {precision, which, (int)ev, (int)eatom, tpa, block, (int)ters_concurrent, (int)hsys.size()};
    key_put(k, ints);
    const void *ptrs[] = {d_arrs, d.sys, d.red_out, stat_ilp, stat_ters, eatom_ters};
    key_put(k, ptrs);
    return k;
  }

  // NVE steps: the gather kernel applies the second half-kick (k_nve2's arithmetic)
  KickArgs kick_args{};
  bool kick_on = false;
  void set_kick(double dtf, double dt = 0.0) {
    kick_args.v = d.v;
    DtfmTab t = dtfm_table(dtf);
    for (int k = 0; k <= MAXTYPE; k++) kick_args.dtfm[k] = t.v[k];
    kick_args.drift = 0;
    kick_args.do_hilo = precision == LMFF_MIXED;
    kick_args.dtv = dt;
    kick_args.trig2 = 0.25 * skin * skin;
    kick_args.xq = d.xq;
    kick_args.xhold = d.xhold;
    kick_args.xh = d.xh;
    kick_args.xl = d.xl;
    kick_args.sys = d.sys;
    kick_args.sysid = d.sysid;
    kick_args.status = d.status;
  }

  DtfmTab dtfm_table(double dtf) const {
    DtfmTab t;
    for (int k = 0; k <= MAXTYPE; k++) {
      double m = (k >= 1 && (size_t)(k - 1) < mass_type.size()) ? mass_type[k - 1] : 1.0;
      t.v[k] = dtf / m;
    }
    return t;
  }

  int build_step_graph(double dt) {
    drop_graph();
    if (!cap_stream) CK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    if (ters_concurrent) {
      int rc2 = ensure_stream2();   // before the capture begins
      if (rc2) return rc2;
    }
    if (!d_graph_rebuilds) {
      CK(cudaMalloc(&d_graph_rebuilds, sizeof(unsigned long long)));
      CK(cudaMemsetAsync(d_graph_rebuilds, 0, sizeof(unsigned long long), stream));
    }
    if (!d_cond_ticket) {
      CK(cudaMalloc(&d_cond_ticket, sizeof(unsigned)));
      CK(cudaMemsetAsync(d_cond_ticket, 0, sizeof(unsigned), stream));
    }
    int prc = push_consts();
    if (prc) return prc;
    if (!built) {
      prc = rebuild();
      if (prc) return prc;
    }
    // headroom so that a rebuild inside the graph rarely outgrows the list
    int64_t want = list_total + list_total / 4 + 4096;
    if (want > d.list_cap) {
      // grow the list and carry the current entries over (no rebuild: the trajectory
      // stays the one the host-driven loop would produce)
      uint32_t *nl = nullptr;
      cudaError_t e = cudaMalloc(&nl, sizeof(uint32_t) * want);
      if (e != cudaSuccess) return fail(LMFF_ENOMEM, "pair list headroom for the step graph does not fit on the device");
      if (list_total > 0) CK(cudaMemcpyAsync(nl, d.list, sizeof(uint32_t) * list_total, cudaMemcpyDeviceToDevice, stream));
      CK(cudaStreamSynchronize(stream));
      if (d.list) cudaFree(d.list);
      d.list = nl;
      d.list_cap = want;
    }
    graph_cap = d.list_cap;
    if (graph_cap_limit > 0 && graph_cap_limit < graph_cap) graph_cap = graph_cap_limit;
    const double dtf = 0.5 * dt * FTM2V;
    bool kt = ktiming;
    ktiming = false;
    set_kick(dtf, dt);   // the graph's rebuild copies back, so d.v stays fixed
    kick_on = true;
    int rc = capture_steps(dt, dtf, 1, true, &step_exec);
    if (!rc && ck > 1) rc = capture_steps(dt, dtf, 1, false, &between_exec);
    if (!rc && ck > 1) rc = capture_steps(dt, dtf, ck, true, &block_exec);
    ktiming = kt;
    kick_on = false;
    if (rc) {
      drop_graph();
      return rc;
    }
    memset(&step_key, 0, sizeof step_key);
    step_key = StepKey{n, precision, tpa, block, list_full, ck, dt, skin, d.list, d.xq, d.list_cap};
    return LMFF_OK;
  }

  // Captures nsteps NVE steps into one graph: the first a check step (its rebuild test
  // sets the condition of an IF node holding the rebuild) when check, the others steps
  // between checks, whose first half the previous step's gather makes (no k_nve1).
  int capture_steps(double dt, double dtf, int nsteps, bool check, cudaGraphExec_t *out) {
    const bool mixed = precision == LMFF_MIXED;
    const double trig2 = 0.25 * skin * skin;
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h = 0;
    if (check) CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    CK(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    for (int s = 0; s < nsteps; s++) {
      const bool chk = check && s == 0;
      if (s == 0)
        k_nve1<<<(n + per_atom_block(n) - 1) / per_atom_block(n), per_atom_block(n), 0, stream>>>(n, d.xq, d.v, d.f, dtfm_table(dtf), dt, d.xhold, d.maxdisp, d.sys,
                                                    d.sysid, d.xh, d.xl, mixed ? 1 : 0, h, trig2,
                                                    chk ? d_cond_ticket : nullptr, lookahead_for(chk, true, dt));
      kick_args.drift = s + 1 < nsteps;
      if (chk) {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        CK(cudaStreamGetCaptureInfo(stream, &cs, nullptr, nullptr, &deps, nullptr, &nd));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        CK(cudaGraphAddNode(&cn, g, deps, nullptr, nd, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        cudaError_t eb = enqueue_rebuild_fixed(cap_stream);
        CK(cudaStreamEndCapture(cap_stream, &body));
        if (eb != cudaSuccess) return cuda_fail(eb, "capturing the rebuild body");
        CK(cudaStreamUpdateCaptureDependencies(stream, &cn, nullptr, 1, cudaStreamSetCaptureDependencies));
      }
      pdl_short = s > 0;   // k_short follows the previous step's gather kernel
      if (precision == LMFF_FP64)
        run_kernels(args<double>(), LMFF_TERSOFF | LMFF_ILP, false, false, f64::launch_short, f64::launch_tersoff,
                    f64::launch_ilp, f64::launch_nframe, f64::launch_nderiv, f64::launch_finish);
      else
        run_kernels(args<float>(), LMFF_TERSOFF | LMFF_ILP, false, false, f32::launch_short, f32::launch_tersoff,
                    f32::launch_ilp, f32::launch_nframe, f32::launch_nderiv, f32::launch_finish);
      pdl_short = false;
    }
    kick_args.drift = 0;
    cudaGraph_t gout = nullptr;
    CK(cudaStreamEndCapture(stream, &gout));
    cudaError_t ei = cudaGraphInstantiate(out, gout, 0);
    cudaGraphDestroy(gout);
    if (ei != cudaSuccess) {
      *out = nullptr;
      return cuda_fail(ei, "cudaGraphInstantiate(step graph)");
    }
    return LMFF_OK;
  }

  int checkpoint(bool restore) {
    if (!restore && bk_cap < cap_n) {
      CK(dalloc(bk_xq, cap_n)); CK(dalloc(bk_v, 3 * (size_t)cap_n)); CK(dalloc(bk_f, 3 * (size_t)cap_n));
      CK(dalloc(bk_mass, cap_n)); CK(dalloc(bk_tag, cap_n)); CK(dalloc(bk_perm, cap_n)); CK(dalloc(bk_sysid, cap_n));
      bk_cap = cap_n;
    }
    auto cp = [&](void *dst, const void *src, size_t b) { return cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, stream); };
    if (!restore) {
      CK(cp(bk_xq, d.xq, sizeof(d4) * n)); CK(cp(bk_v, d.v, sizeof(double) * 3 * n)); CK(cp(bk_f, d.f, sizeof(double) * 3 * n));
      CK(cp(bk_mass, d.mass, sizeof(double) * n)); CK(cp(bk_tag, d.tag, sizeof(int64_t) * n));
      CK(cp(bk_perm, d.perm, sizeof(int) * n)); CK(cp(bk_sysid, d.sysid, sizeof(int) * n));
    } else {
      CK(cp(d.xq, bk_xq, sizeof(d4) * n)); CK(cp(d.v, bk_v, sizeof(double) * 3 * n)); CK(cp(d.f, bk_f, sizeof(double) * 3 * n));
      CK(cp(d.mass, bk_mass, sizeof(double) * n)); CK(cp(d.tag, bk_tag, sizeof(int64_t) * n));
      CK(cp(d.perm, bk_perm, sizeof(int) * n)); CK(cp(d.sysid, bk_sysid, sizeof(int) * n));
    }
    return LMFF_OK;
  }

  // nsteps NVE steps through the step graph; falls back to the eager loop on overflow
  int run_steps_graph(int nsteps, double dt) {
    StepKey want;
    memset(&want, 0, sizeof want);
    want = StepKey{n, precision, tpa, block, list_full, ck, dt, skin, d.list, d.xq, d.list_cap};
    if (!step_exec || !(step_key == want)) {
      int rc = build_step_graph(dt);
      if (rc) return rc;
    }
    int rc = checkpoint(false);
    if (rc) return rc;
    int64_t s = steps;
    for (int left = nsteps; left > 0;) {
      if (ck > 1 && s % ck == 0 && left >= ck) {
        CK(cudaGraphLaunch(block_exec, stream));
        s += ck;
        left -= ck;
      } else {
        CK(cudaGraphLaunch(check_step(s) ? step_exec : between_exec, stream));
        s++;
        left--;
      }
    }
    int st = 0;
    unsigned long long nrb = 0;
    CK(cudaMemcpyAsync(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(&nrb, d_graph_rebuilds, sizeof nrb, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemsetAsync(d_graph_rebuilds, 0, sizeof nrb, stream));
    CK(cudaStreamSynchronize(stream));
    hilo_fresh = precision == LMFF_MIXED;
    if (st & (ST_LIST_OVERFLOW | ST_SHORT_OVERFLOW | ST_SKIN_TRIP)) {
      // redo the chunk on the eager path, which grows the list as needed and rebuilds at
      // any step an atom moved more than skin/2
      CK(cudaMemsetAsync(d.status, 0, sizeof(int), stream));
      rc = checkpoint(true);
      if (rc) return rc;
      drop_graph();
      // the graph's rebuild reordered atoms and overwrote the list: build both again
      // for the restored positions, and the forces in that order (the checkpointed
      // forces are in the chunk-start order)
      built = false;
      rc = rebuild();
      if (rc) return rc;
      rc = forces(LMFF_TERSOFF | LMFF_ILP, false, false, nullptr);
      if (rc) return rc;
      graph_redos++;
      return run_steps_eager(nsteps, dt);
    }
    if (st) return status_error(st);
    rebuilds += (int64_t)nrb;
    graph_steps += nsteps;
    steps += nsteps;
    return LMFF_OK;
  }

  int run_steps_eager(int nsteps, double dt) {
    double dtf = 0.5 * dt * FTM2V;
    for (int s = 1; s <= nsteps; s++) {
      bool mixed = precision == LMFF_MIXED;
      const bool chk = check_step(steps);
      timed(4, [&] {
        k_nve1<<<(n + per_atom_block(n) - 1) / per_atom_block(n), per_atom_block(n), 0, stream>>>(n, d.xq, d.v, d.f, dtfm_table(dtf), dt, d.xhold, d.maxdisp, d.sys,
                                                    d.sysid, d.xh, d.xl, mixed ? 1 : 0, 0, 0.0, nullptr,
                                                    lookahead_for(chk, false, dt));
      });
      CK(cudaGetLastError());
      hilo_fresh = mixed;
      int rc = maybe_rebuild(chk && ck > 1);
      if (rc) return rc;
      set_kick(dtf);   // after any rebuild: it may have moved d.v
      kick_on = true;
      rc = forces(LMFF_TERSOFF | LMFF_ILP, false, false, nullptr);
      kick_on = false;
      if (rc) return rc;
      steps++;
    }
    return LMFF_OK;
  }

  int run_nve(int nsteps, double dt, int thermo_every, lmff_thermo *thermo) {
    if (!loaded) return fail(LMFF_EINVAL, "no resident system: call lmff_upload first");
    double dtf = 0.5 * dt * FTM2V, dtv = dt;
    int rc;
    std::vector<lmff_result> hr;
    int nth = 0;
    auto sample = [&](int64_t step, const std::vector<lmff_result> &r) -> int {
      double kes = 0.0;
      if (n > 0) {
        k_reduce<<<1, 256, 0, stream>>>(n, 1, (const double *const *)d_karrs, d.sys, d_kout);
        CK(cudaMemcpyAsync(&kes, d_kout, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
      }
      if (thermo) {
        lmff_thermo &t = thermo[nth];
        memset(&t, 0, sizeof t);
        t.step = step;
        t.ke = kes;
        t.pe = r.empty() ? 0.0 : r[0].e_tersoff + r[0].e_ilp;
        t.etotal = t.pe + t.ke;
        int dof = 3 * n - 3;
        t.temp = dof > 0 ? 2.0 * kes / (dof * BOLTZ) : 0.0;
        if (!r.empty())
          for (int k = 0; k < 6; k++) t.virial[k] = r[0].virial_tersoff[k] + r[0].virial_ilp[k];
      }
      nth++;
      return LMFF_OK;
    };
    if (!forces_valid) {
      rc = forces(LMFF_TERSOFF | LMFF_ILP, thermo_every > 0, false, &hr);
      if (rc) return rc;
      if (thermo_every > 0) {
        k_nve2<<<(n + 255) / 256, 256, 0, stream>>>(n, d.v, d.f, d.xq, d.mass, dtfm_table(0.0), ke);
        rc = sample(steps, hr);
        if (rc) return rc;
      }
    } else if (thermo_every > 0) {
      rc = forces(LMFF_TERSOFF | LMFF_ILP, true, false, &hr);
      if (rc) return rc;
      k_nve2<<<(n + 255) / 256, 256, 0, stream>>>(n, d.v, d.f, d.xq, d.mass, dtfm_table(0.0), ke);
      rc = sample(steps, hr);
      if (rc) return rc;
    }
    rc = choose_check_every(dt);
    if (rc) return rc;
    cudaEvent_t r0, r1;
    cudaEventCreate(&r0);
    cudaEventCreate(&r1);
    cudaEventRecord(r0, stream);
    // steps between thermo samples go through the step graph (or the eager loop when
    // per-kernel timing is on); a thermo step runs eagerly with energies and virial
    const bool graphs = use_graphs && !ktiming && n > 0;
    int done = 0;
    while (done < nsteps) {
      int chunk = nsteps - done;
      bool th_at_end = false;
      if (thermo_every > 0) {
        int to_next = thermo_every - done % thermo_every;
        if (to_next <= chunk) {
          chunk = to_next;
          th_at_end = true;
        }
      }
      int plain = th_at_end ? chunk - 1 : chunk;
      if (plain > 0) {
        rc = graphs ? run_steps_graph(plain, dt) : run_steps_eager(plain, dt);
        if (rc) return rc;
      }
      if (th_at_end) {
        bool mixed = precision == LMFF_MIXED;
        const bool chk = check_step(steps);
        k_nve1<<<(n + per_atom_block(n) - 1) / per_atom_block(n), per_atom_block(n), 0, stream>>>(n, d.xq, d.v, d.f, dtfm_table(dtf), dtv, d.xhold, d.maxdisp, d.sys,
                                                    d.sysid, d.xh, d.xl, mixed ? 1 : 0, 0, 0.0, nullptr,
                                                    lookahead_for(chk, false, dt));
        CK(cudaGetLastError());
        hilo_fresh = mixed;
        rc = maybe_rebuild(chk && ck > 1);
        if (rc) return rc;
        rc = forces(LMFF_TERSOFF | LMFF_ILP, true, false, &hr);
        if (rc) return rc;
        k_nve2<<<(n + 255) / 256, 256, 0, stream>>>(n, d.v, d.f, d.xq, d.mass, dtfm_table(dtf), ke);
        CK(cudaGetLastError());
        steps++;
        rc = sample(steps, hr);
        if (rc) return rc;
      }
      done += chunk;
    }
    cudaEventRecord(r1, stream);
    CK(cudaStreamSynchronize(stream));
    harvest();
    float ms = 0;
    cudaEventElapsedTime(&ms, r0, r1);
    cudaEventDestroy(r0);
    cudaEventDestroy(r1);
    ms_run = ms;
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- minimiser
  // min_style cg with the quadratic line search (the reference defaults: min_cg.cpp
  // iterate, min_linesearch.cpp linemin_quadratic / alpha_step, min.cpp setup / run /
  // energy_force / cleanup; dmax 0.1, norm two, no normalisation of thermo energies).
  double *m_x0 = nullptr, *m_g = nullptr, *m_h = nullptr, *m_part = nullptr;
  int *m_mask = nullptr;
  int m_cap = 0;
  bool m_masked = false;
  int m_nblk = 0;
  double m_red[MIN_NQ];

  int min_alloc() {
    if (m_cap < cap_n) {
      CK(dalloc(m_x0, 3 * (size_t)cap_n)); CK(dalloc(m_g, 3 * (size_t)cap_n)); CK(dalloc(m_h, 3 * (size_t)cap_n));
      CK(dalloc(m_mask, cap_n)); CK(dalloc(m_part, 1024 * MIN_NQ));
      m_cap = cap_n;
    }
    m_nblk = std::min(1024, std::max(1, (n + 255) / 256));
    return LMFF_OK;
  }

  // m_red = {f.f, f.g, f.h, g.h, max|h|, max|f|} over all atoms
  int min_dots() {
    k_min_dots<<<m_nblk, 256, 0, stream>>>(n, d.perm, d.f, m_g, m_h, m_part);
    CK(cudaGetLastError());
    std::vector<double> part((size_t)m_nblk * MIN_NQ);
    CK(cudaMemcpyAsync(part.data(), m_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    for (int k = 0; k < MIN_NQ; k++) m_red[k] = 0.0;
    for (int b = 0; b < m_nblk; b++)
      for (int k = 0; k < MIN_NQ; k++)
        m_red[k] = k < 4 ? m_red[k] + part[(size_t)b * MIN_NQ + k] : std::max(m_red[k], part[(size_t)b * MIN_NQ + k]);
    return LMFF_OK;
  }

  void min_vec(int mode, double beta) {
    k_min_vec<<<(n + 255) / 256, 256, 0, stream>>>(mode, n, d.perm, d.f, d.xq, m_g, m_h, m_x0, beta);
  }

  // Min::energy_force: rebuild if needed, forces and energy; with resetflag, the line
  // origin follows atoms that the rebuild wrapped across the box
  int min_energy(int resetflag, double &e) {
    int64_t rb = rebuilds;
    int rc = maybe_rebuild();
    if (rc) return rc;
    if (rebuilds != rb && resetflag) {
      k_min_reset<<<(n + 255) / 256, 256, 0, stream>>>(n, d.perm, d.xq, d.sys, d.sysid, m_x0);
      CK(cudaGetLastError());
    }
    std::vector<lmff_result> hr;
    rc = forces(LMFF_TERSOFF | LMFF_ILP, true, false, &hr);
    if (rc) return rc;
    if (m_masked) {
      k_min_mask<<<(n + 255) / 256, 256, 0, stream>>>(n, d.perm, m_mask, d.f);
      CK(cudaGetLastError());
    }
    e = 0.0;
    for (auto &r : hr) e += r.e_tersoff + r.e_ilp;
    return LMFF_OK;
  }

  // MinLineSearch::alpha_step
  int min_alpha_step(double alpha, int resetflag, int &neval, double &e) {
    k_min_step<<<(n + 255) / 256, 256, 0, stream>>>(n, d.perm, m_x0, m_h, alpha, d.xq, d.xhold, d.maxdisp);
    CK(cudaGetLastError());
    hilo_fresh = false;
    forces_valid = false;
    neval++;
    return min_energy(resetflag, e);
  }

  enum { MIN_MAXITER, MIN_MAXEVAL, MIN_ETOL, MIN_FTOL, MIN_DOWNHILL, MIN_ZEROALPHA, MIN_ZEROFORCE, MIN_ZEROQUAD };

  // MinLineSearch::linemin_quadratic; returns 0 or a stop condition
  int min_linemin(double eoriginal, double &ecurrent, double &alpha, int &neval, double dmax, int &err) {
    const double ALPHA_MAX = 1.0, ALPHA_REDUCE = 0.5, BACKTRACK_SLOPE = 0.4, QUADRATIC_TOL = 0.1, EMACH = 1.0e-8,
                 EPS_QUAD = 1.0e-28;
    err = min_dots();
    if (err) return 0;
    double fdothall = m_red[2];
    if (fdothall <= 0.0) return MIN_DOWNHILL;
    double hmaxall = m_red[4];
    if (hmaxall == 0.0) return MIN_ZEROFORCE;
    double alphamax = std::min(ALPHA_MAX, dmax / hmaxall);
    min_vec(3, 0.0);
    alpha = alphamax;
    double fhprev = fdothall, engprev = eoriginal, alphaprev = 0.0;
    for (;;) {
      err = min_alpha_step(alpha, 1, neval, ecurrent);
      if (err) return 0;
      err = min_dots();
      if (err) return 0;
      double fh = m_red[2];
      double delfh = fh - fhprev;
      if (fabs(fh) < EPS_QUAD || fabs(delfh) < EPS_QUAD) {
        err = min_alpha_step(0.0, 0, neval, ecurrent);
        return err ? 0 : MIN_ZEROQUAD;
      }
      double relerr = fabs(1.0 - (0.5 * (alpha - alphaprev) * (fh + fhprev) + ecurrent) / engprev);
      double alpha0 = alpha - (alpha - alphaprev) * fh / delfh;
      if (relerr <= QUADRATIC_TOL && alpha0 > 0.0 && alpha0 < alphamax) {
        err = min_alpha_step(alpha0, 1, neval, ecurrent);
        if (err) return 0;
        if (ecurrent - eoriginal < EMACH) return 0;
      }
      double de_ideal = -BACKTRACK_SLOPE * alpha * fdothall;
      double de = ecurrent - eoriginal;
      if (de <= de_ideal) return 0;
      fhprev = fh;
      engprev = ecurrent;
      alphaprev = alpha;
      alpha *= ALPHA_REDUCE;
      if (alpha <= 0.0 || de_ideal >= -EMACH) {
        err = min_alpha_step(0.0, 0, neval, ecurrent);
        return err ? 0 : MIN_ZEROALPHA;
      }
    }
  }

  int minimize(double etol, double ftol, int maxiter, int maxeval, double dmax, const int *frozen,
               lmff_min_result *out) {
    if (!loaded) return fail(LMFF_EINVAL, "no resident system: call lmff_upload first");
    if (!(dmax > 0.0) || maxiter < 0 || maxeval < 0) return fail(LMFF_EINVAL, "minimize: bad tolerance or limit");
    memset(out, 0, sizeof *out);
    if (n == 0) return LMFF_OK;
    int rc = min_alloc();
    if (rc) return rc;
    m_masked = frozen != nullptr;
    if (m_masked) {
      std::vector<int> mk(n);
      for (int i = 0; i < n; i++) mk[i] = frozen[i] ? 0 : 1;
      CK(cudaMemcpyAsync(m_mask, mk.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream));
    }
    const double EPS_ENERGY = 1.0e-8;
    int neval = 0, niter = 0, err = 0;
    double ecurrent = 0.0, eprevious = 0.0, alpha_final = 0.0;
    // Min::setup
    forces_valid = false;
    rc = min_energy(0, ecurrent);
    if (rc) return rc;
    out->einitial = ecurrent;
    min_vec(0, 0.0);
    rc = min_dots();
    if (rc) return rc;
    out->fnorm2_init = std::sqrt(m_red[0]);
    out->fnorminf_init = m_red[5];
    // MinCG::iterate
    int64_t nlimit = std::min<int64_t>(INT32_MAX, 3 * (int64_t)n);
    double gg = m_red[0];
    int stop = MIN_MAXITER;
    for (int iter = 0; iter < maxiter; iter++) {
      niter++;
      eprevious = ecurrent;
      int fl = min_linemin(ecurrent, ecurrent, alpha_final, neval, dmax, err);
      if (err) return err;
      if (fl) {
        stop = fl;
        break;
      }
      if (neval >= maxeval) {
        stop = MIN_MAXEVAL;
        break;
      }
      if (fabs(ecurrent - eprevious) < etol * 0.5 * (fabs(ecurrent) + fabs(eprevious) + EPS_ENERGY)) {
        stop = MIN_ETOL;
        break;
      }
      rc = min_dots();
      if (rc) return rc;
      double ff = m_red[0], fg = m_red[1];
      if (ftol > 0.0 && ff < ftol * ftol) {
        stop = MIN_FTOL;
        break;
      }
      double beta = std::max(0.0, (ff - fg) / gg);
      if ((niter + 1) % nlimit == 0) beta = 0.0;
      gg = ff;
      min_vec(1, beta);
      rc = min_dots();
      if (rc) return rc;
      if (m_red[3] <= 0.0) min_vec(2, 0.0);
    }
    // Min::run: a final evaluation unless the iteration limit ended it; Min::cleanup
    if (stop != MIN_MAXITER) {
      rc = min_energy(0, ecurrent);
      if (rc) return rc;
    }
    rc = min_dots();
    if (rc) return rc;
    out->niter = niter;
    out->neval = neval;
    out->stop_condition = stop;
    out->efinal = ecurrent;
    out->fnorm2_final = std::sqrt(m_red[0]);
    out->fnorminf_final = m_red[5];
    out->alpha_final = alpha_final;
    return LMFF_OK;
  }

  int count_pairs() {
    if (!built || n == 0) {
      pairs_in_cut = 0;
      return LMFF_OK;
    }
    unsigned long long *dc = nullptr;
    CK(cudaMalloc(&dc, sizeof(unsigned long long)));
    CK(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), stream));
    k_count_pairs<<<(n + 127) / 128, 128, 0, stream>>>(n, d.xq, d.sys, d.sysid, d.list_off, d.list, lc,
                                                       cut_global * cut_global, dc);
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, dc, sizeof h, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    cudaFree(dc);
    pairs_in_cut = (int64_t)h;
    return LMFF_OK;
  }

  int download(double *x, double *v, double *f) {
    if (!loaded) return fail(LMFF_EINVAL, "no resident system");
    if (n == 0) return LMFF_OK;
    double *xo = d_xin, *vo = d_vin, *fo = d_fin;
    k_unpermute_state<<<(n + 255) / 256, 256, 0, stream>>>(n, d.perm, d.xq, d.v, d.f, xo, vo, fo);
    CK(cudaGetLastError());
    if (x) CK(cudaMemcpyAsync(x, xo, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream));
    if (v) CK(cudaMemcpyAsync(v, vo, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream));
    if (f) CK(cudaMemcpyAsync(f, fo, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return LMFF_OK;
  }

  // ---------------------------------------------------------------- batch
  std::vector<int> batch_offsets;

  int batch_set(int nsys, const lmff_system_desc *sys) {
    if (nsys < 1) return fail(LMFF_EINVAL, "empty batch");
    std::vector<std::array<double, 9>> boxes(nsys);
    int64_t total = 0;
    batch_offsets.assign(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
      for (int k = 0; k < 3; k++) {
        boxes[s][k] = sys[s].lo[k];
        boxes[s][3 + k] = sys[s].hi[k];
        boxes[s][6 + k] = sys[s].periodic[k];
      }
      batch_offsets[s] = (int)total;
      total += sys[s].natoms;
    }
    batch_offsets[nsys] = (int)total;
    if (total > (1LL << 30)) return fail(LMFF_EINVAL, "batch too large");
    int nn = (int)total;
    int rc = make_sys(hsys, boxes);
    if (rc) return rc;
    rc = upload_sys();
    if (rc) return rc;
    rc = ensure_atoms(nn);
    if (rc) return rc;
    bool have_v = false;
    for (int s = 0; s < nsys; s++) have_v = have_v || sys[s].v;
    // one pinned staging block, reused across calls: x | v | mol | type | offsets; tags
    // and system ids are generated on the device
    CK(cudaStreamSynchronize(stream));   // the previous batch's copies out of the block are done
    const size_t bx = sizeof(double) * 3 * (size_t)nn, bm = sizeof(int64_t) * (size_t)nn,
                 bt = sizeof(int) * (size_t)nn, bo = sizeof(int) * (size_t)(nsys + 1);
    rc = ensure_pinned(2 * bx + bm + bt + bo);
    if (rc) return rc;
    char *hp = reinterpret_cast<char *>(h_pinned);
    double *hx = reinterpret_cast<double *>(hp), *hv = reinterpret_cast<double *>(hp + bx);
    int64_t *hm = reinterpret_cast<int64_t *>(hp + 2 * bx);
    int *ht = reinterpret_cast<int *>(hp + 2 * bx + bm), *hoff = reinterpret_cast<int *>(hp + 2 * bx + bm + bt);
    // the systems' arrays into the block, by several host threads for a large batch
    std::atomic<int> first_bad{nsys};
    auto stage = [&](int s0, int s1) {
      for (int s = s0; s < s1; s++) {
        const int o = batch_offsets[s], ns = sys[s].natoms;
        if (!ids_ok(ns, sys[s].mol, sys[s].type)) {
          int cur = first_bad.load();
          while (s < cur && !first_bad.compare_exchange_weak(cur, s)) {}
          continue;
        }
        memcpy(hx + 3 * (size_t)o, sys[s].x, sizeof(double) * 3 * ns);
        if (have_v) {
          if (sys[s].v) memcpy(hv + 3 * (size_t)o, sys[s].v, sizeof(double) * 3 * ns);
          else memset(hv + 3 * (size_t)o, 0, sizeof(double) * 3 * ns);
        }
        memcpy(ht + o, sys[s].type, sizeof(int) * ns);
        if (sys[s].mol) memcpy(hm + o, sys[s].mol, sizeof(int64_t) * ns);
        else memset(hm + o, 0, sizeof(int64_t) * ns);
      }
    };
    const int nth = nn >= (1 << 17) ? (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency())) : 1;
    if (nth > 1 && nsys > 1) {
      // contiguous system ranges of about equal atom counts
      std::vector<std::thread> pool;
      int s0 = 0;
      for (int k = 0; k < nth && s0 < nsys; k++) {
        const int64_t goal = (int64_t)nn * (k + 1) / nth;
        int s1 = s0;
        while (s1 < nsys && (k == nth - 1 || batch_offsets[s1 + 1] <= goal || s1 == s0)) s1++;
        pool.emplace_back(stage, s0, s1);
        s0 = s1;
      }
      for (auto &t : pool) t.join();
    } else {
      stage(0, nsys);
    }
    if (first_bad.load() < nsys) {
      const int b = first_bad.load();
      return check_mol(sys[b].natoms, sys[b].mol, sys[b].type);   // sets the message
    }
    for (int s = 0; s <= nsys; s++) hoff[s] = batch_offsets[s];
    if (nsys + 1 > boff_cap) {
      if (d_boff) cudaFree(d_boff);
      d_boff = nullptr;
      CK(cudaMalloc(&d_boff, sizeof(int) * (size_t)(nsys + 1)));
      boff_cap = nsys + 1;
    }
    CK(cudaMemcpyAsync(d_xin, hx, bx, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tin, ht, bt, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_min, hm, bm, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_boff, hoff, bo, cudaMemcpyHostToDevice, stream));
    if (have_v) CK(cudaMemcpyAsync(d_vin, hv, bx, cudaMemcpyHostToDevice, stream));
    if (nn) k_batch_ids<<<(nn + 255) / 256, 256, 0, stream>>>(nn, d_boff, nsys, d_gin, d_sysin);
    if (!mass_type.empty()) {
      if (!d_massT) CK(cudaMalloc(&d_massT, sizeof(double) * (MAXTYPE + 1)));
      CK(cudaMemcpyAsync(d_massT, mass_type.data(), sizeof(double) * mass_type.size(), cudaMemcpyHostToDevice, stream));
    }
    CK(cudaStreamSynchronize(stream));
    return load_from_staging(nn, have_v, true);
  }

  int batch_compute(double *f_out, lmff_result *res) {
    if (!loaded) return fail(LMFF_EINVAL, "no batch loaded");
    std::vector<lmff_result> hr;
    int rc = forces(LMFF_TERSOFF | LMFF_ILP, true, false, &hr);
    if (rc) return rc;
    for (size_t s = 0; s < hr.size() && res; s++) res[s] = hr[s];
    if (f_out && n > 0) {
      k_scatter_add<<<(n + 255) / 256, 256, 0, stream>>>(n, d.perm, d.f, d_fin, 1);
      const size_t bf = sizeof(double) * 3 * (size_t)n;
      if (n >= (1 << 17) && ensure_pinned(bf) == LMFF_OK) {
        // a large batch comes back through the pinned staging block (a pageable copy is
        // staged by the CUDA runtime at a fraction of the link's rate), then into the caller's
        // array on several host threads
        CK(cudaMemcpyAsync(h_pinned, d_fin, bf, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        parallel_copy(f_out, h_pinned, bf);
        return LMFF_OK;
      }
      CK(cudaMemcpyAsync(f_out, d_fin, bf, cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaStreamSynchronize(stream));
    return LMFF_OK;
  }

  // memcpy on up to 8 host threads, in 64-byte aligned pieces
  static void parallel_copy(void *dst, const void *src, size_t bytes) {
    const int nth = (int)std::min<size_t>(8, std::max(1u, std::thread::hardware_concurrency()));
    if (nth <= 1 || bytes < ((size_t)4 << 20)) {
      memcpy(dst, src, bytes);
      return;
    }
    const size_t piece = ((bytes / nth) + 63) & ~(size_t)63;
    std::vector<std::thread> pool;
    for (int k = 0; k < nth; k++) {
      const size_t b = (size_t)k * piece;
      if (b >= bytes) break;
      const size_t e = std::min(bytes, b + piece);
      pool.emplace_back([=] { memcpy((char *)dst + b, (const char *)src + b, e - b); });
    }
    for (auto &t : pool) t.join();
  }

  // ---------------------------------------------------------------- lists export
  int64_t export_list(int which, int64_t *out, int64_t cap) {
    if (!built) return fail(LMFF_EINVAL, "no neighbour list built");
    std::vector<int64_t> tag(n);
    std::vector<int> perm(n);
    cudaMemcpyAsync(tag.data(), d.tag, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, stream);
    std::vector<int64_t> off(n + 1);
    std::vector<uint32_t> ent;
    std::vector<int> cnt;
    if (which == 0) {
      cudaMemcpyAsync(off.data(), d.list_off, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, stream);
      cudaStreamSynchronize(stream);
      ent.resize(off[n]);
      cudaMemcpyAsync(ent.data(), d.list, sizeof(uint32_t) * off[n], cudaMemcpyDeviceToHost, stream);
    } else {
      cnt.resize(n);
      ent.resize((size_t)n * MAXILP);
      cudaMemcpyAsync(cnt.data(), d.ilp_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, stream);
      cudaMemcpyAsync(ent.data(), d.ilp_nb, sizeof(uint32_t) * n * MAXILP, cudaMemcpyDeviceToHost, stream);
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return fail(LMFF_ECUDA, "list export failed");
    int64_t m = 0;
    for (int i = 0; i < n; i++) {
      int64_t b = which == 0 ? off[i] : (int64_t)i * MAXILP;
      int64_t e = which == 0 ? off[i + 1] : b + cnt[i];
      for (int64_t k = b; k < e; k++) {
        int j, sx, sy, sz;
        decode_entry(ent[k], lc, j, sx, sy, sz);
        if (out && m < cap) {
          out[3 * m] = tag[i];
          out[3 * m + 1] = tag[j];
          out[3 * m + 2] = ((int64_t)((sx + 8) & 15)) | ((int64_t)((sy + 8) & 15) << 4) | ((int64_t)((sz + 8) & 15) << 8);
        }
        m++;
      }
    }
    return m;
  }
};

// =========================================================== allocation-free call
// lmff_compute_device_noalloc: the force evaluation of one small system for callers
// that may not allocate device memory once they are running -- for example an
// application that reserves all GPU memory up front for its own pool, or code that
// must not call cudaMalloc where an allocation would synchronise the device or is
// forbidden.  Every buffer the kernels need beyond the caller's inputs and outputs
// comes from one file-scope device array, g_noalloc_scratch, of NOALLOC_BYTES.  The
// array is part of the module image: every GPU that loads this library holds it until
// the process exits.  All calls share it and it keeps the last call's contents, so
// calls that overlap on the GPU (two streams, two host threads, two engine handles)
// race and must be serialised by the caller.

constexpr size_t NOALLOC_BYTES = (size_t)16 << 20;   // 16 MiB
constexpr int NOALLOC_MAX_ATOMS = 2048;
constexpr int NOALLOC_MAX_BINS = 8192;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of g_noalloc_scratch, looked up once per device with that device
// current (in host code the symbol name is only a stand-in, never a device address).
static std::mutex g_noalloc_mu;
static void *g_noalloc_base[64] = {nullptr};

static int noalloc_base(int device, void **base, std::string &err) {
  if (device < 0 || device >= 64) {
    err = "device ordinal out of range";
    return LMFF_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_base[device]) {
    void *ptr = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (rc != cudaSuccess || !ptr) {
      err = std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(rc);
      return LMFF_ECUDA;
    }
    g_noalloc_base[device] = ptr;
  }
  *base = g_noalloc_base[device];
  return LMFF_OK;
}

// bump carving of the scratch array, 256-byte aligned pieces
struct Carve {
  unsigned char *p, *end;
  template <class T>
  T *take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
    if (p + bytes > end) return nullptr;
    T *r = (T *)p;
    p += bytes;
    return r;
  }
};

int noalloc_compute(Engine &g, int nn, const double *dx, const int *dtype, const int64_t *dmol, int which, int eflag,
                    int vflag, double *df, lmff_result *res) {
  if (nn < 0 || nn > NOALLOC_MAX_ATOMS)
    return g.fail(LMFF_EINVAL, "lmff_compute_device_noalloc: natoms must be in 0.." +
                                   std::to_string(NOALLOC_MAX_ATOMS) + " (got " + std::to_string(nn) + ")");
  if (!g.have_box) return g.fail(LMFF_EINVAL, "lmff_set_box must be called first");
  if (nn == 0) {   // an empty subdomain: no force, zero energies and virials (as lmff_compute_device)
    if (res) memset(res, 0, sizeof *res);
    return LMFF_OK;
  }
  void *basev = nullptr;
  int rc = noalloc_base(g.device, &basev, g.err);
  if (rc) return rc;
  rc = g.push_consts();
  if (rc) return rc;
  cudaStream_t st = g.stream;
  // geometry of the one system (same binning rules as the resident path)
  SysDesc sd;
  memset(&sd, 0, sizeof sd);
  int R = 0;
  {
    double L[3] = {g.bhi[0] - g.blo[0], g.bhi[1] - g.blo[1], g.bhi[2] - g.blo[2]};
    sys_geometry(sd, g.blo, L, g.bper, g.cutneigh_max, R);
  }
  sd.atom_begin = 0;
  sd.atom_end = nn;
  long long nbins = (long long)sd.nb[0] * sd.nb[1] * sd.nb[2];
  if (nbins > NOALLOC_MAX_BINS)
    return g.fail(LMFF_EINVAL, "lmff_compute_device_noalloc: box needs " + std::to_string(nbins) +
                                   " bins, more than the limit of " + std::to_string(NOALLOC_MAX_BINS));
  ListCode lc;
  lc.R = R;
  lc.w = 1;
  while ((1 << lc.w) < 2 * R + 1) lc.w++;
  lc.ibits = 32 - 3 * lc.w;
  lc.imask = (1u << lc.ibits) - 1u;
  lc.wmask = (1u << lc.w) - 1u;
  if ((int64_t)nn >= (1LL << lc.ibits))
    return g.fail(LMFF_EOVERFLOW, "too many atoms for the 32-bit neighbour-list code of this box");
  int nbits = 1;
  while ((1LL << nbits) < nbins) nbits++;
  // carve the scratch array
  const int c = NOALLOC_MAX_ATOMS;
  Carve cv{(unsigned char *)basev, (unsigned char *)basev + NOALLOC_BYTES};
  d4 *xq = cv.take<d4>(c), *xq2 = cv.take<d4>(c), *nrm64 = cv.take<d4>(c), *ilp_g = cv.take<d4>(c);
  float4 *xh = cv.take<float4>(c), *xl = cv.take<float4>(c), *nrm32 = cv.take<float4>(c);
  float4 *jrec = cv.take<float4>(3 * (size_t)c), *jrec2 = cv.take<float4>(2 * (size_t)c);
  double *v = cv.take<double>(3 * c), *v2 = cv.take<double>(3 * c), *mass = cv.take<double>(c),
         *mass2 = cv.take<double>(c);
  int64_t *tag = cv.take<int64_t>(c), *tag2 = cv.take<int64_t>(c);
  int *perm = cv.take<int>(c), *perm2 = cv.take<int>(c), *sysid = cv.take<int>(c), *sysid2 = cv.take<int>(c);
  int *ilp_cnt = cv.take<int>(c), *ters_cnt = cv.take<int>(c), *short_cnt = cv.take<int>(c);
  uint32_t *ilp_nb = cv.take<uint32_t>((size_t)c * MAXILP), *ters_nb = cv.take<uint32_t>((size_t)c * MAXTERS);
  uint32_t *short_nb = cv.take<uint32_t>((size_t)c * MAXSHORT);
  uint8_t *list_img = cv.take<uint8_t>(c);
  d4 *ters_g = cv.take<d4>((size_t)c * MAXTERS), *ilp_c = cv.take<d4>((size_t)c * MAXILP);
  double *ters_f = cv.take<double>(3 * c), *ilp_f = cv.take<double>(3 * c), *fs = cv.take<double>(3 * c);
  double *stat_ilp = cv.take<double>(8 * c), *stat_ters = cv.take<double>(8 * c);
  double *eat_i = cv.take<double>(c), *eat_t = cv.take<double>(c);
  int64_t *list_off = cv.take<int64_t>(c + 1), *cnt = cv.take<int64_t>(c + 1);
  uint32_t *key = cv.take<uint32_t>(c), *key2 = cv.take<uint32_t>(c);
  int *idx = cv.take<int>(c), *idx2 = cv.take<int>(c);
  int *bin_start = cv.take<int>(NOALLOC_MAX_BINS), *bin_end = cv.take<int>(NOALLOC_MAX_BINS);
  SysDesc *dsys = cv.take<SysDesc>(1);
  double *red = cv.take<double>(16);
  double **arrs = cv.take<double *>(2);
  int *status = cv.take<int>(1);
  size_t tmp_bytes = nb_sort_tmp_bytes(c, 32);
  void *tmp = cv.take<unsigned char>(tmp_bytes);
  if (!tmp) return g.fail(LMFF_EOVERFLOW, "lmff_compute_device_noalloc: scratch layout does not fit");
  size_t list_cap = (size_t)(cv.end - cv.p) / sizeof(uint32_t);
  uint32_t *list = cv.take<uint32_t>(list_cap);
  // what must start at zero: status word, bin ranges, the count past the last atom
  const double *host_arrs[2] = {stat_ilp, stat_ters};
  CK2(cudaMemsetAsync(status, 0, sizeof(int), st));
  CK2(cudaMemsetAsync(bin_start, 0, sizeof(int) * nbins, st));
  CK2(cudaMemsetAsync(bin_end, 0, sizeof(int) * nbins, st));
  CK2(cudaMemsetAsync(cnt + nn, 0, sizeof(int64_t), st));
  CK2(cudaMemcpyAsync(dsys, &sd, sizeof sd, cudaMemcpyHostToDevice, st));
  CK2(cudaMemcpyAsync(arrs, host_arrs, sizeof host_arrs, cudaMemcpyHostToDevice, st));
  int gb = (nn + 255) / 256;
  k_load<<<gb, 256, 0, st>>>(nn, dx, dtype, dmol, nullptr, nullptr, nullptr, nullptr, xq, tag, perm, sysid, v, mass);
  nb_wrap_bin(nn, xq, dsys, sysid, key, idx, st);
  CK2(nb_sort(tmp, tmp_bytes, key, key2, idx, idx2, nn, nbits, st));
  nb_permute(nn, idx2, xq, xq2, v, v2, tag, tag2, perm, perm2, sysid, sysid2, mass, mass2, st);
  nb_bin_ranges(nn, key2, bin_start, bin_end, st);
  nb_hilo(nn, xq2, dsys, sysid2, xh, xl, st);
  NbArgs na;
  memset(&na, 0, sizeof na);
  na.n = nn;
  na.xq = xq2;
  na.xh = xh;
  na.xl = xl;
  na.sys = dsys;
  na.sysid = sysid2;
  na.bin_start = bin_start;
  na.bin_end = bin_end;
  na.nbins = nbins;
  na.bin_key = key2;
  na.list_off = list_off;
  na.list = list;
  na.list_cap = (int64_t)list_cap;
  na.cnt = cnt;
  na.short_cnt = short_cnt;
  na.short_nb = short_nb;
  na.img = list_img;
  na.lc = lc;
  na.full = g.list_full;
  na.status = status;
  nb_list(na, 0, st);
  CK2(nb_scan(tmp, tmp_bytes, cnt, list_off, nn, st));
  int64_t total = 0;
  CK2(cudaMemcpyAsync(&total, list_off + nn, sizeof total, cudaMemcpyDeviceToHost, st));
  CK2(cudaStreamSynchronize(st));
  if (total < 0 || (size_t)total > list_cap)
    return g.fail(LMFF_EOVERFLOW, "lmff_compute_device_noalloc: pair list of " + std::to_string(total) +
                                      " entries exceeds the scratch capacity of " + std::to_string(list_cap));
  nb_list(na, 1, st);
  auto fill = [&](auto &a) {
    memset(&a, 0, sizeof a);
    a.A.xq = xq2;
    a.A.xh = xh;
    a.A.xl = xl;
    a.A.jrec = jrec;
    a.A.jrec2 = jrec2;
    a.A.sys = dsys;
    a.A.sysid = sysid2;
    a.lc = lc;
    a.n = nn;
    a.tag = tag2;
    a.list_off = list_off;
    a.list = list;
    a.list_img = list_img;
    a.short_cnt = short_cnt;
    a.short_nb = short_nb;
    a.ilp_cnt = ilp_cnt;
    a.ilp_nb = ilp_nb;
    a.ters_cnt = ters_cnt;
    a.ters_nb = ters_nb;
    a.nrm64 = nrm64;
    a.nrm32 = nrm32;
    a.jrec = jrec;
    a.jrec2 = jrec2;
    a.ters_g = ters_g;
    a.ters_f = ters_f;
    a.ilp_f = ilp_f;
    a.ilp_c = ilp_c;
    a.ilp_g = ilp_g;
    a.stat_ilp = stat_ilp;
    a.stat_ters = stat_ters;
    a.eatom_ilp = eat_i;
    a.eatom_ters = eat_t;
    a.f_out = fs;
    a.status = status;
    a.do_ters = g.t_on && (which & LMFF_TERSOFF);
    a.do_ilp = g.i_on && (which & LMFF_ILP);
    a.list_full = g.list_full;
    a.kc = g.i_on && g.hi.model == LMFF_INTERLAYER_KC;
  };
  const bool ev = true;
  if (g.precision == LMFF_FP64) {
    ForceArgs<double> a;
    fill(a);
    f64::launch_short(a, g.d_cutILPsq, g.ht.cutmax * g.ht.cutmax, st);
    if (a.do_ters) f64::launch_tersoff(a, ev, false, st);
    else CK2(cudaMemsetAsync(stat_ters, 0, sizeof(double) * 8 * (size_t)nn, st));
    if (a.do_ilp) {
      f64::launch_ilp(a, ev, false, g.tpa, g.block, g.i_one, st);
      f64::launch_nderiv(a, ev, st);
    } else {
      CK2(cudaMemsetAsync(stat_ilp, 0, sizeof(double) * 8 * (size_t)nn, st));
    }
    f64::launch_finish(a, false, nullptr, st);
  } else {
    ForceArgs<float> a;
    fill(a);
    f32::launch_short(a, g.d_cutILPsq, g.ht.cutmax * g.ht.cutmax, st);
    if (a.do_ters) f32::launch_tersoff(a, ev, false, st);
    else CK2(cudaMemsetAsync(stat_ters, 0, sizeof(double) * 8 * (size_t)nn, st));
    if (a.do_ilp) {
      f32::launch_ilp(a, ev, false, g.tpa, g.block, g.i_one, st);
      f32::launch_nderiv(a, ev, st);
    } else {
      CK2(cudaMemsetAsync(stat_ilp, 0, sizeof(double) * 8 * (size_t)nn, st));
    }
    f32::launch_finish(a, false, nullptr, st);
  }
  k_reduce<<<16, 256, 0, st>>>(nn, 16, (const double *const *)arrs, dsys, red);
  k_scatter_add<<<gb, 256, 0, st>>>(nn, perm2, fs, df, 1);
  CK2(cudaGetLastError());
  double hred[16];
  int hst = 0;
  CK2(cudaMemcpyAsync(hred, red, sizeof hred, cudaMemcpyDeviceToHost, st));
  CK2(cudaMemcpyAsync(&hst, status, sizeof hst, cudaMemcpyDeviceToHost, st));
  CK2(cudaStreamSynchronize(st));
  if (hst & ST_TOO_MANY_ILP)
    return g.fail(LMFF_ETOO_MANY_ILP_NEIGH, "There are too many neighbors for some atoms, please check your configuration");
  if (hst & ST_ZERO_NORMAL) return g.fail(LMFF_EZERO_NORMAL, "The magnitude of the normal vector is zero");
  if (hst) return g.fail(LMFF_EOVERFLOW, "lmff_compute_device_noalloc: neighbour capacity exceeded");
  if (res) {
    memset(res, 0, sizeof *res);
    if (eflag || vflag) {
      res->pvector[0] = hred[0];
      res->pvector[1] = hred[1];
      res->e_ilp = hred[0] + hred[1];
      for (int k = 0; k < 6; k++) res->virial_ilp[k] = hred[2 + k];
      res->e_tersoff = hred[8];
      for (int k = 0; k < 6; k++) res->virial_tersoff[k] = hred[10 + k];
    }
  }
  return LMFF_OK;
}

}  // namespace lmff

using lmff::Engine;

// One API call on an engine: holds the device lock in shared mode and makes sure the
// device's constant tables are this engine's (uploading them under the exclusive lock
// when another engine's tables are resident).
struct DeviceCall {
  std::shared_lock<std::shared_mutex> lk;
  explicit DeviceCall(Engine &g) {
    g.calls++;
    int dev = (g.device >= 0 && g.device < 64) ? g.device : 0;
    cudaSetDevice(g.device);
    for (int attempt = 0;; attempt++) {
      lk = std::shared_lock<std::shared_mutex>(lmff::g_dev_rw[dev]);
      if (lmff::g_dev_tables[dev] == g.table_hash || attempt == 3) break;  // 3 failed uploads: the call reports the CUDA error
      lk.unlock();
      std::unique_lock<std::shared_mutex> ex(lmff::g_dev_rw[dev]);
      if (lmff::g_dev_tables[dev] != g.table_hash) {
        cudaDeviceSynchronize();
        if (g.upload_tables() == LMFF_OK) lmff::g_dev_tables[dev] = g.table_hash;
      }
    }
  }
};

// ====================================================================== C ABI

struct lmff_engine {
  Engine e;
};

static thread_local std::string g_create_error;

extern "C" {

int lmff_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int lmff_create(lmff_engine **out, const lmff_params *p, int device) {
  if (!out) return LMFF_EINVAL;
  *out = nullptr;
  lmff_engine *h = new (std::nothrow) lmff_engine;
  if (!h) return LMFF_ENOMEM;
  int rc = h->e.set_params(p);
  if (rc == LMFF_OK) rc = h->e.init_device(device);
  if (rc != LMFF_OK) {
    g_create_error = h->e.err;
    delete h;
    return rc;
  }
  *out = h;
  return LMFF_OK;
}

int lmff_create_from_files(lmff_engine **out, const char *tersoff_file, const char *ilp_file, int ntypes,
                           const char *const *elements, double cut_global, int tap_flag, double skin, int device) {
  return lmff_create_from_files2(out, tersoff_file, elements, ilp_file, elements, ntypes, cut_global, tap_flag, skin,
                                 device);
}

int lmff_create_kc_from_files(lmff_engine **out, const char *tersoff_file, const char *const *tersoff_elements,
                              const char *kc_file, const char *const *kc_elements, int ntypes, double cut_global,
                              int tap_flag, double skin, int device) {
  if (!out || ntypes < 1 || ntypes > lmff::MAXTYPE || !kc_file || !kc_elements) return LMFF_EINVAL;
  if (tersoff_file && !tersoff_elements) return LMFF_EINVAL;
  *out = nullptr;
  lmff::HostTersoff ht;
  lmff::HostIlp hk;
  std::string err;
  if (tersoff_file && !lmff::parse_tersoff(tersoff_file, ntypes, tersoff_elements, ht, err)) {
    g_create_error = err;
    return LMFF_EBADPARAM;
  }
  if (!lmff::parse_kc(kc_file, ntypes, kc_elements, hk, err)) {
    g_create_error = err;
    return LMFF_EBADPARAM;
  }
  lmff_params p;
  memset(&p, 0, sizeof p);
  p.ntypes = ntypes;
  if (tersoff_file) {
    p.tersoff_nelements = (int)ht.elements.size();
    p.tersoff_nparams = (int)ht.params.size();
    p.tersoff_params = ht.params.data();
    p.tersoff_elem2param = ht.elem2param.data();
    p.tersoff_map = ht.map.data();
    p.tersoff_cutmax = ht.cutmax;
  }
  p.ilp_nelements = (int)hk.elements.size();
  p.ilp_nparams = (int)hk.kc.size();
  p.ilp_elem2param = hk.elem2param.data();
  p.ilp_map = hk.map.data();
  p.ilp_cutILPsq = hk.cutILPsq.data();
  p.interlayer_model = LMFF_INTERLAYER_KC;
  p.kc_params = hk.kc.data();
  p.ilp_cut_global = cut_global;
  p.ilp_tap_flag = tap_flag;
  p.skin = skin;
  return lmff_create(out, &p, device);
}

int lmff_create_from_files2(lmff_engine **out, const char *tersoff_file, const char *const *tersoff_elements,
                            const char *ilp_file, const char *const *ilp_elements, int ntypes, double cut_global,
                            int tap_flag, double skin, int device) {
  if (!out || ntypes < 1 || ntypes > lmff::MAXTYPE) return LMFF_EINVAL;
  if ((tersoff_file && !tersoff_elements) || (ilp_file && !ilp_elements)) return LMFF_EINVAL;
  *out = nullptr;
  lmff::HostTersoff ht;
  lmff::HostIlp hi;
  std::string err;
  if (tersoff_file && !lmff::parse_tersoff(tersoff_file, ntypes, tersoff_elements, ht, err)) {
    g_create_error = err;
    return LMFF_EBADPARAM;
  }
  if (ilp_file && !lmff::parse_ilp(ilp_file, ntypes, ilp_elements, hi, err)) {
    g_create_error = err;
    return LMFF_EBADPARAM;
  }
  lmff_params p;
  memset(&p, 0, sizeof p);
  p.ntypes = ntypes;
  if (tersoff_file) {
    p.tersoff_nelements = (int)ht.elements.size();
    p.tersoff_nparams = (int)ht.params.size();
    p.tersoff_params = ht.params.data();
    p.tersoff_elem2param = ht.elem2param.data();
    p.tersoff_map = ht.map.data();
    p.tersoff_cutmax = ht.cutmax;
  }
  if (ilp_file) {
    p.ilp_nelements = (int)hi.elements.size();
    p.ilp_nparams = (int)hi.params.size();
    p.ilp_params = hi.params.data();
    p.ilp_elem2param = hi.elem2param.data();
    p.ilp_map = hi.map.data();
    p.ilp_cutILPsq = hi.cutILPsq.data();
  }
  p.ilp_cut_global = cut_global;
  p.ilp_tap_flag = tap_flag;
  p.skin = skin;
  return lmff_create(out, &p, device);
}

void lmff_destroy(lmff_engine *e) { delete e; }

int lmff_set_precision(lmff_engine *e, int mode) {
  if (!e || (mode != LMFF_FP64 && mode != LMFF_MIXED)) return LMFF_EINVAL;
  e->e.precision = mode;
  e->e.hilo_fresh = false;
  return LMFF_OK;
}

int lmff_set_box(lmff_engine *e, const double lo[3], const double hi[3], double xy, double xz, double yz,
                 const int periodic[3]) {
  if (!e || !lo || !hi || !periodic) return LMFF_EINVAL;
  if (!std::isfinite(xy) || !std::isfinite(xz) || !std::isfinite(yz)) return e->e.fail(LMFF_EINVAL, "non-finite tilt");
  if (xy != 0.0 || xz != 0.0 || yz != 0.0) {
    for (int k = 0; k < 3; k++)
      if (!(hi[k] > lo[k])) return e->e.fail(LMFF_EINVAL, "box hi must exceed lo");
    Engine &g = e->e;
    for (int k = 0; k < 3; k++) {
      g.tlo[k] = lo[k];
      g.thi[k] = hi[k];
      g.tper[k] = periodic[k] != 0;
    }
    g.tilt[0] = xy;
    g.tilt[1] = xz;
    g.tilt[2] = yz;
    g.tri = true;
    g.tri_n = -1;
    return LMFF_OK;
  }
  if (e->e.tri) {   // leaving a triclinic box (and the subdomain form it ran through)
    e->e.tri = false;
    e->e.tri_n = -1;
    e->e.have_box = false;
  }
  bool changed = false;
  for (int k = 0; k < 3; k++) {
    if (!(hi[k] > lo[k])) return e->e.fail(LMFF_EINVAL, "box hi must exceed lo");
    changed |= e->e.blo[k] != lo[k] || e->e.bhi[k] != hi[k] || e->e.bper[k] != (periodic[k] != 0);
    e->e.blo[k] = lo[k];
    e->e.bhi[k] = hi[k];
    e->e.bper[k] = periodic[k] != 0;
  }
  e->e.have_box = true;
  if (e->e.ghost_nlocal >= 0) {   // leaving subdomain mode
    e->e.ghost_nlocal = -1;
    changed = true;
  }
  if (changed) {
    e->e.built = false;
    e->e.loaded = false;
  }
  return LMFF_OK;
}

// calls that evaluate the periodic-system form refuse an engine left in subdomain mode,
// and every call but lmff_compute a triclinic box
static int refuse_ghost_mode(lmff_engine *e) {
  if (e->e.tri)
    return e->e.fail(LMFF_EUNSUPPORTED, "triclinic boxes: only lmff_compute and lmff_compute_vatom evaluate them");
  if (e->e.ghost_nlocal < 0) return LMFF_OK;
  return e->e.fail(LMFF_EINVAL, "the engine is in subdomain mode (lmff_compute_ghost): call lmff_set_box to leave it");
}

int lmff_set_option(lmff_engine *e, const char *key, double value) {
  if (!e || !key) return LMFF_EINVAL;
  std::string k(key);
  if (k == "tpa") {
    int v = (int)value;
    if (v != 4 && v != 8 && v != 16 && v != 32) return e->e.fail(LMFF_EINVAL, "tpa must be 4, 8, 16 or 32");
    e->e.tpa = v;
  } else if (k == "block") {
    int v = (int)value;
    if (v < 32 || v > 256 || (v & 31)) return e->e.fail(LMFF_EINVAL, "block must be a multiple of 32 in 32..256");
    e->e.block = v;
  } else if (k == "list_full") {
    e->e.list_full = value != 0.0;
    e->e.built = false;
  } else if (k == "skin") {
    if (!(value >= 0.0)) return e->e.fail(LMFF_EINVAL, "skin must be >= 0");
    e->e.skin = value;
    e->e.build_consts();
    e->e.loaded = false;
  } else if (k == "pair_tile") {
    const int v = (int)value;
    if (v != 1 && v != 2) return e->e.fail(LMFF_EINVAL, "pair_tile must be 1 or 2");
    e->e.pair_tile = v;
    e->e.drop_graph();
  } else if (k == "check_every") {
    if (!(value >= 0.0 && value <= 64.0)) return e->e.fail(LMFF_EINVAL, "check_every must be in 0..64");
    e->e.check_every_opt = (int)value;
    e->e.drop_graph();
  } else if (k == "small_variants") {
    e->e.small_variants = value != 0.0;
    e->e.drop_graph();
    e->e.built = false;
  } else if (k == "pdl") {
    if (!(value >= 0.0 && value < 32.0)) return e->e.fail(LMFF_EINVAL, "pdl must be a mask in 0..31");
    e->e.pdl_mask = (int)value;
    e->e.drop_graph();
  } else if (k == "ters_concurrent") {
    e->e.ters_concurrent = value != 0.0;
    e->e.drop_graph();
  } else if (k == "graphs") {
    e->e.use_graphs = value != 0.0;
    e->e.drop_graph();
  } else if (k == "graph_list_cap") {
    e->e.graph_cap_limit = value > 0 ? (int64_t)value : 0;
    e->e.drop_graph();
  } else if (k == "kernel_timing") {
    e->e.ktiming = value != 0.0;
  } else if (k == "reset_timing") {
    for (int q = 0; q < 7; q++) {
      e->e.kms[q] = 0.0;
      e->e.klaunch[q] = 0;
    }
  } else if (k == "count_pairs") {
    DeviceCall dc(e->e);
    return e->e.count_pairs();
  } else {
    return e->e.fail(LMFF_EINVAL, "unknown option " + k);
  }
  return LMFF_OK;
}

int lmff_compute(lmff_engine *e, int natoms, const double *x, const int *type, const int64_t *mol, const int64_t *tag,
                 int which, int eflag, int vflag, double *f, double *eatom, lmff_result *res) {
  if (!e || natoms < 0 || (natoms > 0 && (!x || !type))) return LMFF_EINVAL;
  if (e->e.tri) {
    DeviceCall dc(e->e);
    const int rc = e->e.compute_tri(natoms, x, type, mol, tag, which, eflag, vflag, f, eatom, res);
    if (rc == LMFF_OK) e->e.va_call = e->e.calls;
    return rc;
  }
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  const int rc = e->e.compute_host(natoms, x, type, mol, tag, which, eflag, vflag, f, eatom, res);
  if (rc == LMFF_OK) e->e.va_call = e->e.calls;
  return rc;
}

int lmff_compute_ghost(lmff_engine *e, int nlocal, int nall, const double *x, const int *type, const int64_t *mol,
                       const int64_t *tag, int which, int eflag, int vflag, double *f, double *eatom,
                       lmff_result *res) {
  if (!e || nlocal < 0 || nall < nlocal || (nall > 0 && (!x || !type || !tag))) return LMFF_EINVAL;
  if (e->e.tri) return e->e.fail(LMFF_EINVAL, "the engine has a triclinic box: call lmff_set_box with an orthogonal one first");
  DeviceCall dc(e->e);
  const int rc = e->e.compute_ghost(nlocal, nall, x, type, mol, tag, which, eflag, vflag, f, eatom, res);
  if (rc == LMFF_OK) e->e.va_call = e->e.calls;
  return rc;
}

int lmff_compute_device(lmff_engine *e, int natoms, const double *d_x, const int *d_type, const int64_t *d_mol,
                        const int64_t *d_tag, int which, int eflag, int vflag, double *d_f, lmff_result *res) {
  if (!e || natoms < 0 || (natoms > 0 && (!d_x || !d_type))) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  const int rc = e->e.compute_device(natoms, d_x, d_type, d_mol, d_tag, which, eflag, vflag, d_f, res);
  if (rc == LMFF_OK) e->e.va_call = e->e.calls;
  return rc;
}

int lmff_compute_device_noalloc(lmff_engine *e, int natoms, const double *d_x, const int *d_type,
                                const int64_t *d_mol, int which, int eflag, int vflag, double *d_f, lmff_result *res) {
  if (!e || natoms < 0 || (natoms > 0 && (!d_x || !d_type || !d_f))) return LMFF_EINVAL;
  if (natoms > 0 && !d_mol) return e->e.fail(LMFF_EINVAL, "lmff_compute_device_noalloc: d_mol is required");
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return lmff::noalloc_compute(e->e, natoms, d_x, d_type, d_mol, which, eflag, vflag, d_f, res);
}

int lmff_upload(lmff_engine *e, int natoms, const double *x, const double *v, const int *type, const int64_t *mol,
                const int64_t *tag, const double *mass) {
  if (!e || natoms < 0 || (natoms > 0 && (!x || !type))) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return e->e.upload(natoms, x, v, type, mol, tag, mass);
}

int lmff_compute_resident(lmff_engine *e, int which, int eflag, int vflag, lmff_result *res) {
  if (!e) return LMFF_EINVAL;
  if (!e->e.loaded) return e->e.fail(LMFF_EINVAL, "no resident system");
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  int rc = e->e.maybe_rebuild();
  if (rc) return rc;
  std::vector<lmff_result> hr;
  rc = e->e.forces(which, eflag || vflag, false, &hr);
  if (rc) return rc;
  if (res) *res = hr.empty() ? lmff_result() : hr[0];
  e->e.va_call = e->e.calls;
  return LMFF_OK;
}

int lmff_compute_vatom(lmff_engine *e, int which, int natoms, double *vatom) {
  if (!e || natoms < 0 || (natoms > 0 && !vatom)) return LMFF_EINVAL;
  if (e->e.va_call == 0 || e->e.va_call != e->e.calls)
    return e->e.fail(LMFF_EINVAL, "lmff_compute_vatom: must directly follow an evaluation on this engine");
  DeviceCall dc(e->e);
  const int rc = e->e.vatom(which, natoms, vatom);
  e->e.va_call = rc == LMFF_OK ? e->e.calls : 0;   // the two styles may be asked one after the other
  return rc;
}

int lmff_run_nve(lmff_engine *e, int nsteps, double dt, int thermo_every, lmff_thermo *thermo) {
  if (!e || nsteps < 0 || thermo_every < 0) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return e->e.run_nve(nsteps, dt, thermo_every, thermo);
}

int lmff_download(lmff_engine *e, double *x, double *v, double *f) {
  if (!e) return LMFF_EINVAL;
  DeviceCall dc(e->e);
  return e->e.download(x, v, f);
}

int lmff_batch_set(lmff_engine *e, int nsys, const lmff_system_desc *sys) {
  if (!e || !sys) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return e->e.batch_set(nsys, sys);
}

int lmff_batch_compute(lmff_engine *e, double *f_out, lmff_result *res) {
  if (!e) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return e->e.batch_compute(f_out, res);
}

int lmff_minimize(lmff_engine *e, double etol, double ftol, int maxiter, int maxeval, double dmax,
                  const int *frozen, lmff_min_result *out) {
  if (!e || !out) return LMFF_EINVAL;
  if (int rc = refuse_ghost_mode(e)) return rc;
  DeviceCall dc(e->e);
  return e->e.minimize(etol, ftol, maxiter, maxeval, dmax, frozen, out);
}

int lmff_batch_results(lmff_engine *e, int nsys, lmff_result *res) {
  if (!e || !res || nsys < 0) return LMFF_EINVAL;
  Engine &g = e->e;
  if (!g.last_res_valid) return g.fail(LMFF_EINVAL, "no energies computed since the last upload");
  if ((size_t)nsys != g.last_res.size())
    return g.fail(LMFF_EINVAL, "nsys does not match the resident batch (" + std::to_string(g.last_res.size()) + ")");
  for (int s = 0; s < nsys; s++) res[s] = g.last_res[s];
  return LMFF_OK;
}

int lmff_set_masses(lmff_engine *e, int ntypes, const double *mass) {
  if (!e || !mass || ntypes < 1 || ntypes > lmff::MAXTYPE) return LMFF_EINVAL;
  e->e.mass_type.assign(lmff::MAXTYPE + 1, 1.0);
  for (int t = 0; t < ntypes; t++) e->e.mass_type[t] = mass[t];
  e->e.drop_graph();   // a captured step holds dt/mass per type
  return LMFF_OK;
}

int lmff_clone(const lmff_engine *src, lmff_engine **out) {
  if (!src || !out) return LMFF_EINVAL;
  *out = nullptr;
  lmff_engine *h = new (std::nothrow) lmff_engine;
  if (!h) return LMFF_ENOMEM;
  int rc = h->e.clone_from(src->e);
  if (rc != LMFF_OK) {
    g_create_error = h->e.err;
    delete h;
    return rc;
  }
  *out = h;
  return LMFF_OK;
}

int lmff_get_stats(lmff_engine *e, lmff_stats *out) {
  if (!e || !out) return LMFF_EINVAL;
  memset(out, 0, sizeof *out);
  Engine &g = e->e;
  out->natoms = g.n;
  out->list_entries = g.list_total;
  out->list_capacity = g.d.list_cap;
  out->rebuilds = g.rebuilds;
  out->steps = g.steps;
  out->list_per_atom = g.n ? (double)g.list_total / g.n : 0.0;
  out->ms_last_build = g.ms_build;
  out->ms_last_forces = g.ms_forces;
  out->precision = g.precision;
  out->tpa = g.tpa;
  out->block = g.block;
  out->ms_last_run = g.ms_run;
  out->graph_steps = g.graph_steps;
  out->graph_redos = g.graph_redos;
  for (int q = 0; q < 7; q++) {
    out->kernel_ms[q] = g.kms[q];
    out->kernel_launches[q] = g.klaunch[q];
  }
  out->pairs_in_cutoff = g.pairs_in_cut;
  out->bytes_device = g.device_bytes();
  out->bytes_per_atom_need = g.bytes_per_atom_need();
  return LMFF_OK;
}

int64_t lmff_export_list(lmff_engine *e, int which, int64_t *out, int64_t cap) {
  if (!e) return LMFF_EINVAL;
  DeviceCall dc(e->e);
  return e->e.export_list(which, out, cap);
}

const char *lmff_last_error(const lmff_engine *e) {
  if (!e) return g_create_error.c_str();
  return e->e.err.c_str();
}

const char *lmff_strerror(int code) {
  switch (code) {
    case LMFF_OK: return "success";
    case LMFF_EINVAL: return "invalid argument";
    case LMFF_ECUDA: return "CUDA error";
    case LMFF_EOVERFLOW: return "neighbour list overflow";
    case LMFF_ETOO_MANY_ILP_NEIGH: return "There are too many neighbors for some atoms, please check your configuration";
    case LMFF_EZERO_NORMAL: return "The magnitude of the normal vector is zero";
    case LMFF_EBADPARAM: return "potential file or parameter error";
    case LMFF_ETIMEDOUT: return "device wait timed out";
    case LMFF_EUNSUPPORTED: return "unsupported request";
    case LMFF_ENOMEM: return "out of memory";
    case LMFF_ENODEV: return "no CUDA device";
    default: return "unknown error";
  }
}

}  // extern "C"
