// GPU neighbour build: cell binning, stable sort of atoms by bin, and the two lists
// the force kernels consume, built with skin like LAMMPS's binned full list
// (npair_full_bin_ghost.cpp:75-117, accept rsq <= cutneighsq; cutneigh = cutforce + skin,
// neighbor.cpp:294-317):
//   * the pair list: for the ILP pair kernel, every j within cutneigh with a different
//     molecule id (or, with list_full, every j: the reference's full list), stored as
//     32-bit (index, periodic image) codes in CSR form;
//   * the short candidate list: every j within max(ILP intralayer rcut, Tersoff
//     cutmax) + skin, from which each step picks the ILP intralayer and Tersoff lists.
// Periodic images are explicit image codes, never minimum image, so boxes shorter than
// the cutoff (several images of one atom, self images) are exact.
#include <climits>

#include <cub/cub.cuh>

#include "engine.cuh"
#include "neighbor.cuh"

namespace lmff {

__constant__ NbConst c_nb;

__device__ __forceinline__ int bin_coord(double x, double lo, double binv, int nb) {
  int b = (int)floor((x - lo) * binv);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

// Wrap periodic coordinates into the box (LAMMPS Domain::pbc at reneighbouring) and
// compute each atom's global bin.
__global__ void k_wrap_bin(int n, d4 *xq, const SysDesc *sys, const int *sysid, uint32_t *key, int *idx) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const SysDesc &sd = sys[sysid[p]];
  d4 q = xq[p];
  double c[3] = {q.x, q.y, q.z};
  int b[3];
  for (int d = 0; d < 3; d++) {
    if (sd.per[d]) {
      double hi = sd.lo[d] + sd.L[d];
      if (c[d] < sd.lo[d]) c[d] += sd.L[d] * ceil((sd.lo[d] - c[d]) / sd.L[d]);
      if (c[d] >= hi) c[d] -= sd.L[d] * floor((c[d] - sd.lo[d]) / sd.L[d]);
      if (c[d] < sd.lo[d] || c[d] >= hi) c[d] = sd.lo[d];
    }
    b[d] = bin_coord(c[d], sd.lo[d], sd.binv[d], sd.nb[d]);
  }
  xq[p] = make_d4(c[0], c[1], c[2], q.w);
  const uint32_t bin = (uint32_t)(sd.bin_begin + (b[2] * sd.nb[1] + b[1]) * sd.nb[0] + b[0]);
  const uint32_t molbits = (uint32_t)(__double_as_longlong(q.w) >> 8) & ((1u << KEY_MOL_BITS) - 1u);
  key[p] = (bin << KEY_MOL_BITS) | molbits;
  idx[p] = p;
}

__global__ void k_permute(int n, const int *idx2, const d4 *xq, d4 *xq2, const double *v, double *v2,
                          const int64_t *tag, int64_t *tag2, const int *perm, int *perm2, const int *sysid,
                          int *sysid2, const double *mass, double *mass2) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int o = idx2[q];
  xq2[q] = xq[o];
  v2[q] = v[o];
  v2[n + q] = v[n + o];
  v2[2 * n + q] = v[2 * n + o];
  tag2[q] = tag[o];
  perm2[q] = perm[o];
  sysid2[q] = sysid[o];
  mass2[q] = mass[o];
}

// Atom range of every occupied bin, and (rowocc) a flag at the first bin of every bin
// row that holds atoms: the list build skips empty rows of its stencil whole (a bilayer
// in a box with vacuum leaves most of them empty).
__global__ void k_bin_ranges(int n, const uint32_t *key, int *bin_start, int *bin_end, const SysDesc *sys,
                             const int *sysid, int *rowocc) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint32_t k = key[q] >> KEY_MOL_BITS;
  if (q == 0 || (key[q - 1] >> KEY_MOL_BITS) != k) {
    bin_start[k] = q;
    if (rowocc) {
      const SysDesc &sd = sys[sysid[q]];
      rowocc[k - (uint32_t)((int)k - sd.bin_begin) % (uint32_t)sd.nb[0]] = 1;
    }
  }
  if (q == n - 1 || (key[q + 1] >> KEY_MOL_BITS) != k) bin_end[k] = q + 1;
}

// double-float split of each position: X = x - lo + 32 + base lies in [base, 2 base) for
// every position within 32 A of the box (base = 2^ceil(log2(Lmax + 64))), so
// the hi parts of any two atoms of a system share one binade and their difference is
// exact in FP32; lo = X - hi carries the remaining bits.
__global__ void k_hilo(int n, const d4 *xq, const SysDesc *sys, const int *sysid, float4 *xh, float4 *xl) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const SysDesc &sd = sys[sysid[p]];
  d4 q = xq[p];
  double X = q.x - sd.lo[0] + 32.0 + sd.base;
  double Y = q.y - sd.lo[1] + 32.0 + sd.base;
  double Z = q.z - sd.lo[2] + 32.0 + sd.base;
  float hx = (float)X, hy = (float)Y, hz = (float)Z;
  int info = (int)__double_as_longlong(q.w);
  xh[p] = make_float4(hx, hy, hz, __int_as_float(info));
  xl[p] = make_float4((float)(X - (double)hx), (float)(Y - (double)hy), (float)(Z - (double)hz), 0.f);
}

__device__ __forceinline__ bool le_exact(float rsq, float thr, double thr64, const d4 *xq, const SysDesc &sd,
                                         int i, int j, int sx, int sy, int sz) {
  float m = 1e-5f * thr;
  if (rsq < thr - m) return true;
  if (rsq > thr + m) return false;
  d4 a = xq[i];
  d4 b = xq[j];
  double xj = sx ? __dadd_rn(b.x, sx * sd.L[0]) : b.x;
  double yj = sy ? __dadd_rn(b.y, sy * sd.L[1]) : b.y;
  double zj = sz ? __dadd_rn(b.z, sz * sd.L[2]) : b.z;
  double dx = __dsub_rn(a.x, xj), dy = __dsub_rn(a.y, yj), dz = __dsub_rn(a.z, zj);
  double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return r2 <= thr64;
}

// One warp per 32 consecutive atoms of the sorted order, one lane per atom.  Atoms are
// sorted by bin and bins are numbered x fastest, so the lanes of a warp almost always
// share one bin row (same system, y and z bin) and sit in one or two neighbouring x
// bins.  The warp walks the union of its lanes' stencils (the x range widened by the
// lanes' spread; a lane skips x bins outside its own stencil), staging each stencil
// bin's j atoms 32 at a time in warp-private shared memory; every lane then tests its i
// against them in order (a broadcast).  Lanes of another row (a warp that straddles a
// row boundary) are handled in a second pass.  No block-wide barrier is involved.
// The entries of each i come out in the order of a per-atom scan: stencil bins (dz, dy,
// dx), then j ascending.
// MODE 0: counts pair-list entries into cnt[i] and writes the short list.
// MODE 1: writes the pair list at list_off[i], candidates inside the force cutoff from
// the front and the skin shell from the back (the pair kernel's lanes then mostly accept
// or reject together).
// MODE 2: both in one pass over the candidates: counts, short list, and the entries in
// the same order into atom i's slice of the strided buffer, for nb_compact after the
// scan; an atom with more entries than the stride raises ST_STRIDE_OVERFLOW (with
// ST_LIST_OVERFLOW, so that a captured rebuild is redone) and the host falls back to
// MODE 1.
constexpr int LW = 4;   // warps per block

template <int MODE>
__global__ void __launch_bounds__(32 * LW) k_list(NbArgs a) {
  constexpr bool FILL = MODE != 0;
  const int wg = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int wl = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  if (wg * 32 >= a.n) return;                       // whole warps only
  __shared__ float4 th[LW][32], tl[LW][32];
  const int i = wg * 32 + lane;
  const bool act = i < a.n;
  int sys = -1, bx = 0, by = 0, bz = 0;
  float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
  if (act) {
    sys = a.sysid[i];
    const SysDesc &sd = a.sys[sys];
    const int lb = (int)(a.bin_key[i] >> KEY_MOL_BITS) - sd.bin_begin;
    bx = lb % sd.nb[0];
    by = (lb / sd.nb[0]) % sd.nb[1];
    bz = lb / (sd.nb[0] * sd.nb[1]);
    hi = a.xh[i];
    lo = a.xl[i];
  }
  const int infoi = __float_as_int(hi.w);
  const int ti = infoi & 255;
  const int mi = infoi >> 8;
  const int ilp_i = c_nb.ilp_mapped[ti];
  int nlong = 0, nin = 0, nsh = 0, nshort = 0;
  bool img = false;
  const int64_t base = !act ? 0 : MODE == 1 ? a.list_off[i] : MODE == 2 ? (int64_t)i * a.stride : 0;
  const int64_t lend = !act ? 0 : MODE == 1 ? a.list_off[i + 1] : MODE == 2 ? base + a.stride : 0;
  uint32_t *const dst = MODE == 2 ? a.tmp : a.list;
  const int64_t dcap = MODE == 2 ? (int64_t)a.n * a.stride : a.list_cap;
  unsigned todo = __ballot_sync(FULL, act);
  while (todo) {
    const int leader = __ffs(todo) - 1;
    const int rs = __shfl_sync(FULL, sys, leader);
    const int ry = __shfl_sync(FULL, by, leader);
    const int rz = __shfl_sync(FULL, bz, leader);
    const bool mine = ((todo >> lane) & 1u) && sys == rs && by == ry && bz == rz;
    todo &= ~__ballot_sync(FULL, mine);
    const int xmin = __reduce_min_sync(FULL, mine ? bx : INT_MAX);
    const int xmax = __reduce_max_sync(FULL, mine ? bx : INT_MIN);
    const SysDesc &sd = a.sys[rs];
    const float prefilt = sd.prefilt_sq;
    for (int dz = -sd.reach[2]; dz <= sd.reach[2]; dz++) {
      int jz = rz + dz, sz = 0;
      if (sd.per[2]) {
        sz = jz >= 0 ? jz / sd.nb[2] : -((-jz + sd.nb[2] - 1) / sd.nb[2]);
        jz -= sz * sd.nb[2];
      } else if (jz < 0 || jz >= sd.nb[2]) continue;
      for (int dy = -sd.reach[1]; dy <= sd.reach[1]; dy++) {
        int jy = ry + dy, sy = 0;
        if (sd.per[1]) {
          sy = jy >= 0 ? jy / sd.nb[1] : -((-jy + sd.nb[1] - 1) / sd.nb[1]);
          jy -= sy * sd.nb[1];
        } else if (jy < 0 || jy >= sd.nb[1]) continue;
        if (a.rowocc && !a.rowocc[sd.bin_begin + (jz * sd.nb[1] + jy) * sd.nb[0]]) continue;   // empty row
        for (int xu = xmin - sd.reach[0]; xu <= xmax + sd.reach[0]; xu++) {
          int jx = xu, sx = 0;
          if (sd.per[0]) {
            sx = jx >= 0 ? jx / sd.nb[0] : -((-jx + sd.nb[0] - 1) / sd.nb[0]);
            jx -= sx * sd.nb[0];
          } else if (jx < 0 || jx >= sd.nb[0]) continue;
          const bool use = mine && xu >= bx - sd.reach[0] && xu <= bx + sd.reach[0];
          if (!__any_sync(FULL, use)) continue;
          const int gbj = sd.bin_begin + (jz * sd.nb[1] + jy) * sd.nb[0] + jx;
          const int jstart = a.bin_start[gbj], jend = a.bin_end[gbj];
          const float shx = (float)sx * sd.Lhi[0], shy = (float)sy * sd.Lhi[1], shz = (float)sz * sd.Lhi[2];
          const float slx = (float)sx * sd.Llo[0], sly = (float)sy * sd.Llo[1], slz = (float)sz * sd.Llo[2];
          const bool self_image = (sx | sy | sz) == 0;
          // a tile whose candidates all share the molecule of every lane using this bin
          // holds no interlayer partner; beyond the adjacent bins it holds no short-list
          // candidate either (the short cutoff is below the bin size), so it is passed over
          const bool far_bin = !use || dz > 1 || dz < -1 || dy > 1 || dy < -1 || xu > bx + 1 || xu < bx - 1;
          const bool may_skip = !a.full && (MODE == 1 || __all_sync(FULL, far_bin));
          for (int jt0 = jstart, nj = 0; jt0 < jend; jt0 += nj) {
            nj = min(32, jend - jt0);
            __syncwarp();
            float4 hl = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < nj) {
              hl = a.xh[jt0 + lane];
              th[wl][lane] = hl;
              tl[wl][lane] = a.xl[jt0 + lane];
            }
            if (may_skip) {
              // the tile ends where the bin's run of its first candidate's molecule ends
              // (atoms are sorted by molecule within a bin)
              const int mt = __float_as_int(hl.w) >> 8;
              const int m0 = __shfl_sync(FULL, mt, 0);
              const unsigned chg = __ballot_sync(FULL, lane < nj && mt != m0);
              if (chg) nj = __ffs(chg) - 1;
              if (__all_sync(FULL, !use || m0 == mi)) continue;
            }
            __syncwarp();
            if (!use) continue;
            // the prefilter over the whole tile first, into a bit mask: a uniform loop, and
            // the candidates that pass are then taken in order by each lane on its own
            // (testing and accepting inside one loop would run the accepting path for the
            // warp whenever any of its lanes accepts; 2.7M-atom rebuild 39.4 -> 36.0 ms.
            // The prefilter in FP32x2 lanes, two candidates per iteration, measured slower:
            // 37.9 ms)
            unsigned pass = 0u;
            for (int jj = 0; jj < nj; jj++) {
              const float4 hj = th[wl][jj];
              const float hx = (hi.x - hj.x) - shx, hy = (hi.y - hj.y) - shy, hz = (hi.z - hj.z) - shz;
              pass |= (hx * hx + hy * hy + hz * hz > prefilt ? 0u : 1u) << jj;   // most candidates fail
            }
            while (pass) {
              const int jj = __ffs(pass) - 1;
              pass &= pass - 1u;
              const int j = jt0 + jj;
              const float4 hj = th[wl][jj];
              const float hx = (hi.x - hj.x) - shx, hy = (hi.y - hj.y) - shy, hz = (hi.z - hj.z) - shz;
              const float4 lj = tl[wl][jj];
              float ddx = hx + ((lo.x - lj.x) - slx);
              float ddy = hy + ((lo.y - lj.y) - sly);
              float ddz = hz + ((lo.z - lj.z) - slz);
              float rsq = ddx * ddx + ddy * ddy + ddz * ddz;
              const int infoj = __float_as_int(hj.w);
              const int tj = infoj & 255;
              const int mj = infoj >> 8;
              const int tt = ti * (MAXTYPE + 1) + tj;
              bool take_long = false;
              if ((a.full || (mj != mi && ilp_i && c_nb.ilp_mapped[tj])) && !(self_image && j == i))
                take_long = le_exact(rsq, c_nb.cutnsq_f[tt], c_nb.cutnsq_d[tt], a.xq, sd, i, j, sx, sy, sz);
              if (FILL && take_long) {
                const bool inner = rsq < c_nb.innersq_f;
                int64_t pos = inner ? base + nin : lend - 1 - nsh;
                if (pos >= base && pos < lend && pos < dcap) dst[pos] = encode_entry(j, sx, sy, sz, a.lc);
                nin += inner;
                nsh += !inner;
                img |= !self_image;
              }
              if (MODE != 1 && !(self_image && j == i) &&
                  le_exact(rsq, c_nb.rshortsq_f, c_nb.rshortsq_d, a.xq, sd, i, j, sx, sy, sz)) {
                if (nshort < MAXSHORT) a.short_nb[(size_t)i * MAXSHORT + nshort] = encode_entry(j, sx, sy, sz, a.lc);
                nshort++;
              }
              nlong += take_long;
            }
          }
        }
      }
    }
  }
  if (act) {
    if (MODE != 1) {
      a.cnt[i] = nlong;
      a.short_cnt[i] = nshort < MAXSHORT ? nshort : MAXSHORT;
      if (nshort > MAXSHORT) atomicOr(a.status, ST_SHORT_OVERFLOW);
    }
    if (MODE != 0) a.img[i] = img;
    if (MODE == 1 && base + nlong > a.list_cap) atomicOr(a.status, ST_LIST_OVERFLOW);
    if (MODE == 2) {
      a.nin[i] = nin;
      if (nlong > a.stride) atomicOr(a.status, ST_STRIDE_OVERFLOW | ST_LIST_OVERFLOW);
    }
  }
  if (MODE != 1) {   // largest count, for the next strided build's stride
    int m = act ? nlong : 0;
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
    if (lane == 0 && a.maxcnt) atomicMax(a.maxcnt, m);
  }
}


// One warp per atom, for small systems: the lanes take 32 consecutive candidates of the
// atom's stencil at a time (the bins and the order of k_list's walk for that atom), and
// ballots give every accepted entry its place -- inner entries from the front, the skin
// shell from the back, short candidates in order -- so the lists equal k_list's entry for
// entry.  k_list's warp walks its 32 atoms' stencils one candidate at a time, a serial
// chain that the few warps of a small system cannot hide (7,200 atoms: 225 warps, about
// 0.5 ms per build).  Per build, this kernel against k_list: 7,200-atom bilayer 0.26 vs
// 0.62 ms, 36,800-atom graphite 1.61 vs 1.94 ms, 331,200-atom graphite 12.8 vs 5.2 ms
// (there k_list's shared tiles save most candidate loads).
constexpr int LIST_ATOM_MAX_ATOMS = 40000;
template <int MODE>
__global__ void __launch_bounds__(128) k_list_atom(NbArgs a) {
  constexpr bool FILL = MODE != 0;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= a.n) return;   // whole warps
  const unsigned FULL = 0xffffffffu, below = (1u << lane) - 1u;
  const SysDesc &sd = a.sys[a.sysid[i]];
  const int lb = (int)(a.bin_key[i] >> KEY_MOL_BITS) - sd.bin_begin;
  const int bx = lb % sd.nb[0], by = (lb / sd.nb[0]) % sd.nb[1], bz = lb / (sd.nb[0] * sd.nb[1]);
  const float4 hi = a.xh[i], lo = a.xl[i];
  const int infoi = __float_as_int(hi.w);
  const int ti = infoi & 255;
  const int mi = infoi >> 8;
  const int ilp_i = c_nb.ilp_mapped[ti];
  const float prefilt = sd.prefilt_sq;
  int nlong = 0, nin = 0, nsh = 0, nshort = 0;
  bool img = false;
  const int64_t base = MODE == 1 ? a.list_off[i] : MODE == 2 ? (int64_t)i * a.stride : 0;
  const int64_t lend = MODE == 1 ? a.list_off[i + 1] : MODE == 2 ? base + a.stride : 0;
  uint32_t *const dst = MODE == 2 ? a.tmp : a.list;
  const int64_t dcap = MODE == 2 ? (int64_t)a.n * a.stride : a.list_cap;
  for (int dz = -sd.reach[2]; dz <= sd.reach[2]; dz++) {
    int jz = bz + dz, sz = 0;
    if (sd.per[2]) {
      sz = jz >= 0 ? jz / sd.nb[2] : -((-jz + sd.nb[2] - 1) / sd.nb[2]);
      jz -= sz * sd.nb[2];
    } else if (jz < 0 || jz >= sd.nb[2]) continue;
    for (int dy = -sd.reach[1]; dy <= sd.reach[1]; dy++) {
      int jy = by + dy, sy = 0;
      if (sd.per[1]) {
        sy = jy >= 0 ? jy / sd.nb[1] : -((-jy + sd.nb[1] - 1) / sd.nb[1]);
        jy -= sy * sd.nb[1];
      } else if (jy < 0 || jy >= sd.nb[1]) continue;
      if (a.rowocc && !a.rowocc[sd.bin_begin + (jz * sd.nb[1] + jy) * sd.nb[0]]) continue;   // empty row
      for (int xu = bx - sd.reach[0]; xu <= bx + sd.reach[0]; xu++) {
        int jx = xu, sx = 0;
        if (sd.per[0]) {
          sx = jx >= 0 ? jx / sd.nb[0] : -((-jx + sd.nb[0] - 1) / sd.nb[0]);
          jx -= sx * sd.nb[0];
        } else if (jx < 0 || jx >= sd.nb[0]) continue;
        const int gbj = sd.bin_begin + (jz * sd.nb[1] + jy) * sd.nb[0] + jx;
        const int jstart = a.bin_start[gbj], jend = a.bin_end[gbj];
        const float shx = (float)sx * sd.Lhi[0], shy = (float)sy * sd.Lhi[1], shz = (float)sz * sd.Lhi[2];
        const float slx = (float)sx * sd.Llo[0], sly = (float)sy * sd.Llo[1], slz = (float)sz * sd.Llo[2];
        const bool self_image = (sx | sy | sz) == 0;
        for (int j0 = jstart; j0 < jend; j0 += 32) {
          const int j = j0 + lane;
          bool take_long = false, inner = false, take_short = false;
          if (j < jend) {
            const float4 hj = a.xh[j];
            const float hx = (hi.x - hj.x) - shx, hy = (hi.y - hj.y) - shy, hz = (hi.z - hj.z) - shz;
            if (!(hx * hx + hy * hy + hz * hz > prefilt)) {
              const float4 lj = a.xl[j];
              float ddx = hx + ((lo.x - lj.x) - slx);
              float ddy = hy + ((lo.y - lj.y) - sly);
              float ddz = hz + ((lo.z - lj.z) - slz);
              float rsq = ddx * ddx + ddy * ddy + ddz * ddz;
              const int infoj = __float_as_int(hj.w);
              const int tj = infoj & 255;
              const int mj = infoj >> 8;
              const int tt = ti * (MAXTYPE + 1) + tj;
              if ((a.full || (mj != mi && ilp_i && c_nb.ilp_mapped[tj])) && !(self_image && j == i))
                take_long = le_exact(rsq, c_nb.cutnsq_f[tt], c_nb.cutnsq_d[tt], a.xq, sd, i, j, sx, sy, sz);
              inner = rsq < c_nb.innersq_f;
              if (MODE != 1 && !(self_image && j == i))
                take_short = le_exact(rsq, c_nb.rshortsq_f, c_nb.rshortsq_d, a.xq, sd, i, j, sx, sy, sz);
            }
          }
          const unsigned bin_ = __ballot_sync(FULL, take_long && inner);
          const unsigned bsh_ = __ballot_sync(FULL, take_long && !inner);
          if (FILL && take_long) {
            const int64_t pos = inner ? base + nin + __popc(bin_ & below) : lend - 1 - (nsh + __popc(bsh_ & below));
            if (pos >= base && pos < lend && pos < dcap) dst[pos] = encode_entry(j, sx, sy, sz, a.lc);
          }
          if (MODE != 1) {
            const unsigned bs = __ballot_sync(FULL, take_short);
            if (take_short) {
              const int q = nshort + __popc(bs & below);
              if (q < MAXSHORT) a.short_nb[(size_t)i * MAXSHORT + q] = encode_entry(j, sx, sy, sz, a.lc);
            }
            nshort += __popc(bs);
          }
          nin += __popc(bin_);
          nsh += __popc(bsh_);
          nlong += __popc(bin_ | bsh_);
          if ((bin_ | bsh_) && !self_image) img = true;
        }
      }
    }
  }
  if (lane != 0) return;
  if (MODE != 1) {
    a.cnt[i] = nlong;
    a.short_cnt[i] = nshort < MAXSHORT ? nshort : MAXSHORT;
    if (nshort > MAXSHORT) atomicOr(a.status, ST_SHORT_OVERFLOW);
    if (a.maxcnt) atomicMax(a.maxcnt, nlong);
  }
  if (MODE != 0) a.img[i] = img;
  if (MODE == 1 && base + nlong > a.list_cap) atomicOr(a.status, ST_LIST_OVERFLOW);
  if (MODE == 2) {
    a.nin[i] = nin;
    if (nlong > a.stride) atomicOr(a.status, ST_STRIDE_OVERFLOW | ST_LIST_OVERFLOW);
  }
}

// Strided buffer -> CSR list, one warp per atom: the entries inside the cutoff, then the
// shell (kept at the end of the atom's slice, in the order MODE 1 writes them), so the
// list equals MODE 1's.  Does nothing after a stride overflow (the host then fills).
__global__ void k_compact(int n, int stride, const uint32_t *tmp, const int *nin, const int64_t *off, uint32_t *list,
                          int64_t list_cap, const int *status) {
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n || (*status & ST_STRIDE_OVERFLOW)) return;
  const int64_t b = off[i];
  const int c = (int)(off[i + 1] - b), ni = nin[i];
  const uint32_t *src = tmp + (int64_t)i * stride;
  // four loads in flight per lane before the stores (the copy is latency-bound otherwise)
  for (int k0 = lane; k0 < c; k0 += 128) {
    uint32_t v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = k0 + 32 * u;
      v[u] = k >= c ? 0u : k < ni ? src[k] : src[stride - c + k];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = k0 + 32 * u;
      if (k < c && b + k < list_cap) list[b + k] = v[u];
    }
  }
}

__global__ void k_copy_hold(int n, const d4 *xq, double *xhold) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  d4 q = xq[p];
  xhold[3 * p] = q.x;
  xhold[3 * p + 1] = q.y;
  xhold[3 * p + 2] = q.z;
}

// ---------------------------------------------------------------- host side

void nb_upload_const(const NbConst &c, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_nb, &c, sizeof(c), 0, cudaMemcpyHostToDevice, s);
}

void nb_wrap_bin(int n, d4 *xq, const SysDesc *sys, const int *sysid, uint32_t *key, int *idx, cudaStream_t s) {
  if (n) k_wrap_bin<<<(n + 255) / 256, 256, 0, s>>>(n, xq, sys, sysid, key, idx);
}

size_t nb_sort_tmp_bytes(int n, int nbits) {
  size_t a = 0, b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, a, (uint32_t *)nullptr, (uint32_t *)nullptr, (int *)nullptr, (int *)nullptr, n, 0,
                                  nbits);
  cub::DeviceScan::ExclusiveSum(nullptr, b, (int64_t *)nullptr, (int64_t *)nullptr, n + 1);
  return a > b ? a : b;
}

// nbits: bits of the global bin index; the key's molecule bits come below them
cudaError_t nb_sort(void *tmp, size_t tmp_bytes, const uint32_t *k, uint32_t *k2, const int *v, int *v2, int n, int nbits,
                    cudaStream_t s) {
  return cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k, k2, v, v2, n, 0, nbits + KEY_MOL_BITS, s);
}

cudaError_t nb_scan(void *tmp, size_t tmp_bytes, const int64_t *cnt, int64_t *off, int n, cudaStream_t s) {
  return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, cnt, off, n + 1, s);
}

void nb_permute(int n, const int *idx2, const d4 *xq, d4 *xq2, const double *v, double *v2, const int64_t *tag,
                int64_t *tag2, const int *perm, int *perm2, const int *sysid, int *sysid2, const double *mass,
                double *mass2, cudaStream_t s) {
  if (n) k_permute<<<(n + 255) / 256, 256, 0, s>>>(n, idx2, xq, xq2, v, v2, tag, tag2, perm, perm2, sysid, sysid2, mass, mass2);
}

void nb_bin_ranges(int n, const uint32_t *key, int *bs, int *be, cudaStream_t s, const SysDesc *sys, const int *sysid,
                   int *rowocc) {
  if (n) k_bin_ranges<<<(n + 255) / 256, 256, 0, s>>>(n, key, bs, be, sys, sysid, rowocc);
}

void nb_hilo(int n, const d4 *xq, const SysDesc *sys, const int *sysid, float4 *xh, float4 *xl, cudaStream_t s) {
  if (n) k_hilo<<<(n + 255) / 256, 256, 0, s>>>(n, xq, sys, sysid, xh, xl);
}

void nb_list(const NbArgs &a, int mode, cudaStream_t s) {
  if (!a.n) return;
  if (a.n <= LIST_ATOM_MAX_ATOMS && !a.no_small) {
    const int ga = (int)(((int64_t)a.n * 32 + 127) / 128);
    if (mode == 1) k_list_atom<1><<<ga, 128, 0, s>>>(a);
    else if (mode == 2) k_list_atom<2><<<ga, 128, 0, s>>>(a);
    else k_list_atom<0><<<ga, 128, 0, s>>>(a);
    return;
  }
  const int g = (a.n + 32 * LW - 1) / (32 * LW);
  if (mode == 1) k_list<1><<<g, 32 * LW, 0, s>>>(a);
  else if (mode == 2) k_list<2><<<g, 32 * LW, 0, s>>>(a);
  else k_list<0><<<g, 32 * LW, 0, s>>>(a);
}

void nb_compact(const NbArgs &a, int64_t list_cap, cudaStream_t s) {
  if (!a.n) return;
  k_compact<<<(int)(((int64_t)a.n * 32 + 255) / 256), 256, 0, s>>>(a.n, a.stride, a.tmp, a.nin, a.list_off, a.list,
                                                                   list_cap, a.status);
}

void nb_copy_hold(int n, const d4 *xq, double *xhold, cudaStream_t s) {
  if (n) k_copy_hold<<<(n + 255) / 256, 256, 0, s>>>(n, xq, xhold);
}

}  // namespace lmff
