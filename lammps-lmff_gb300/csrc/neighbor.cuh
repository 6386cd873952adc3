// Neighbour-build interface between neighbor.cu and the engine.
#pragma once

#include "engine.cuh"

namespace lmff {

// Sort key of an atom: its global bin above KEY_MOL_BITS low bits of its molecule id, so
// that within a bin the atoms of one molecule (layer) are contiguous and the list build
// can pass over whole tiles of same-molecule candidates (never interlayer partners).
// Equal low bits of different molecules only make fewer tiles skippable.
constexpr int KEY_MOL_BITS = 4;
constexpr int64_t MAX_GLOBAL_BINS = 1LL << (32 - KEY_MOL_BITS);

// per type-pair cutoffs of the pair list and the short-candidate cutoff
struct NbConst {
  float cutnsq_f[(MAXTYPE + 1) * (MAXTYPE + 1)];
  double cutnsq_d[(MAXTYPE + 1) * (MAXTYPE + 1)];
  int ilp_mapped[MAXTYPE + 1];
  float rshortsq_f;
  double rshortsq_d;
  float innersq_f;   // ILP force cutoff squared: fill puts candidates inside it first
};

struct NbArgs {
  int n;
  const d4 *xq;
  const float4 *xh;
  const float4 *xl;
  const SysDesc *sys;
  const int *sysid;
  const int *bin_start;
  const int *bin_end;
  const int *rowocc;  // 1 at the first bin of every bin row (fixed y, z) holding atoms, or null
  int nbins;          // global bins
  const uint32_t *bin_key;   // sort key of each atom (sorted order): global bin << KEY_MOL_BITS | mol bits
  const int64_t *list_off;
  uint32_t *list;
  int64_t list_cap;
  int64_t *cnt;       // per-atom pair-list counts (int64: totals exceed 2^31)
  int *short_cnt;
  uint32_t *short_nb;
  uint8_t *img;       // fill pass: 1 per atom whose list holds periodic-image entries
  uint32_t *tmp;      // strided build: atom i's entries at tmp[i*stride, (i+1)*stride)
  int stride;
  int *nin;           // strided build: entries inside the force cutoff per atom
  int *maxcnt;        // count passes: largest per-atom count (atomicMax)
  ListCode lc;
  int full;
  int *status;
  int no_small;       // 1: the warp-per-32-atoms build at every size (option small_variants 0)
};

void nb_upload_const(const NbConst &c, cudaStream_t s);
void nb_wrap_bin(int n, d4 *xq, const SysDesc *sys, const int *sysid, uint32_t *key, int *idx, cudaStream_t s);
size_t nb_sort_tmp_bytes(int n, int nbits);
cudaError_t nb_sort(void *tmp, size_t tmp_bytes, const uint32_t *k, uint32_t *k2, const int *v, int *v2, int n, int nbits,
                    cudaStream_t s);
cudaError_t nb_scan(void *tmp, size_t tmp_bytes, const int64_t *cnt, int64_t *off, int n, cudaStream_t s);
void nb_permute(int n, const int *idx2, const d4 *xq, d4 *xq2, const double *v, double *v2, const int64_t *tag,
                int64_t *tag2, const int *perm, int *perm2, const int *sysid, int *sysid2, const double *mass,
                double *mass2, cudaStream_t s);
void nb_bin_ranges(int n, const uint32_t *key, int *bs, int *be, cudaStream_t s, const SysDesc *sys = nullptr,
                   const int *sysid = nullptr, int *rowocc = nullptr);
void nb_hilo(int n, const d4 *xq, const SysDesc *sys, const int *sysid, float4 *xh, float4 *xl, cudaStream_t s);
// mode 0: count (+ short lists); 1: fill the CSR list; 2: count and write each atom's
// entries into the strided buffer, for nb_compact after the scan
void nb_list(const NbArgs &a, int mode, cudaStream_t s);
void nb_compact(const NbArgs &a, int64_t list_cap, cudaStream_t s);
void nb_copy_hold(int n, const d4 *xq, double *xhold, cudaStream_t s);

}  // namespace lmff
