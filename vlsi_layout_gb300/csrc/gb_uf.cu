// gb_uf.cu -- PNUM connectivity on the GPU.
//
// Semantics of PerformMerge (pnummerge.f90:279-385) with UnionFind
// (datastructures.f90:26-215): two boxes are connected when their closed
// extents overlap (edge and corner touches count); the root of a component is
// its smallest box index; after the final reduction the non-singleton roots
// are numbered 1..R in index order and singletons keep label 0; the
// component count is R + #singletons.
//
// Candidate pairs come from a closed-range tile binning (every box is listed
// in each tile its closed extent touches, so two touching boxes share at
// least one tile).  Tiles of up to UF_WARP_BOXES boxes (nearly all: the grid
// is sized for about 32 boxes per tile) are taken one per warp, with the
// tile's boxes staged in the warp's shared memory; larger tiles are taken one
// per CTA.  Every pair that meets is hooked with atomicCAS, the larger root
// under the smaller, so the surviving root is the component minimum whatever
// the order of the hooks.  Pointer jumping then flattens the forest.
#include "gb_internal.h"
#include "gb_scan.cuh"

#define UF_SMEM_BOXES 1024
#define UF_WARP_BOXES 64   // tiles up to this size go one per warp
#define UF_WARPS 8         // warps per CTA of the per-warp kernels
#define KID_UF 30

__device__ __forceinline__ int uf_find(int* parent, int x) {
  // Path halving.  Parents only ever point to smaller indices, so writing a
  // grandparent is always a valid ancestor even under concurrent updates.
  int guard = 0;
  while (true) {
    const int p = parent[x];
    if (p == x || guard++ > (1 << 26)) return x;
    const int gp = parent[p];
    if (gp != p) atomicMin(&parent[x], gp);
    x = gp == p ? p : gp;
  }
}

__device__ __forceinline__ void uf_unite(int* parent, int a, int b, DStatus* st) {
  for (int it = 0; it < (1 << 24); ++it) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b) return;
    if (a > b) { const int t = a; a = b; b = t; }
    const int old = atomicCAS(&parent[b], b, a);
    if (old == b) return;
  }
  gb_set_error(st, GB_ERR_TIMEOUT, KID_UF, 0);
}

__global__ void k_uf_init(int* parent, unsigned char* touched, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    parent[i] = (int)i;
    touched[i] = 0;
  }
}

__device__ __forceinline__ bool closed_overlap(int4 a, int4 b) {
  return max(a.x, b.x) <= min(a.z, b.z) && max(a.y, b.y) <= min(a.w, b.w);
}

// The tile's pairs, one warp per tile of at most UF_WARP_BOXES boxes (tiles
// are taken in a grid stride over all warps; larger tiles are skipped and left
// to the per-CTA kernel).  act(ia, ba, ib, bb, t) handles one pair that meets.
template <typename Act>
__device__ __forceinline__ void warp_tiles(const DLayer* raw, const DLayer* bin, int4 (*sb)[UF_WARP_BOXES],
                                           int (*si)[UF_WARP_BOXES], Act act) {
  const int4* boxes = raw->boxes;
  const int* idx = (const int*)bin->pcs;
  const int w = gb_warp(), lane = gb_lane();
  const long long nt = bin->ntiles;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long t = (long long)blockIdx.x * (blockDim.x >> 5) + w; t < nt; t += nwarps) {
    const int k = bin->tcount[t];
    if (k < 2 || k > UF_WARP_BOXES) continue;
    const int* ti = idx + bin->tstart[t];
    for (int j = lane; j < k; j += 32) {
      const int i = ti[j];
      si[w][j] = i;
      sb[w][j] = boxes[i];
    }
    __syncwarp();
    for (int a = 0; a + 1 < k; ++a) {
      const int ia = si[w][a];
      const int4 ba = sb[w][a];
      for (int b = a + 1 + lane; b < k; b += 32) {
        const int4 bb = sb[w][b];
        if (closed_overlap(ba, bb)) act(ia, ba, si[w][b], bb, t);
      }
    }
    __syncwarp();  // the next tile overwrites the warp's boxes
  }
}

__global__ void __launch_bounds__(UF_WARPS * 32) k_uf_tile_warp(const DLayer* raw, const DLayer* bin, int* parent,
                                                              unsigned char* touched, DStatus* st) {
  __shared__ int4 sb[UF_WARPS][UF_WARP_BOXES];
  __shared__ int si[UF_WARPS][UF_WARP_BOXES];
  if (st->err) return;
  warp_tiles(raw, bin, sb, si, [&](int ia, int4, int ib, int4, long long) {
    touched[ia] = 1;
    touched[ib] = 1;
    uf_unite(parent, ia, ib, st);
  });
}

// Tiles of more than UF_WARP_BOXES boxes, one per CTA (a grid stride over
// the tiles; the others are skipped without a barrier).
__global__ void __launch_bounds__(256) k_uf_tile(const DLayer* raw, const DLayer* bin, int* parent,
                                                 unsigned char* touched, DStatus* st) {
  __shared__ int4 sb[UF_SMEM_BOXES];
  __shared__ int si[UF_SMEM_BOXES];
  const int4* boxes = raw->boxes;
  const int* idx = (const int*)bin->pcs;
  if (st->err) return;
  for (long long t = blockIdx.x; t < bin->ntiles; t += gridDim.x) {
    const int k = bin->tcount[t];
    if (k <= UF_WARP_BOXES) continue;
    const int* ti = idx + bin->tstart[t];
    const bool in_smem = k <= UF_SMEM_BOXES;
    __syncthreads();  // the previous tile's boxes are no longer read
    if (in_smem) {
      for (int j = threadIdx.x; j < k; j += blockDim.x) { si[j] = ti[j]; sb[j] = boxes[si[j]]; }
      __syncthreads();
    }
    const int nw = blockDim.x >> 5;
    for (int a = gb_warp(); a < k; a += nw) {
      const int ia = in_smem ? si[a] : ti[a];
      const int4 ba = in_smem ? sb[a] : boxes[ia];
      for (int b = a + 1 + gb_lane(); b < k; b += 32) {
        const int ib = in_smem ? si[b] : ti[b];
        const int4 bb = in_smem ? sb[b] : boxes[ib];
        if (closed_overlap(ba, bb)) {
          touched[ia] = 1;
          touched[ib] = 1;
          uf_unite(parent, ia, ib, st);
        }
      }
    }
  }
}

// Overlap statistics (ComputeInteractionsCPU, pnummerge.f90:483-562, and
// FindSingletonsCPU, :388-482).  Every pair meeting with closed bounds marks
// both boxes as non-singletons.  A pair overlapping with positive area is
// counted once: in the tile holding the lower-left corner of its
// intersection (both boxes are binned there, being closed-range binned).
__device__ __forceinline__ bool strict_overlap(int4 a, int4 b) {
  return max(a.x, b.x) < min(a.z, b.z) && max(a.y, b.y) < min(a.w, b.w);
}

// A strict pair is counted in the tile holding the lower-left corner of its
// intersection.
__device__ __forceinline__ bool counted_here(int4 ba, int4 bb, int g, const DLayer* bin, long long t) {
  if (!strict_overlap(ba, bb)) return false;
  const int4 w = bin->win[0];
  const long long li = t - bin->tbase[0];
  const int tx = w.x + (int)(li % w.z), ty = w.y + (int)(li / w.z);
  return (max(ba.x, bb.x) >> g) == tx && (max(ba.y, bb.y) >> g) == ty;
}

__global__ void __launch_bounds__(UF_WARPS * 32) k_pair_stats_warp(const DLayer* raw, const DLayer* bin, int g,
                                                                 unsigned char* touched,
                                                                 unsigned long long* strict, DStatus* st) {
  __shared__ int4 sb[UF_WARPS][UF_WARP_BOXES];
  __shared__ int si[UF_WARPS][UF_WARP_BOXES];
  if (st->err) return;
  unsigned long long cnt = 0;
  warp_tiles(raw, bin, sb, si, [&](int ia, int4 ba, int ib, int4 bb, long long t) {
    touched[ia] = 1;
    touched[ib] = 1;
    if (counted_here(ba, bb, g, bin, t)) ++cnt;
  });
  cnt = gb_warp_sum(cnt);
  if (gb_lane() == 0 && cnt) atomicAdd(strict, cnt);
}

// Tiles of more than UF_WARP_BOXES boxes, one per CTA.
__global__ void __launch_bounds__(256) k_pair_stats(const DLayer* raw, const DLayer* bin, int g,
                                                    unsigned char* touched, unsigned long long* strict,
                                                    DStatus* st) {
  __shared__ int4 sb[UF_SMEM_BOXES];
  __shared__ int si[UF_SMEM_BOXES];
  const int4* boxes = raw->boxes;
  const int* idx = (const int*)bin->pcs;
  if (st->err) return;
  unsigned long long cnt = 0;
  for (long long t = blockIdx.x; t < bin->ntiles; t += gridDim.x) {
    const int k = bin->tcount[t];
    if (k <= UF_WARP_BOXES) continue;
    const int* ti = idx + bin->tstart[t];
    const bool in_smem = k <= UF_SMEM_BOXES;
    __syncthreads();  // the previous tile's boxes are no longer read
    if (in_smem) {
      for (int j = threadIdx.x; j < k; j += blockDim.x) { si[j] = ti[j]; sb[j] = boxes[si[j]]; }
      __syncthreads();
    }
    const int nw = blockDim.x >> 5;
    for (int a = gb_warp(); a < k; a += nw) {
      const int ia = in_smem ? si[a] : ti[a];
      const int4 ba = in_smem ? sb[a] : boxes[ia];
      for (int b = a + 1 + gb_lane(); b < k; b += 32) {
        const int ib = in_smem ? si[b] : ti[b];
        const int4 bb = in_smem ? sb[b] : boxes[ib];
        if (closed_overlap(ba, bb)) {
          touched[ia] = 1;
          touched[ib] = 1;
          if (counted_here(ba, bb, g, bin, t)) ++cnt;
        }
      }
    }
  }
  cnt = gb_warp_sum(cnt);
  if (gb_lane() == 0 && cnt) atomicAdd(strict, cnt);
}

__global__ void k_singletons(const unsigned char* touched, long long n, unsigned char* mask,
                             unsigned long long* nsingle) {
  unsigned long long ns = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned char s = touched[i] ? 0 : 1;
    if (mask) mask[i] = s;
    ns += s;
  }
  ns = gb_warp_sum(ns);
  if (gb_lane() == 0 && ns) atomicAdd(nsingle, ns);
}

__global__ void k_uf_flatten(int* parent, const unsigned char* touched, int* flag, long long n,
                             long long* nsingle) {
  long long ns = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = uf_find(parent, (int)i);
    parent[i] = r;
    flag[i] = (touched[i] && r == (int)i) ? 1 : 0;
    ns += touched[i] ? 0 : 1;
  }
  ns = gb_warp_sum(ns);
  if (gb_lane() == 0 && ns) atomicAdd((unsigned long long*)nsingle, (unsigned long long)ns);
}

__global__ void k_uf_label(const int* parent, const unsigned char* touched, const long long* map,
                           long long* labels, long long n, const long long* nroots,
                           const long long* nsingle, long long* ncomp) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    labels[i] = touched[i] ? map[parent[i]] + 1 : 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *ncomp = *nroots + *nsingle;
}

__global__ void k_zero_ll(long long* p, int n) {
  if (threadIdx.x < n) p[threadIdx.x] = 0;
}
__global__ void k_set_ptrs(long long* slots, int* flag, long long* map, long long n) {
  slots[8] = (long long)flag;
  slots[9] = (long long)map;
  slots[10] = n;
}

void gb_launch_pair_stats(GbCtx& c, const DLayer* raw, DLayer* binidx, int g, unsigned char* touched,
                          long long n, unsigned long long* strict_dev, unsigned long long* single_dev,
                          unsigned char* mask_dev) {
  cudaMemsetAsync(touched, 0, (size_t)n, c.stream);
  cudaMemsetAsync(strict_dev, 0, 8, c.stream);
  cudaMemsetAsync(single_dev, 0, 8, c.stream);
  k_pair_stats_warp<<<c.nsm * 8, UF_WARPS * 32, 0, c.stream>>>(raw, binidx, g, touched, strict_dev, c.st);
  k_pair_stats<<<c.nsm * 4, 256, 0, c.stream>>>(raw, binidx, g, touched, strict_dev, c.st);
  k_singletons<<<c.work_blocks, 256, 0, c.stream>>>(touched, n, mask_dev, single_dev);
  c.launches += 3;
}

void gb_launch_components(GbCtx& c, const DLayer* raw, DLayer* binidx, int* parent,
                          unsigned char* touched, long long* labels, long long n,
                          long long* out_ncomp_dev, int* flag_tmp, long long* map_tmp) {
  const int wb = c.work_blocks;
  long long* sl = c.dscal;  // [4] nsingle, [5] nroots, [8..10] scan pointer slots
  k_zero_ll<<<1, 32, 0, c.stream>>>(sl + 4, 2);
  k_uf_init<<<wb, 256, 0, c.stream>>>(parent, touched, n);
  k_uf_tile_warp<<<c.nsm * 8, UF_WARPS * 32, 0, c.stream>>>(raw, binidx, parent, touched, c.st);
  k_uf_tile<<<c.nsm * 4, 256, 0, c.stream>>>(raw, binidx, parent, touched, c.st);
  k_uf_flatten<<<wb, 256, 0, c.stream>>>(parent, touched, flag_tmp, n, sl + 4);
  k_set_ptrs<<<1, 1, 0, c.stream>>>(sl, flag_tmp, map_tmp, n);
  gb_launch_scan_i32(c, (int* const*)&sl[8], (long long* const*)&sl[9], &sl[10], sl + 5);
  k_uf_label<<<wb, 256, 0, c.stream>>>(parent, touched, map_tmp, labels, n, sl + 5, sl + 4,
                                       out_ncomp_dev);
}
