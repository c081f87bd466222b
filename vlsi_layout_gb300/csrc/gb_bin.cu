// gb_bin.cu -- device-sized scans, tile windows and the binning (split) pass.
//
// Binning is a counting sort of box pieces by tile: per-cell bounding boxes
// give a dense tile window, every (grown) box adds one to each tile it covers,
// an exclusive scan turns counts into starts, and a scatter writes the clipped
// 8-byte tile-relative pieces.  The order of pieces inside a tile is not
// significant: the tile kernel is order independent.
#include "gb_internal.h"
#include "gb_scan.cuh"

#define KID_BBOX 10
#define KID_WINDOW 11
#define KID_ALLOC 12
#define KID_SCAN 13
#define KID_EXPORT 14

// ------------------------------------------------------------------ scans
__global__ void k_scan1(int* const* inp, const long long* np, long long* part) {
  __shared__ long long tmp[33];
  const int* __restrict__ in = *inp;
  const long long n = in ? *np : 0;
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long long beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  long long s = 0;
  for (long long i = beg + threadIdx.x; i < end; i += blockDim.x) s += in[i];
  s = gb_block_sum(s, tmp);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_scan2(long long* part, int nb, long long* total) {
  __shared__ long long tmp[33];
  long long v = threadIdx.x < nb ? part[threadIdx.x] : 0;
  long long tot;
  long long ex = gb_block_excl(v, tmp, &tot);
  if (threadIdx.x < nb) part[threadIdx.x] = ex;
  if (threadIdx.x == 0 && total) *total = tot;
}

__global__ void k_scan3(int* const* inp, long long* const* outp, const long long* np,
                        const long long* part) {
  __shared__ long long tmp[33];
  constexpr int IT = 8;
  const int* __restrict__ in = *inp;
  long long* __restrict__ out = *outp;
  const long long n = (in && out) ? *np : 0;
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long long beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  long long carry = part[blockIdx.x];
  for (long long base = beg; base < end; base += (long long)blockDim.x * IT) {
    long long v[IT];
    long long s = 0;
    const long long my = base + (long long)threadIdx.x * IT;
#pragma unroll
    for (int k = 0; k < IT; ++k) {
      v[k] = (my + k < end) ? in[my + k] : 0;
      s += v[k];
    }
    long long tot;
    long long ex = gb_block_excl(s, tmp, &tot);
    long long run = carry + ex;
#pragma unroll
    for (int k = 0; k < IT; ++k) {
      if (my + k < end) out[my + k] = run;
      run += v[k];
    }
    carry += tot;
  }
}

void gb_launch_scan_i32(GbCtx& c, int* const* in_field, long long* const* out_field,
                        const long long* n_dev, long long* total_dev) {
  k_scan1<<<GB_SCAN_BLOCKS, GB_SCAN_THREADS, 0, c.stream>>>(in_field, n_dev, c.scan_part);
  k_scan2<<<1, GB_SCAN_BLOCKS, 0, c.stream>>>(c.scan_part, GB_SCAN_BLOCKS, total_dev);
  k_scan3<<<GB_SCAN_BLOCKS, GB_SCAN_THREADS, 0, c.stream>>>(in_field, out_field, n_dev, c.scan_part);
}

// ------------------------------------------------------------------ arena
__global__ void k_arena_reset(DStatus* st, unsigned long long mark) {
  st->arena_off = mark;
}
void gb_launch_arena_reset(GbCtx& c, unsigned long long mark) {
  k_arena_reset<<<1, 1, 0, c.stream>>>(c.st, mark);
}

// ------------------------------------------------------------------ bbox
__device__ __forceinline__ bool grow_box(int4 b, int E, int N, int W, int S, int4& o) {
  // box_grow_directional (geometry.f90:184-193): x2+=E, y2+=N, x1-=W, y1-=S.
  long long x1 = (long long)b.x - W, y1 = (long long)b.y - S;
  long long x2 = (long long)b.z + E, y2 = (long long)b.w + N;
  if (!(b.x < b.z && b.y < b.w) || x1 >= x2 || y1 >= y2 || x1 < INT32_MIN || y1 < INT32_MIN ||
      x2 > INT32_MAX || y2 > INT32_MAX)
    return false;
  o = make_int4((int)x1, (int)y1, (int)x2, (int)y2);
  return true;
}

__global__ void k_cbox_init(DLayer* O, int ncell, DStatus* st) {
  if (st->err) return;
  if (blockIdx.x == 0 && threadIdx.x == 0 && O->cbox == nullptr) {
    O->cbox = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * sizeof(int4), KID_ALLOC);
    O->cell_count = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_ALLOC);
    O->cell_area = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_ALLOC);
    O->tbase = (long long*)gb_arena_alloc(st, (unsigned long long)(ncell + 1) * 8, KID_ALLOC);
    O->win = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * sizeof(int4), KID_ALLOC);
  }
}

__global__ void k_cbox_fill(DLayer* O, int ncell, DStatus* st) {
  if (st->err) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
    O->cbox[k] = make_int4(INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN);
    O->cell_count[k] = 0;
    O->cell_area[k] = 0;
  }
}

__device__ __forceinline__ void warp_bbox_atomic(int4* dst, int x1, int y1, int x2, int y2) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    x1 = min(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y1 = min(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    x2 = max(x2, __shfl_xor_sync(0xffffffffu, x2, o));
    y2 = max(y2, __shfl_xor_sync(0xffffffffu, y2, o));
  }
  if (gb_lane() == 0 && x1 <= x2) {
    atomicMin(&dst->x, x1);
    atomicMin(&dst->y, y1);
    atomicMax(&dst->z, x2);
    atomicMax(&dst->w, y2);
  }
}

// Raw-source kernels walk the boxes in one contiguous chunk per warp (the
// boxes divided evenly over the grid's warps, in multiples of 32), 32
// consecutive boxes per step (coalesced), BIN_LD steps loaded before any is
// processed.  The cell of a box comes from one search of the cell
// offsets at the chunk's start; after that a lane only steps past the cells
// that end before its box (cells are sorted and hold many boxes, so nearly
// always none), which removes the dependent chain of a binary search per box.
#define BIN_LD 4

template <int LD, typename F>
__device__ __forceinline__ void walk_raw_boxes(const int4* bx, const long long* coff, int ncell, long long n, F f) {
  const int lane = gb_lane();
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const long long ch = max(32ll, (((n + nw - 1) / nw) + 31) & ~31ll);
  for (long long c0 = ((long long)blockIdx.x * (blockDim.x >> 5) + gb_warp()) * ch; c0 < n; c0 += nw * ch) {
    const long long c1 = min(n, c0 + ch);
    int k = 0;
    long long hi = 0;
    if (lane == 0) {
      k = gb_find_cell(coff, ncell, c0);
      hi = coff[k + 1];
    }
    k = __shfl_sync(0xffffffffu, k, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    for (long long b0 = c0; b0 < c1; b0 += 32 * LD) {
      int4 ld[LD];
#pragma unroll
      for (int u = 0; u < LD; ++u) {
        const long long i = b0 + 32 * u + lane;
        if (i < c1) ld[u] = bx[i];
      }
#pragma unroll
      for (int u = 0; u < LD; ++u) {
        const long long b = b0 + 32 * u;
        if (b >= c1) break;  // warp-uniform
        const long long i = b + lane;
        int kl = k;
        long long hl = hi;
        if (i < c1)
          while (i >= hl && kl + 1 < ncell) {
            ++kl;
            hl = coff[kl + 1];
          }
        f(i, i < c1, ld[u], kl);  // called by all lanes (warp collectives allowed)
        k = __shfl_sync(0xffffffffu, kl, 31);  // the last lane holds the furthest cell
        hi = __shfl_sync(0xffffffffu, hl, 31);
      }
    }
  }
}

// Raw source: one thread per box; boxes of a warp can straddle cells, so the
// warp reduces per cell only when all lanes agree, else atomics per lane.
__global__ void k_bbox_raw(const DLayer* S, DLayer* O, int ncell, int E, int N, int W, int Sg,
                           DStatus* st) {
  if (st->err) return;
  const long long n = S->nbox;
  const int4* bx = S->boxes;
  const long long* coff = S->coff;
  walk_raw_boxes<BIN_LD>(bx, coff, ncell, n, [&](long long i, bool valid_i, int4 box, int kc) {
    int x1 = INT32_MAX, y1 = INT32_MAX, x2 = INT32_MIN, y2 = INT32_MIN, k = -1;
    if (valid_i) {
      int4 g;
      if (!grow_box(box, E, N, W, Sg, g)) {
        gb_set_error(st, GB_ERR_INVALID_BOX, KID_BBOX, i);
      } else {
        x1 = g.x; y1 = g.y; x2 = g.z; y2 = g.w;
        k = kc;
      }
    }
    const int k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool same = __all_sync(0xffffffffu, k == k0 || k < 0);
    if (same) {
      if (k0 >= 0 || __any_sync(0xffffffffu, k >= 0)) {
        int kk = k0;
        if (kk < 0) {
          unsigned m = __ballot_sync(0xffffffffu, k >= 0);
          kk = __shfl_sync(0xffffffffu, k, __ffs(m) - 1);
        }
        warp_bbox_atomic(&O->cbox[kk], x1, y1, x2, y2);
      }
    } else if (k >= 0) {
      atomicMin(&O->cbox[k].x, x1);
      atomicMin(&O->cbox[k].y, y1);
      atomicMax(&O->cbox[k].z, x2);
      atomicMax(&O->cbox[k].w, y2);
    }
  });
}

__device__ __forceinline__ void tile_of_index(const DLayer* L, long long t, int& k, int& tx, int& ty) {
  k = gb_find_cell(L->tbase, L->ncell, t);
  const int4 w = L->win[k];
  const long long li = t - L->tbase[k];
  tx = w.x + (int)(li % w.z);
  ty = w.y + (int)(li / w.z);
}

// Binned source: one warp per source tile.
__global__ void k_bbox_bin(const DLayer* S, DLayer* O, int E, int N, int W, int Sg, DStatus* st) {
  if (st->err) return;
  const long long nt = S->ntiles;
  const int g = S->g;
  const int wpb = blockDim.x >> 5;
  for (long long t = (long long)blockIdx.x * wpb + gb_warp(); t < nt; t += (long long)gridDim.x * wpb) {
    const int cnt = S->tcount[t];
    if (cnt == 0) continue;
    int k, tx, ty;
    tile_of_index(S, t, k, tx, ty);
    const unsigned long long* p = S->pcs + S->tstart[t];
    const int ox = tx << g, oy = ty << g;
    int x1 = INT32_MAX, y1 = INT32_MAX, x2 = INT32_MIN, y2 = INT32_MIN;
    for (int j = gb_lane(); j < cnt; j += 32) {
      int a, b, c, d;
      gb_unpack(p[j], a, b, c, d);
      int4 gbx;
      if (!grow_box(make_int4(ox + a, oy + b, ox + c, oy + d), E, N, W, Sg, gbx)) {
        gb_set_error(st, GB_ERR_INVALID_BOX, KID_BBOX, t);
        continue;
      }
      x1 = min(x1, gbx.x); y1 = min(y1, gbx.y); x2 = max(x2, gbx.z); y2 = max(y2, gbx.w);
    }
    warp_bbox_atomic(&O->cbox[k], x1, y1, x2, y2);
  }
}

// ------------------------------------------------------------------ windows
// One block: per-cell tile window from the cell bbox, scan into tbase, and
// allocate the per-tile arrays.  closed=1 uses closed tile ranges (x2 >> g).
__global__ void k_window(DLayer* O, int ncell, int g, int closed, DStatus* st) {
  __shared__ long long tmp[33];
  __shared__ long long carry;
  if (st->err) return;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int k = base + threadIdx.x;
    long long nt = 0;
    if (k < ncell) {
      int4 b = O->cbox[k];
      int4 w = make_int4(0, 0, 0, 0);
      if (b.x <= b.z && b.y <= b.w && (closed || (b.x < b.z && b.y < b.w))) {
        const int tx0 = gb_floor_shift(b.x, g), ty0 = gb_floor_shift(b.y, g);
        const int tx1 = closed ? gb_floor_shift(b.z, g) : gb_floor_shift(b.z - 1, g);
        const int ty1 = closed ? gb_floor_shift(b.w, g) : gb_floor_shift(b.w - 1, g);
        w = make_int4(tx0, ty0, tx1 - tx0 + 1, ty1 - ty0 + 1);
        nt = (long long)w.z * w.w;
      }
      O->win[k] = w;
    }
    long long tot;
    long long ex = gb_block_excl(nt, tmp, &tot);
    if (k < ncell) O->tbase[k] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const long long total = carry;
    O->tbase[ncell] = total;
    O->ntiles = total;
    O->g = g;
    O->binned = 1;
    if (total > GB_MAX_TILES_PER_OP) {
      gb_set_error(st, GB_ERR_CAPACITY, KID_WINDOW, total);
      O->ntiles = 0;
      return;
    }
    O->tstart = (long long*)gb_arena_alloc(st, (unsigned long long)(total + 1) * 8, KID_ALLOC);
    O->tcount = (int*)gb_arena_alloc(st, (unsigned long long)(total + 1) * 4, KID_ALLOC);
    if (!O->tstart || !O->tcount) O->ntiles = 0;
  }
}

__global__ void k_zero_tcount(DLayer* O, DStatus* st) {
  if (st->err) return;
  const long long n = O->ntiles;
  int* c = O->tcount;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    c[i] = 0;
}

__global__ void k_alloc_pcs(DLayer* O, int elem_bytes, DStatus* st) {
  if (st->err) return;
  O->pcs = (unsigned long long*)gb_arena_alloc(st, (unsigned long long)(O->npcs + 1) * elem_bytes,
                                               KID_ALLOC);
  O->nused = O->npcs;
  O->ntot = O->npcs;
  if (!O->pcs) O->ntiles = 0;
}

// ------------------------------------------------------------------ count / scatter
// mode 0: half-open tile ranges, packed pieces; mode 1: closed ranges, int index payload.
template <int MODE, bool SCATTER>
__device__ __forceinline__ void emit_box_tiles(DLayer* O, int k, int4 b, long long payload_idx, int g) {
  const int4 w = O->win[k];
  const int tx0 = gb_floor_shift(b.x, g), ty0 = gb_floor_shift(b.y, g);
  const int tx1 = MODE ? gb_floor_shift(b.z, g) : gb_floor_shift(b.z - 1, g);
  const int ty1 = MODE ? gb_floor_shift(b.w, g) : gb_floor_shift(b.w - 1, g);
  const long long tb = O->tbase[k];
  for (int ty = ty0; ty <= ty1; ++ty) {
    for (int tx = tx0; tx <= tx1; ++tx) {
      const long long t = tb + (long long)(ty - w.y) * w.z + (tx - w.x);
      if (!SCATTER) {
        atomicAdd(&O->tcount[t], 1);
      } else {
        const long long pos = O->tstart[t] + atomicAdd(&O->tcount[t], 1);
        if (MODE == 0) {
          const int ox = tx << g, oy = ty << g;
          const int x1 = max(b.x, ox) - ox, y1 = max(b.y, oy) - oy;
          const int x2 = (int)(min((long long)b.z, (long long)ox + (1ll << g)) - ox);
          const int y2 = (int)(min((long long)b.w, (long long)oy + (1ll << g)) - oy);
          O->pcs[pos] = gb_pack(x1, y1, x2, y2);
        } else {
          ((int*)O->pcs)[pos] = (int)payload_idx;
        }
      }
    }
  }
}

// All 32 lanes call: a box that lies in one tile (nearly all) takes its slot
// with one atomic per group of lanes that target the same tile (the group's
// first lane adds the group's size; each lane's slot is its rank in the
// group), so the pieces of one source tile, which mostly land in one target
// tile, do not serialise on that tile's counter.  Boxes over several tiles
// take the per-tile path.  valid = false: the lane places nothing.  Used for
// binned sources (count 1.71 -> 0.83 ms, scatter 1.93 -> 1.38 ms per two
// 1024-cell decks); raw sources scatter over many tiles and keep per-lane
// slots.
template <int MODE, bool SCATTER>
__device__ __forceinline__ void emit_warp(DLayer* O, int k, int4 b, long long payload_idx, int g, bool valid) {
  const int lane = gb_lane();
  long long t = -1 - lane;  // distinct for lanes without a single tile
  bool single = false;
  int tx0 = 0, ty0 = 0;
  if (valid) {
    tx0 = gb_floor_shift(b.x, g);
    ty0 = gb_floor_shift(b.y, g);
    const int tx1 = MODE ? gb_floor_shift(b.z, g) : gb_floor_shift(b.z - 1, g);
    const int ty1 = MODE ? gb_floor_shift(b.w, g) : gb_floor_shift(b.w - 1, g);
    single = tx0 == tx1 && ty0 == ty1;
    if (single) {
      const int4 w = O->win[k];
      t = O->tbase[k] + (long long)(ty0 - w.y) * w.z + (tx0 - w.x);
    }
  }
  const unsigned grp = __match_any_sync(0xffffffffu, t);
  const int lead = __ffs(grp) - 1;
  int base = 0;
  if (single && lane == lead) base = atomicAdd(&O->tcount[t], __popc(grp));
  base = __shfl_sync(0xffffffffu, base, lead);
  if (single) {
    if (SCATTER) {
      const long long pos = O->tstart[t] + base + __popc(grp & ((1u << lane) - 1u));
      if (MODE == 0) {
        const int ox = tx0 << g, oy = ty0 << g;
        O->pcs[pos] = gb_pack(b.x - ox, b.y - oy, b.z - ox, b.w - oy);
      } else {
        ((int*)O->pcs)[pos] = (int)payload_idx;
      }
    }
  } else if (valid) {
    emit_box_tiles<MODE, SCATTER>(O, k, b, payload_idx, g);
  }
}

template <int MODE, bool SCATTER>
__global__ void k_split_raw(const DLayer* S, DLayer* O, int ncell, int g, int E, int N, int W,
                            int Sg, DStatus* st) {
  if (st->err) return;
  walk_raw_boxes<SCATTER ? 2 : BIN_LD>(S->boxes, S->coff, ncell, S->nbox,
                                       [&](long long i, bool valid_i, int4 box, int k) {
    // raw boxes of one warp fall in scattered tiles of their cell, so a per-lane slot is cheaper
    // here than grouping lanes by tile
    int4 b;
    if (!valid_i || !grow_box(box, E, N, W, Sg, b)) return;  // invalid: reported by k_bbox_raw
    emit_box_tiles<MODE, SCATTER>(O, k, b, i, g);
  });
}

template <bool SCATTER>
__global__ void k_split_bin(const DLayer* S, DLayer* O, int g, int E, int N, int W, int Sg,
                            DStatus* st) {
  if (st->err) return;
  const long long nt = S->ntiles;
  const int sg = S->g;
  const int wpb = blockDim.x >> 5;
  for (long long t = (long long)blockIdx.x * wpb + gb_warp(); t < nt; t += (long long)gridDim.x * wpb) {
    const int cnt = S->tcount[t];
    if (cnt == 0) continue;
    int k, tx, ty;
    tile_of_index(S, t, k, tx, ty);
    const unsigned long long* p = S->pcs + S->tstart[t];
    const int ox = tx << sg, oy = ty << sg;
    for (int j0 = 0; j0 < cnt; j0 += 32) {  // whole warps: emit_warp is a warp collective
      const int j = j0 + gb_lane();
      int4 gbx = make_int4(0, 0, 1, 1);
      bool ok = false;
      if (j < cnt) {
        int a, b, c, d;
        gb_unpack(p[j], a, b, c, d);
        ok = grow_box(make_int4(ox + a, oy + b, ox + c, oy + d), E, N, W, Sg, gbx);
      }
      emit_warp<0, SCATTER>(O, k, gbx, 0, g, ok);
    }
  }
}

// ------------------------------------------------------------------ launchers
static void launch_bin_common(GbCtx& c, const DLayer* src, int src_binned, DLayer* out, int ncell,
                              int g, int E, int N, int W, int S, int mode) {
  const int wb = c.work_blocks, T = 256;
  k_cbox_init<<<1, 32, 0, c.stream>>>(out, ncell, c.st);
  k_cbox_fill<<<(ncell + 255) / 256, 256, 0, c.stream>>>(out, ncell, c.st);
  if (src_binned) k_bbox_bin<<<wb, T, 0, c.stream>>>(src, out, E, N, W, S, c.st);
  else k_bbox_raw<<<wb, T, 0, c.stream>>>(src, out, ncell, E, N, W, S, c.st);
  k_window<<<1, 1024, 0, c.stream>>>(out, ncell, g, mode, c.st);
  k_zero_tcount<<<wb, T, 0, c.stream>>>(out, c.st);
  if (mode == 0) {
    if (src_binned) k_split_bin<false><<<wb, T, 0, c.stream>>>(src, out, g, E, N, W, S, c.st);
    else k_split_raw<0, false><<<wb, T, 0, c.stream>>>(src, out, ncell, g, E, N, W, S, c.st);
  } else {
    k_split_raw<1, false><<<wb, T, 0, c.stream>>>(src, out, ncell, g, 0, 0, 0, 0, c.st);
  }
  gb_launch_scan_i32(c, &out->tcount, &out->tstart, &out->ntiles, &out->npcs);
  k_alloc_pcs<<<1, 1, 0, c.stream>>>(out, mode == 0 ? 8 : 4, c.st);
  k_zero_tcount<<<wb, T, 0, c.stream>>>(out, c.st);
  if (mode == 0) {
    if (src_binned) k_split_bin<true><<<wb, T, 0, c.stream>>>(src, out, g, E, N, W, S, c.st);
    else k_split_raw<0, true><<<wb, T, 0, c.stream>>>(src, out, ncell, g, E, N, W, S, c.st);
  } else {
    k_split_raw<1, true><<<wb, T, 0, c.stream>>>(src, out, ncell, g, 0, 0, 0, 0, c.st);
  }
}

void gb_launch_rebin(GbCtx& c, const DLayer* src, int src_binned, DLayer* out, int ncell, int g,
                     int E, int N, int W, int S) {
  launch_bin_common(c, src, src_binned, out, ncell, g, E, N, W, S, 0);
}

void gb_launch_bin_index(GbCtx& c, const DLayer* src, DLayer* out, int ncell, int g) {
  launch_bin_common(c, src, 0, out, ncell, g, 0, 0, 0, 0, 1);
}

// Per-cell bounding box of a raw layer (no grow) into its own cbox.
void gb_launch_cell_bbox_fill(GbCtx& c, DLayer* L, int ncell) {
  k_cbox_init<<<1, 32, 0, c.stream>>>(L, ncell, c.st);
  k_cbox_fill<<<(ncell + 255) / 256, 256, 0, c.stream>>>(L, ncell, c.st);
  k_bbox_raw<<<c.work_blocks, 256, 0, c.stream>>>(L, L, ncell, 0, 0, 0, 0, c.st);
}

// ------------------------------------------------------------------ Boolean op setup
__device__ __forceinline__ int tile_index_in(const DLayer* L, int k, int tx, int ty, long long* t) {
  if (L == nullptr) return 0;
  const int4 w = L->win[k];
  if (tx < w.x || ty < w.y || tx >= w.x + w.z || ty >= w.y + w.w) return 0;
  *t = L->tbase[k] + (long long)(ty - w.y) * w.z + (tx - w.x);
  return 1;
}

// Output window per cell: the union of both windows for OR / XOR, A's window
// otherwise (AND, NOT and MERGE results lie inside A).
__global__ void k_bool_window(int op, const DLayer* A, const DLayer* B, DLayer* O, int ncell, int g,
                              DStatus* st) {
  __shared__ long long tmp[33];
  __shared__ long long carry;
  if (st->err) return;
  if (threadIdx.x == 0) {
    carry = 0;
    O->cbox = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * sizeof(int4), KID_ALLOC);
    O->cell_count = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_ALLOC);
    O->cell_area = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_ALLOC);
    O->tbase = (long long*)gb_arena_alloc(st, (unsigned long long)(ncell + 1) * 8, KID_ALLOC);
    O->win = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * sizeof(int4), KID_ALLOC);
  }
  __syncthreads();
  if (st->err) return;
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int k = base + threadIdx.x;
    long long nt = 0;
    if (k < ncell) {
      int4 wa = A->win[k];
      int4 w = wa;
      if ((op == GB_OP_OR || op == GB_OP_XOR) && B) {
        int4 wb = B->win[k];
        if (wa.z == 0 || wa.w == 0) w = wb;
        else if (wb.z > 0 && wb.w > 0) {
          const int x0 = min(wa.x, wb.x), y0 = min(wa.y, wb.y);
          const int x1 = max(wa.x + wa.z, wb.x + wb.z), y1 = max(wa.y + wa.w, wb.y + wb.w);
          w = make_int4(x0, y0, x1 - x0, y1 - y0);
        }
      }
      if (w.z <= 0 || w.w <= 0) w = make_int4(0, 0, 0, 0);
      O->win[k] = w;
      O->cell_count[k] = 0;
      O->cell_area[k] = 0;
      O->cbox[k] = make_int4(w.x << g, w.y << g, (w.x + w.z) << g, (w.y + w.w) << g);
      nt = (long long)w.z * w.w;
    }
    long long tot;
    long long ex = gb_block_excl(nt, tmp, &tot);
    if (k < ncell) O->tbase[k] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const long long total = carry;
    O->tbase[ncell] = total;
    O->ntiles = total;
    O->g = g;
    O->binned = 1;
    if (total > GB_MAX_TILES_PER_OP) {
      gb_set_error(st, GB_ERR_CAPACITY, KID_WINDOW, total);
      O->ntiles = 0;
      return;
    }
    O->tstart = (long long*)gb_arena_alloc(st, (unsigned long long)(total + 1) * 8, KID_ALLOC);
    O->tcount = (int*)gb_arena_alloc(st, (unsigned long long)(total + 1) * 4, KID_ALLOC);
    O->tdesc = (TileDesc*)gb_arena_alloc(st, (unsigned long long)(total + 1) * sizeof(TileDesc), KID_ALLOC);
    if (!O->tstart || !O->tcount || !O->tdesc) O->ntiles = 0;
  }
}

// Every output tile's cell and the operands' pieces of that tile, so the tile
// kernel looks a tile up with one load.  Only B's pieces of a two-operand op.
__global__ void k_tile_descs(int op, const DLayer* A, const DLayer* B, DLayer* O, DStatus* st) {
  if (st->err) return;
  const long long n = O->ntiles;
  const bool useB = B && op != GB_OP_MERGE && op != GB_OP_OVERLAP;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int k = gb_find_cell(O->tbase, O->ncell, t);
    const int4 w = O->win[k];
    const long long li = t - O->tbase[k];
    const int tx = w.x + (int)(li % w.z), ty = w.y + (int)(li / w.z);
    TileDesc d;
    d.cell = k;
    d.nA = d.nB = d.pad = 0;
    d.offA = d.offB = 0;
    long long ta = 0, tb = 0;
    if (tile_index_in(A, k, tx, ty, &ta)) {
      d.nA = A->tcount[ta];
      d.offA = A->tstart[ta];
    }
    if (useB && tile_index_in(B, k, tx, ty, &tb)) {
      d.nB = B->tcount[tb];
      d.offB = B->tstart[tb];
    }
    O->tdesc[t] = d;
  }
}

// Output pool of a Boolean op: factor x (pieces of A + pieces of B) plus a
// little per tile.  Each tile reserves exactly its strip count from the pool
// cursor (nused) once it knows it, so no per-tile slack is needed; a tile
// that no longer fits takes its slots from the arena directly (atomically),
// at an offset relative to the pool base.
__global__ void k_pool_alloc(const DLayer* A, const DLayer* B, DLayer* O, int factor, DStatus* st) {
  if (st->err) return;
  const long long na = A ? A->ntot : 0, nb = B ? B->ntot : 0;
  O->npcs = (na + nb) * factor + 16 * O->ntiles + 64;
  O->nused = 0;
  O->ntot = 0;
  O->pcs = (unsigned long long*)gb_arena_alloc(st, (unsigned long long)O->npcs * 8, KID_ALLOC);
  if (!O->pcs) O->ntiles = 0;
}

void gb_launch_bool_setup(GbCtx& c, int op, const DLayer* A, const DLayer* B, DLayer* O, int ncell,
                          int g, int alloc_slots) {
  k_bool_window<<<1, 1024, 0, c.stream>>>(op, A, B, O, ncell, g, c.st);
  k_tile_descs<<<c.work_blocks, 256, 0, c.stream>>>(op, A, B, O, c.st);
  if (!alloc_slots) return;
  k_pool_alloc<<<1, 1, 0, c.stream>>>(A, op == GB_OP_MERGE ? nullptr : B, O, c.cap_factor, c.st);
}

// ------------------------------------------------------------------ export
// Slots of c.dscal used by the export: [0] = int4* array, [1] = offsets*, [2] = total.
__global__ void k_export_alloc1(const DLayer* L, long long* dscal, DStatus* st) {
  if (st->err) { dscal[0] = 0; dscal[1] = 0; dscal[2] = 0; return; }
  dscal[1] = (long long)gb_arena_alloc(st, (unsigned long long)(L->ntiles + 1) * 8, KID_EXPORT);
  dscal[3] = L->ntiles;
}
__global__ void k_export_alloc2(long long* dscal, DStatus* st) {
  if (st->err) { dscal[0] = 0; return; }
  dscal[0] = (long long)gb_arena_alloc(st, (unsigned long long)(dscal[2] + 1) * 16, KID_EXPORT);
}
__global__ void k_export(const DLayer* L, const long long* dscal, DStatus* st) {
  if (st->err) return;
  int4* out = (int4*)dscal[0];
  const long long* off = (const long long*)dscal[1];
  if (!out || !off) return;
  const long long nt = L->ntiles;
  const int g = L->g;
  const int wpb = blockDim.x >> 5;
  for (long long t = (long long)blockIdx.x * wpb + gb_warp(); t < nt; t += (long long)gridDim.x * wpb) {
    const int cnt = L->tcount[t];
    if (cnt == 0) continue;
    int k, tx, ty;
    tile_of_index(L, t, k, tx, ty);
    const unsigned long long* p = L->pcs + L->tstart[t];
    const int ox = tx << g, oy = ty << g;
    const long long o = off[t];
    for (int j = gb_lane(); j < cnt; j += 32) {
      int a, b, cc, d;
      gb_unpack(p[j], a, b, cc, d);
      out[o + j] = make_int4(ox + a, oy + b, ox + cc, oy + d);
    }
  }
}

// Per-cell digest of a binned layer: the sum (mod 2^64) of gb_strip_hash over
// its strips in global coordinates.  A sum is independent of the strip order,
// so two layers with the same canonical strips per cell have equal digests
// whatever order their tiles were written in.  One warp per tile.
__global__ void k_cell_digest(const DLayer* L, unsigned long long* out, int stride) {
  const long long nt = L->ntiles;
  const int g = L->g;
  const int wpb = blockDim.x >> 5;
  for (long long t = (long long)blockIdx.x * wpb + gb_warp(); t < nt; t += (long long)gridDim.x * wpb) {
    const int cnt = L->tcount[t];
    if (cnt == 0) continue;
    int k, tx, ty;
    tile_of_index(L, t, k, tx, ty);
    const unsigned long long* p = L->pcs + L->tstart[t];
    const int ox = tx << g, oy = ty << g;
    unsigned long long h = 0;
    for (int j = gb_lane(); j < cnt; j += 32) {
      int a, b, cc, d;
      gb_unpack(p[j], a, b, cc, d);
      h += gb_strip_hash(ox + a, oy + b, ox + cc, oy + d);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if (gb_lane() == 0) atomicAdd(&out[(size_t)k * stride], h);
  }
}

void gb_launch_digest(GbCtx& c, const DLayer* L, unsigned long long* out, int stride) {
  k_cell_digest<<<c.work_blocks, 256, 0, c.stream>>>(L, out, stride);
}

void gb_launch_export(GbCtx& c, const DLayer* L, int4** out_ptr_dev, long long* total_dev) {
  (void)out_ptr_dev;
  (void)total_dev;
  k_export_alloc1<<<1, 1, 0, c.stream>>>(L, c.dscal, c.st);
  gb_launch_scan_i32(c, (int* const*)&L->tcount, (long long* const*)&c.dscal[1], &c.dscal[3],
                     &c.dscal[2]);
  k_export_alloc2<<<1, 1, 0, c.stream>>>(c.dscal, c.st);
  k_export<<<c.work_blocks, 256, 0, c.stream>>>(L, c.dscal, c.st);
}
