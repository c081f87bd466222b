// gb_common.cuh -- shared device-side definitions of the box-Boolean engine.
//
// Layers live in HBM in one of two forms:
//   raw    : AoS int4 boxes {x1,y1,x2,y2} (global dbu) grouped into cells by
//            an offsets array (a cell is an independent layout, e.g. one of
//            the 4096 cells of a batched deck, or the whole layer);
//   binned : boxes clipped to the fixed 2^g-dbu tile grid and packed to 8 B
//            tile-relative pieces (x1 | (x2-1)<<16 | y1<<32 | (y2-1)<<48);
//            per cell a dense tile window, per tile a (start, count) pair.
// Every result of a Boolean operator is binned, so a chain of operators reads
// its operands tile by tile without re-binning.
//
// Sizes that depend on the data (tile windows, piece counts, slot capacities)
// are computed and consumed on the device: a descriptor (DLayer) in device
// memory is filled by small setup kernels and read by the worker kernels,
// whose grids are persistent.  No operator needs a host round trip, so a
// whole deck can be captured into one CUDA graph.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define GB_OK 0
#define GB_ERR_CAPACITY 1
#define GB_ERR_INVALID_BOX 2
#define GB_ERR_OOM 3
#define GB_ERR_TIMEOUT 4
#define GB_ERR_CUDA 5
#define GB_ERR_ARG 6
#define GB_ERR_INTERNAL 7

// Boolean opcodes: same numbering as the reference's Boost control parameter
// (boost_polygon_api.cpp:116-137): 0 XOR, 1 OR, 2 AND, 3 NOT (A-B), 4 MERGE.
#define GB_OP_XOR 0
#define GB_OP_OR 1
#define GB_OP_AND 2
#define GB_OP_NOT 3
#define GB_OP_MERGE 4
// No Boost counterpart: single-layer AND (design_impl.f90:385-498), the area
// covered by at least two boxes of A.
#define GB_OP_OVERLAP 7

#define GB_MAX_TILES_PER_OP (1ll << 28)

struct DStatus {          // one per context, in device memory
  int err;                // first error code (GB_ERR_*), 0 if none
  int where;              // kernel id that raised it
  long long need;         // size hint for capacity errors (bytes or slots)
  unsigned long long arena_off;   // device bump pointer of the work arena
  unsigned long long arena_cap;
  unsigned long long arena_high;  // high-water mark
  char* arena_base;
};

// A Boolean result's tile: its cell and where the operands' pieces of that
// tile start (offsets into their piece arrays).
struct TileDesc {
  int cell, nA, nB, pad;
  long long offA, offB;
};

struct DLayer {
  // common
  int ncell;
  int g;            // grid log2 (binned form)
  int binned;       // 1 = binned, 0 = raw
  int pad0;
  long long* cell_count;   // [ncell] boxes (raw) or strips (binned result)
  long long* cell_area;    // [ncell] union area when computed
  // raw form
  int4* boxes;
  long long* coff;         // [ncell+1]
  long long nbox;
  // binned form
  int4* win;               // [ncell]: tx0, ty0, ntx, nty
  long long* tbase;        // [ncell+1]
  long long* tstart;       // [ntiles]
  int* tcount;             // [ntiles]
  unsigned long long* pcs; // packed pieces
  long long ntiles;
  long long npcs;          // capacity of pcs (pieces)
  long long nused;         // pool cursor (Boolean results reserve per tile from it)
  long long ntot;          // pieces held by the layer
  int4* cbox;              // [ncell] bounding box (raw and binned)
  TileDesc* tdesc;         // [ntiles] Boolean results: each tile's cell and operand pieces (else null)
};

__host__ __device__ inline unsigned long long gb_pack(int x1, int y1, int x2, int y2) {
  return (unsigned long long)(unsigned)x1 | ((unsigned long long)(unsigned)(x2 - 1) << 16) |
         ((unsigned long long)(unsigned)y1 << 32) | ((unsigned long long)(unsigned)(y2 - 1) << 48);
}
__host__ __device__ inline void gb_unpack(unsigned long long p, int& x1, int& y1, int& x2, int& y2) {
  x1 = (int)(p & 0xFFFFu);
  x2 = (int)((p >> 16) & 0xFFFFu) + 1;
  y1 = (int)((p >> 32) & 0xFFFFu);
  y2 = (int)((p >> 48) & 0xFFFFu) + 1;
}
__host__ __device__ inline int gb_floor_shift(int v, int g) { return v >> g; }  // arithmetic shift = floor

// Hash of one strip in global coordinates, for order-independent per-cell
// digests (sum mod 2^64 over a layer's strips): the MurmurHash3 64-bit
// finaliser (fmix64) applied to the packed corners.  The oracle computes the
// same function.
__host__ __device__ inline unsigned long long gb_fmix64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}
__host__ __device__ inline unsigned long long gb_strip_hash(int x1, int y1, int x2, int y2) {
  const unsigned long long u = ((unsigned long long)(unsigned)x1 << 32) | (unsigned)y1;
  const unsigned long long v = ((unsigned long long)(unsigned)x2 << 32) | (unsigned)y2;
  return gb_fmix64(u ^ gb_fmix64(v + 0x9e3779b97f4a7c15ull));
}

__device__ inline void gb_set_error(DStatus* st, int code, int where, long long need) {
  if (atomicCAS(&st->err, 0, code) == 0) {
    st->where = where;
    st->need = need;
  } else if (code == GB_ERR_CAPACITY) {
    atomicMax(&st->need, need);
  }
}

// Device bump allocation from the work arena (called by one thread).
__device__ inline void* gb_arena_alloc(DStatus* st, unsigned long long bytes, int where) {
  unsigned long long off = (st->arena_off + 255ull) & ~255ull;
  unsigned long long end = off + ((bytes + 255ull) & ~255ull);
  if (end > st->arena_cap) {
    gb_set_error(st, GB_ERR_CAPACITY, where, (long long)end);
    if (end > st->arena_high) st->arena_high = end;
    return nullptr;
  }
  st->arena_off = end;
  if (end > st->arena_high) st->arena_high = end;
  return st->arena_base + off;
}

// Concurrent bump allocation (many CTAs at once).  Setup kernels use the
// single-thread form above; both never run at the same time on one stream.
__device__ inline void* gb_arena_alloc_atomic(DStatus* st, unsigned long long bytes, int where) {
  const unsigned long long sz = (bytes + 255ull) & ~255ull;
  const unsigned long long off = atomicAdd(&st->arena_off, sz);
  if (off + sz > st->arena_cap) {
    gb_set_error(st, GB_ERR_CAPACITY, where, (long long)(off + sz));
    return nullptr;
  }
  atomicMax(&st->arena_high, off + sz);
  return st->arena_base + off;
}

// Cell lookup: index k with off[k] <= i < off[k+1] (off has n+1 entries).
__device__ inline int gb_find_cell(const long long* off, int n, long long i) {
  int lo = 0, hi = n;  // invariant off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// ---- kernels shared across translation units (declared here, defined in .cu files)
struct GbLaunch {
  int nsm;
  int tile_blocks;  // persistent grid of the tile kernel
  int work_blocks;  // persistent grid of streaming kernels
};
