// gb_api.cu -- host side of the C-ABI (include/gbool.h): contexts, layers,
// operators, connectivity, sorts and the reference drop-in symbols.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <functional>
#include <mutex>
#include <vector>

#include "gbool.h"
#include "gb_internal.h"
#include "gb_scan.cuh"

#define KID_FRAME 50
#define KID_KEYS 51

namespace gbi {

int set_err(gb_context* ctx, int code, const char* msg) {
  if (ctx) ctx->c.last_error = msg;
  return code;
}

__global__ void k_desc_init(DLayer* d, int ncell, int g, int binned) {
  DLayer z;
  memset(&z, 0, sizeof(z));
  z.ncell = ncell;
  z.g = g;
  z.binned = binned;
  *d = z;
}

int alloc_slot(gb_context* ctx) {
  if (ctx->c.desc_free.empty()) return -1;
  int s = ctx->c.desc_free.back();
  ctx->c.desc_free.pop_back();
  return s;
}

gb_layer* new_arena_layer(gb_context* ctx, int ncell, int g) {
  int s = alloc_slot(ctx);
  if (s < 0) return nullptr;
  gb_layer* L = new gb_layer();
  L->slot = s;
  L->d = ctx->c.desc + s;
  L->ncell = ncell;
  L->g = g;
  L->binned = 1;
  L->arena_owned = 1;
  L->seq = ++ctx->seq;
  k_desc_init<<<1, 1, 0, ctx->c.stream>>>(L->d, ncell, g, 1);
  ctx->arena_layers.push_back(L);
  return L;
}

void drop_layer(gb_context* ctx, gb_layer* L) {
  if (!L) return;
  if (L->slot >= 0) ctx->c.desc_free.push_back(L->slot);
  L->slot = -1;
  if (L->own_boxes) cudaFree(L->own_boxes);
  if (L->own_coff) cudaFree(L->own_coff);
  if (L->own_cell) cudaFree(L->own_cell);
  L->own_boxes = L->own_coff = L->own_cell = nullptr;
}

// The binned form of L on grid g: L itself, the cached binning of a raw
// layer, or a new binning (from raw boxes or from a result on another grid).
gb_layer* binned_of(gb_context* ctx, gb_layer* L, int g) {
  if (L->binned && L->g == g) return L;
  if (!L->binned && L->bin_cache && !L->bin_cache->dead && L->bin_cache->g == g) return L->bin_cache;
  gb_layer* B = new_arena_layer(ctx, L->ncell, g);
  if (!B) return nullptr;
  gb_launch_rebin(ctx->c, L->d, L->binned, B->d, L->ncell, g, 0, 0, 0, 0);
  if (!L->binned) L->bin_cache = B;
  return B;
}

DStatus read_status(gb_context* ctx) {
  DStatus s;
  cudaStreamSynchronize(ctx->c.stream);
  cudaMemcpy(&s, ctx->c.st, sizeof(DStatus), cudaMemcpyDeviceToHost);
  return s;
}

__global__ void k_clear_status(DStatus* st) {
  st->err = 0;
  st->where = 0;
  st->need = 0;
}

DLayer read_desc(gb_context* ctx, gb_layer* L) {
  DLayer d;
  cudaStreamSynchronize(ctx->c.stream);
  cudaMemcpy(&d, L->d, sizeof(DLayer), cudaMemcpyDeviceToHost);
  return d;
}

// Frame of an erosion: per cell the cell bbox grown by t (a superset of
// bbox(P) (+) t is all the construction needs); empty cells get a unit box,
// which leaves their (empty) result unchanged.
__global__ void k_make_frame(const DLayer* P, DLayer* F, int ncell, int t, DStatus* st) {
  if (st->err) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    F->boxes = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * 16, KID_FRAME);
    F->coff = (long long*)gb_arena_alloc(st, (unsigned long long)(ncell + 1) * 8, KID_FRAME);
    F->cbox = (int4*)gb_arena_alloc(st, (unsigned long long)ncell * 16, KID_FRAME);
    F->cell_count = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_FRAME);
    F->cell_area = (long long*)gb_arena_alloc(st, (unsigned long long)ncell * 8, KID_FRAME);
    F->nbox = ncell;
    F->binned = 0;
    if (F->boxes && F->coff) F->coff[ncell] = ncell;
  }
}
__global__ void k_fill_frame(const DLayer* P, DLayer* F, int ncell, int t, DStatus* st) {
  if (st->err) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
    const int4 b = P->cbox[k];
    int4 o = make_int4(0, 0, 1, 1);
    if (b.x < b.z && b.y < b.w) {
      const long long x1 = (long long)b.x - t, y1 = (long long)b.y - t;
      const long long x2 = (long long)b.z + t, y2 = (long long)b.w + t;
      if (x1 < INT32_MIN || y1 < INT32_MIN || x2 > INT32_MAX || y2 > INT32_MAX) {
        gb_set_error(st, GB_ERR_INVALID_BOX, KID_FRAME, k);
      } else {
        o = make_int4((int)x1, (int)y1, (int)x2, (int)y2);
      }
    }
    F->boxes[k] = o;
    F->coff[k] = k;
    F->cbox[k] = o;
    F->cell_count[k] = 1;
    F->cell_area[k] = 0;
  }
}

__global__ void k_count_tiles(const DLayer* L, long long* per_cell, int ncell, DStatus* st) {
  if (st->err || !L->tcount || !L->tbase) return;
  const long long nt = L->ntiles;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = L->tcount[t];
    if (c) {
      const int k = gb_find_cell(L->tbase, ncell, t);
      atomicAdd((unsigned long long*)&per_cell[k], (unsigned long long)c);
    }
  }
}

// ComputeMorton (gpu_morton.cu:113-144): the box centre's coordinates with the
// sign bit flipped, x in the even bits and y in the odd bits.
__device__ __forceinline__ unsigned long long morton_key(const int4 q) {
  const unsigned cx = (unsigned)(((long long)q.x + q.z) / 2) ^ 0x80000000u;
  const unsigned cy = (unsigned)(((long long)q.y + q.w) / 2) ^ 0x80000000u;
  unsigned long long mx = cx, my = cy;
  mx = (mx | (mx << 16)) & 0x0000FFFF0000FFFFull;
  mx = (mx | (mx << 8)) & 0x00FF00FF00FF00FFull;
  mx = (mx | (mx << 4)) & 0x0F0F0F0F0F0F0F0Full;
  mx = (mx | (mx << 2)) & 0x3333333333333333ull;
  mx = (mx | (mx << 1)) & 0x5555555555555555ull;
  my = (my | (my << 16)) & 0x0000FFFF0000FFFFull;
  my = (my | (my << 8)) & 0x00FF00FF00FF00FFull;
  my = (my | (my << 4)) & 0x0F0F0F0F0F0F0F0Full;
  my = (my | (my << 2)) & 0x3333333333333333ull;
  my = (my | (my << 1)) & 0x5555555555555555ull;
  return (my << 1) | mx;
}

// Keys and the identity payload; with orx, also the OR of every key with the
// first key (the span the sort's passes must cover), so the sort needs no
// separate read of the keys for it.
__global__ void k_morton_keys(const int4* b, long long n, unsigned long long* keys, unsigned* vals,
                              unsigned long long* orx = nullptr) {
  unsigned long long acc = 0;
  const unsigned long long k0 = (orx && n > 0) ? morton_key(b[0]) : 0ull;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = morton_key(b[i]);
    keys[i] = k;
    vals[i] = (unsigned)i;
    acc |= k ^ k0;
  }
  if (orx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicOr(orx, acc);
  }
}

// Highest bit in which any key differs from the first key: the LSD passes
// above it are skipped (they would not move anything).
__global__ void k_key_span(const unsigned long long* keys, long long n, unsigned long long* orx) {
  unsigned long long acc = 0;
  const unsigned long long k0 = keys[0];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    acc |= keys[i] ^ k0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicOr(orx, acc);
}

__global__ void k_gather_boxes(const int4* src, const unsigned* perm, int4* dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

__global__ void k_perm_out(const unsigned* perm, long long* out, long long n, long long add) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (long long)perm[i] + add;
}

__global__ void k_tracker_keys(const XYTracker* t, long long n, unsigned long long* keys, unsigned* vals) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    // PackKeys (event_sorter.cu:48-59)
    const unsigned ux = (unsigned)t[i].X ^ 0x80000000u;
    const unsigned uy = (unsigned)t[i].Y ^ 0x80000000u;
    keys[i] = ((unsigned long long)ux << 32) | uy;
    vals[i] = (unsigned)i;
  }
}

__global__ void k_gather_trackers(const XYTracker* src, const unsigned* perm, XYTracker* dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

__global__ void k_canon_keys(const int4* b, long long n, unsigned long long* keys, int second) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 q = b[i];
    const unsigned a = (unsigned)(second ? q.z : q.x) ^ 0x80000000u;
    const unsigned c = (unsigned)(second ? q.w : q.y) ^ 0x80000000u;
    keys[i] = ((unsigned long long)a << 32) | c;
  }
}
__global__ void k_iota(unsigned* v, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = (unsigned)i;
}
__global__ void k_canon_keys_perm(const int4* b, const unsigned* perm, long long n,
                                  unsigned long long* keys) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 q = b[perm[i]];
    keys[i] = ((unsigned long long)((unsigned)q.x ^ 0x80000000u) << 32) | ((unsigned)q.y ^ 0x80000000u);
  }
}

std::mutex g_default_mu;
gb_context* g_default = nullptr;

gb_context* default_ctx() {
  if (!g_default) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (gb_context_create(dev, 0, &g_default) != GB_OK) g_default = nullptr;
  }
  return g_default;
}

int realloc_scratch(gb_context* ctx, size_t bytes) {
  GbCtx& c = ctx->c;
  cudaStreamSynchronize(c.stream);
  if (c.tile_scratch) cudaFree(c.tile_scratch);
  c.tile_scratch = nullptr;
  if (cudaMalloc(&c.tile_scratch, bytes * (size_t)c.tile_blocks) != cudaSuccess) {
    c.tile_scr_bytes = 0;
    return GB_ERR_OOM;
  }
  c.tile_scr_bytes = bytes;
  return GB_OK;
}

}  // namespace gbi
using namespace gbi;

// ======================================================================= context
extern "C" int gb_context_create(int device, unsigned long long arena_bytes, gb_context** out) {
  if (!out) return GB_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return GB_ERR_CUDA;
  std::unique_ptr<gb_context> ctx(new gb_context());
  GbCtx& c = ctx->c;
  c.device = device;
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) return GB_ERR_CUDA;
  c.own_stream = true;
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  c.nsm = prop.multiProcessorCount;
  c.work_blocks = c.nsm * 4;
  size_t freeb = 0, totb = 0;
  cudaMemGetInfo(&freeb, &totb);
  if (arena_bytes == 0) {
    arena_bytes = (unsigned long long)(freeb / 2);
    const unsigned long long lim = 120ull << 30;
    if (arena_bytes > lim) arena_bytes = lim;
  }
  if (cudaMalloc(&c.arena, arena_bytes) != cudaSuccess) return GB_ERR_OOM;
  c.arena_cap = arena_bytes;
  if (cudaMalloc(&c.st, sizeof(DStatus)) != cudaSuccess) return GB_ERR_OOM;
  DStatus s0;
  memset(&s0, 0, sizeof(s0));
  s0.arena_base = c.arena;
  s0.arena_cap = arena_bytes;
  cudaMemcpy(c.st, &s0, sizeof(s0), cudaMemcpyHostToDevice);
  if (cudaMalloc(&c.scan_part, (GB_SCAN_BLOCKS + 1) * sizeof(long long)) != cudaSuccess) return GB_ERR_OOM;
  if (cudaMalloc(&c.dscal, 64 * sizeof(long long)) != cudaSuccess) return GB_ERR_OOM;
  if (cudaMalloc(&c.tile_counter, 64 * sizeof(long long)) != cudaSuccess) return GB_ERR_OOM;
  cudaMemset(c.dscal, 0, 64 * sizeof(long long));
  cudaMemset(c.tile_counter, 0, 64 * sizeof(long long));
  if (cudaMalloc(&c.desc, GB_NDESC * sizeof(DLayer)) != cudaSuccess) return GB_ERR_OOM;
  cudaMemset(c.desc, 0, GB_NDESC * sizeof(DLayer));
  for (int i = GB_NDESC - 1; i >= 0; --i) c.desc_free.push_back(i);
  gb_tile_setup(c);
  if (realloc_scratch(ctx.get(), 8ull << 20) != GB_OK) return GB_ERR_OOM;
  cudaDeviceSynchronize();
  if (cudaGetLastError() != cudaSuccess) return GB_ERR_CUDA;
  *out = ctx.release();
  return GB_OK;
}

extern "C" int gb_context_destroy(gb_context* ctx) {
  if (!ctx) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  cudaStreamSynchronize(c.stream);
  for (gb_layer* L : ctx->arena_layers) delete L;
  ctx->arena_layers.clear();
  cudaFree(c.arena);
  cudaFree(c.st);
  cudaFree(c.scan_part);
  cudaFree(c.dscal);
  cudaFree(c.tile_counter);
  cudaFree(c.desc);
  cudaFree(c.tile_scratch);
  if (c.io_buf) cudaFree(c.io_buf);
  if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
  gb_radix_free(c);
  if (c.own_stream) cudaStreamDestroy(c.stream);
  if (ctx == g_default) g_default = nullptr;
  delete ctx;
  return GB_OK;
}

// The context destroys only a stream it created: adopting the caller's
// stream releases the context's own one, and the caller keeps ownership.
extern "C" int gb_set_stream(gb_context* ctx, void* stream) {
  if (!ctx) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  cudaStreamSynchronize(c.stream);
  if (stream && (cudaStream_t)stream == c.stream) return GB_OK;
  cudaStream_t next = (cudaStream_t)stream;
  if (!next && cudaStreamCreateWithFlags(&next, cudaStreamNonBlocking) != cudaSuccess) return GB_ERR_CUDA;
  if (c.own_stream) cudaStreamDestroy(c.stream);
  c.stream = next;
  c.own_stream = stream == nullptr;
  return GB_OK;
}

extern "C" const char* gb_last_error(gb_context* ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }

extern "C" int gb_sync(gb_context* ctx, long long* need) {
  if (!ctx) return GB_ERR_ARG;
  cudaError_t e = cudaStreamSynchronize(ctx->c.stream);
  if (e != cudaSuccess) return set_err(ctx, GB_ERR_CUDA, cudaGetErrorString(e));
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(ctx, GB_ERR_CUDA, cudaGetErrorString(e));
  DStatus s = read_status(ctx);
  if (need) *need = s.need;
  if (s.err) {
    char buf[160];
    snprintf(buf, sizeof buf, "device status %d raised by kernel %d (need %lld)", s.err, s.where, s.need);
    ctx->c.last_error = buf;
  }
  return s.err;
}

int sync_where(gb_context* ctx, int* where, long long* need) {
  int e = gb_sync(ctx, need);
  DStatus s = read_status(ctx);
  if (where) *where = s.where;
  return e;
}

extern "C" void gb_clear_status(gb_context* ctx) {
  if (ctx) k_clear_status<<<1, 1, 0, ctx->c.stream>>>(ctx->c.st);
}

extern "C" unsigned long long gb_arena_mark(gb_context* ctx) {
  if (!ctx) return 0;
  DStatus s = read_status(ctx);
  ctx->marks.push_back({s.arena_off, ctx->seq});
  return (unsigned long long)(ctx->marks.size() - 1);
}

extern "C" int gb_arena_release(gb_context* ctx, unsigned long long mark) {
  if (!ctx || mark >= ctx->marks.size()) return GB_ERR_ARG;
  const auto m = ctx->marks[mark];
  ctx->marks.resize(mark);
  gb_launch_arena_reset(ctx->c, m.first);
  std::vector<gb_layer*> keep;
  for (gb_layer* L : ctx->arena_layers) {
    if (L->seq > m.second) {
      L->dead = true;
      drop_layer(ctx, L);
    } else {
      keep.push_back(L);
    }
  }
  ctx->arena_layers.swap(keep);
  return GB_OK;
}

extern "C" int gb_set_grid(gb_context* ctx, int g) {
  if (!ctx || g < 10 || g > 16) return GB_ERR_ARG;
  ctx->c.grid = g;
  return GB_OK;
}

extern "C" int gb_get_grid(gb_context* ctx) { return ctx ? ctx->c.grid : -1; }

extern "C" int gb_set_capacity_factor(gb_context* ctx, int factor) {
  if (!ctx || factor < 1) return GB_ERR_ARG;
  ctx->c.cap_factor = factor;
  return GB_OK;
}

extern "C" int gb_set_tile_scratch(gb_context* ctx, unsigned long long bytes) {
  if (!ctx || bytes < (1ull << 16)) return GB_ERR_ARG;
  // every CTA's scratch (and its upper half, the record region) starts on 256 bytes: the tile kernel's bulk
  // copies and 16-byte records need 16-byte aligned addresses
  return realloc_scratch(ctx, (size_t)((bytes + 511ull) & ~511ull));
}

// ======================================================================= layers
// borrow: boxes is a device pointer used in place (coff then a host pointer).
static int make_raw_layer(gb_context* ctx, const c_box* boxes, unsigned long long n,
                          const long long* coff, int ncell, bool device_src, gb_layer** out, bool borrow = false) {
  if (!ctx || !out || ncell < 1) return GB_ERR_ARG;
  *out = nullptr;
  GbCtx& c = ctx->c;
  int s = alloc_slot(ctx);
  if (s < 0) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
  gb_layer* L = new gb_layer();
  L->slot = s;
  L->d = c.desc + s;
  L->ncell = ncell;
  L->binned = 0;
  L->nbox_host = (long long)n;
  void *pb = borrow ? (void*)boxes : nullptr, *pc = nullptr, *pcell = nullptr;
  if ((!borrow && cudaMalloc(&pb, std::max<size_t>(16, n * 16)) != cudaSuccess) ||
      cudaMalloc(&pc, (size_t)(ncell + 1) * 8) != cudaSuccess ||
      cudaMalloc(&pcell, (size_t)ncell * (16 + 8 + 8 + 16) + (size_t)(ncell + 1) * 8) != cudaSuccess) {
    if (pb && !borrow) cudaFree(pb);
    if (pc) cudaFree(pc);
    c.desc_free.push_back(s);
    delete L;
    return set_err(ctx, GB_ERR_OOM, "cudaMalloc failed for a layer");
  }
  L->own_boxes = borrow ? nullptr : pb;
  L->own_coff = pc;
  L->own_cell = pcell;
  const cudaMemcpyKind kind = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (n && !borrow) cudaMemcpyAsync(pb, boxes, n * 16, kind, c.stream);
  if (coff) {
    cudaMemcpyAsync(pc, coff, (size_t)(ncell + 1) * 8, borrow ? cudaMemcpyHostToDevice : kind, c.stream);
  } else {
    long long h[2] = {0, (long long)n};
    cudaMemcpyAsync(pc, h, 16, cudaMemcpyHostToDevice, c.stream);
    cudaStreamSynchronize(c.stream);
  }
  DLayer d;
  memset(&d, 0, sizeof(d));
  d.ncell = ncell;
  d.binned = 0;
  d.boxes = (int4*)pb;
  d.coff = (long long*)pc;
  d.nbox = (long long)n;
  char* q = (char*)pcell;
  d.cbox = (int4*)q; q += (size_t)ncell * 16;
  d.cell_count = (long long*)q; q += (size_t)ncell * 8;
  d.cell_area = (long long*)q; q += (size_t)ncell * 8;
  d.win = (int4*)q; q += (size_t)ncell * 16;
  d.tbase = (long long*)q;
  cudaMemcpyAsync(L->d, &d, sizeof(d), cudaMemcpyHostToDevice, c.stream);
  cudaStreamSynchronize(c.stream);
  gb_launch_cell_bbox_fill(c, L->d, ncell);
  *out = L;
  return GB_OK;
}

namespace gbi {
int layer_over_device(gb_context* ctx, const void* d_boxes, long long n, const long long* h_offsets, int ncell,
                      gb_layer** out) {
  return make_raw_layer(ctx, (const c_box*)d_boxes, (unsigned long long)n, h_offsets, ncell, true, out, true);
}
}  // namespace gbi

extern "C" int gb_layer_from_host(gb_context* ctx, const c_box* boxes, unsigned long long n,
                                  const long long* cell_offsets, int ncell, gb_layer** out) {
  if (!cell_offsets) ncell = 1;
  return make_raw_layer(ctx, boxes, n, cell_offsets, ncell, false, out);
}

extern "C" int gb_layer_from_device(gb_context* ctx, const c_box* d_boxes, unsigned long long n,
                                    const long long* d_cell_offsets, int ncell, gb_layer** out) {
  if (!d_cell_offsets) {
    // one cell: offsets are built on the host
    return make_raw_layer(ctx, d_boxes, n, nullptr, 1, true, out);
  }
  return make_raw_layer(ctx, d_boxes, n, d_cell_offsets, ncell, true, out);
}

extern "C" int gb_layer_ncell(gb_layer* L) { return L ? L->ncell : 0; }

extern "C" int gb_layer_digest(gb_context* ctx, gb_layer* L, unsigned long long* out) {
  if (!ctx || !L || L->dead || !out || !L->binned) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, (size_t)L->ncell * 8) != cudaSuccess) return set_err(ctx, GB_ERR_OOM, "digest buffer");
  cudaMemsetAsync(d, 0, (size_t)L->ncell * 8, c.stream);
  gb_launch_digest(c, L->d, d, 1);
  cudaStreamSynchronize(c.stream);
  const cudaError_t ce = cudaMemcpy(out, d, (size_t)L->ncell * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (ce != cudaSuccess) return set_err(ctx, GB_ERR_CUDA, "digest copy");
  return gb_sync(ctx, nullptr);
}

extern "C" int gb_layer_count(gb_context* ctx, gb_layer* L, long long* total, long long* per_cell) {
  if (!ctx || !L || L->dead) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  std::vector<long long> pc(L->ncell, 0);
  DLayer d = read_desc(ctx, L);
  if (!L->binned) {
    std::vector<long long> off(L->ncell + 1);
    cudaMemcpy(off.data(), d.coff, off.size() * 8, cudaMemcpyDeviceToHost);
    for (int k = 0; k < L->ncell; ++k) pc[k] = off[k + 1] - off[k];
  } else if (L->counted) {
    if (d.cell_count) cudaMemcpy(pc.data(), d.cell_count, pc.size() * 8, cudaMemcpyDeviceToHost);
  } else {
    long long* tmp = nullptr;
    cudaMalloc(&tmp, pc.size() * 8);
    cudaMemsetAsync(tmp, 0, pc.size() * 8, c.stream);
    k_count_tiles<<<c.work_blocks, 256, 0, c.stream>>>(L->d, tmp, L->ncell, c.st);
    cudaStreamSynchronize(c.stream);
    cudaMemcpy(pc.data(), tmp, pc.size() * 8, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
  }
  long long t = 0;
  for (long long v : pc) t += v;
  if (total) *total = t;
  if (per_cell) memcpy(per_cell, pc.data(), pc.size() * 8);
  return gb_sync(ctx, nullptr);
}

extern "C" int gb_layer_to_host(gb_context* ctx, gb_layer* L, c_box* out, unsigned long long cap,
                                unsigned long long* n, long long* cell_offsets) {
  if (!ctx || !L || L->dead || !n) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  if (!L->binned) {
    DLayer d = read_desc(ctx, L);
    *n = (unsigned long long)d.nbox;
    if (cell_offsets) cudaMemcpy(cell_offsets, d.coff, (size_t)(L->ncell + 1) * 8, cudaMemcpyDeviceToHost);
    if ((unsigned long long)d.nbox > cap) return set_err(ctx, GB_ERR_CAPACITY, "output buffer too small");
    if (d.nbox && out) cudaMemcpy(out, d.boxes, (size_t)d.nbox * 16, cudaMemcpyDeviceToHost);
    return GB_OK;
  }
  gb_launch_export(c, L->d, nullptr, nullptr);
  int e = gb_sync(ctx, nullptr);
  if (e) return e;
  long long sc[4];
  cudaMemcpy(sc, c.dscal, sizeof(sc), cudaMemcpyDeviceToHost);
  *n = (unsigned long long)sc[2];
  if (cell_offsets) {
    DLayer d = read_desc(ctx, L);
    std::vector<long long> tb(L->ncell + 1);
    cudaMemcpy(tb.data(), d.tbase, tb.size() * 8, cudaMemcpyDeviceToHost);
    std::vector<long long> off(d.ntiles + 1);
    cudaMemcpy(off.data(), (void*)sc[1], (size_t)(d.ntiles + 1) * 8, cudaMemcpyDeviceToHost);
    off[d.ntiles] = sc[2];
    for (int k = 0; k <= L->ncell; ++k) cell_offsets[k] = off[std::min<long long>(tb[k], d.ntiles)];
  }
  if ((unsigned long long)sc[2] > cap) return set_err(ctx, GB_ERR_CAPACITY, "output buffer too small");
  if (sc[2] && out) cudaMemcpy(out, (void*)sc[0], (size_t)sc[2] * 16, cudaMemcpyDeviceToHost);
  return GB_OK;
}

namespace gbi {
// The layer's boxes in device memory (global coordinates): a raw layer's own
// array, or a binned layer exported into the work arena (valid until the
// arena is released past it).
int layer_device_boxes(gb_context* ctx, gb_layer* L, const c_box** d_boxes, long long* n) {
  if (!ctx || !L || L->dead || !d_boxes || !n) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  if (!L->binned) {
    DLayer d = read_desc(ctx, L);
    *d_boxes = (const c_box*)d.boxes;
    *n = d.nbox;
    return GB_OK;
  }
  gb_launch_export(c, L->d, nullptr, nullptr);
  int e = gb_sync(ctx, nullptr);
  if (e) return e;
  long long sc[4];
  cudaMemcpy(sc, c.dscal, sizeof(sc), cudaMemcpyDeviceToHost);
  *d_boxes = (const c_box*)sc[0];
  *n = sc[2];
  return GB_OK;
}
}  // namespace gbi

extern "C" void gb_layer_free(gb_context* ctx, gb_layer* L) {
  if (!ctx || !L) return;
  cudaStreamSynchronize(ctx->c.stream);
  if (L->arena_owned) {
    // arena layers are reclaimed by gb_arena_release; only the handle goes
    drop_layer(ctx, L);
    L->dead = true;
    return;
  }
  drop_layer(ctx, L);
  delete L;
}

// ======================================================================= operators
gb_layer* op_bool(gb_context* ctx, int op, gb_layer* A, gb_layer* B, int mode) {
  GbCtx& c = ctx->c;
  const int g = c.grid;
  gb_layer* Ab = binned_of(ctx, A, g);
  const bool single = op == GB_OP_MERGE || op == GB_OP_OVERLAP;
  gb_layer* Bb = (B && !single) ? binned_of(ctx, B, g) : nullptr;
  if (!Ab || (B && !single && !Bb)) return nullptr;
  gb_layer* O = new_arena_layer(ctx, A->ncell, g);
  if (!O) return nullptr;
  gb_launch_bool_setup(c, op, Ab->d, Bb ? Bb->d : nullptr, O->d, A->ncell, g, mode == 0);
  gb_launch_tile_bool(c, op, Ab->d, Bb ? Bb->d : nullptr, O->d, g, mode);
  O->counted = 1;
  return O;
}

extern "C" int gb_op_bool(gb_context* ctx, int op, gb_layer* A, gb_layer* B, gb_layer** out) {
  if (!ctx || !A || !out || A->dead || (B && B->dead)) return GB_ERR_ARG;
  if ((op < GB_OP_XOR || op > GB_OP_MERGE) && op != GB_OP_OVERLAP) return GB_ERR_ARG;
  const bool single = op == GB_OP_MERGE || op == GB_OP_OVERLAP;
  if (!single && !B) return GB_ERR_ARG;
  if (single) B = nullptr;
  if (B && B->ncell != A->ncell) return set_err(ctx, GB_ERR_ARG, "operands differ in cell count");
  *out = op_bool(ctx, op, A, B, 0);
  return *out ? GB_OK : set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
}

gb_layer* op_grow(gb_context* ctx, gb_layer* A, int E, int N, int W, int S, bool merge) {
  const int g = ctx->c.grid;
  gb_layer* R = new_arena_layer(ctx, A->ncell, g);
  if (!R) return nullptr;
  gb_launch_rebin(ctx->c, A->d, A->binned, R->d, A->ncell, g, E, N, W, S);
  if (!merge) return R;
  return op_bool(ctx, GB_OP_MERGE, R, nullptr, 0);
}

extern "C" int gb_op_grow(gb_context* ctx, gb_layer* A, int32_t E, int32_t N, int32_t W, int32_t S,
                          gb_layer** out) {
  if (!ctx || !A || !out || A->dead) return GB_ERR_ARG;
  *out = op_grow(ctx, A, E, N, W, S, true);
  return *out ? GB_OK : set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
}

// SIZE(-t): R = P - ((F - P) (+) [-t,t]^2), F = cell bbox grown by t.
gb_layer* op_erode(gb_context* ctx, gb_layer* P, int t, gb_layer** frame_out, gb_layer** comp_out) {
  GbCtx& c = ctx->c;
  const int g = c.grid;
  gb_layer* Pb = binned_of(ctx, P, g);
  if (!Pb) return nullptr;
  gb_layer* F = new_arena_layer(ctx, P->ncell, g);
  if (!F) return nullptr;
  F->binned = 0;
  k_desc_init<<<1, 1, 0, c.stream>>>(F->d, P->ncell, g, 0);
  k_make_frame<<<1, 1, 0, c.stream>>>(Pb->d, F->d, P->ncell, t, c.st);
  k_fill_frame<<<(P->ncell + 255) / 256, 256, 0, c.stream>>>(Pb->d, F->d, P->ncell, t, c.st);
  gb_layer* Q = op_bool(ctx, GB_OP_NOT, F, Pb, 0);
  if (!Q) return nullptr;
  if (frame_out) *frame_out = F;
  if (comp_out) *comp_out = Q;
  gb_layer* D = op_grow(ctx, Q, t, t, t, t, false);
  if (!D) return nullptr;
  return op_bool(ctx, GB_OP_NOT, Pb, D, 0);
}

extern "C" int gb_op_size(gb_context* ctx, gb_layer* A, int32_t s, gb_layer** out) {
  if (!ctx || !A || !out || A->dead) return GB_ERR_ARG;
  if (s > 0) *out = op_grow(ctx, A, s, s, s, s, true);
  else if (s == 0) *out = op_bool(ctx, GB_OP_MERGE, A, nullptr, 0);
  else *out = op_erode(ctx, A, -s);
  return *out ? GB_OK : set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
}

extern "C" int gb_op_area(gb_context* ctx, gb_layer* A, long long* area_per_cell) {
  if (!ctx || !A || A->dead || !area_per_cell) return GB_ERR_ARG;
  gb_layer* O = op_bool(ctx, GB_OP_MERGE, A, nullptr, 1);
  if (!O) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
  int e = gb_sync(ctx, nullptr);
  if (e) return e;
  DLayer d = read_desc(ctx, O);
  cudaMemcpy(area_per_cell, d.cell_area, (size_t)A->ncell * 8, cudaMemcpyDeviceToHost);
  return GB_OK;
}

// ======================================================================= retry wrapper
// Host-synchronous entry points run their device sequence, check the device
// status, and on a capacity error enlarge the failing resource and run again.
template <typename F>
int run_retry(gb_context* ctx, F&& body) {
  int e = GB_OK;
  for (int attempt = 0; attempt < 6; ++attempt) {
    gb_clear_status(ctx);
    const unsigned long long mk = gb_arena_mark(ctx);
    e = body();
    int where = 0;
    long long need = 0;
    const int dev = sync_where(ctx, &where, &need);
    if (dev != GB_OK) e = dev;  // the device status explains a failing body
    if (e == GB_OK) {
      gb_arena_release(ctx, mk);
      return GB_OK;
    }
    gb_arena_release(ctx, mk);
    if (e != GB_ERR_CAPACITY) break;
    if (where == 20) {  // tile scratch
      if (realloc_scratch(ctx, ctx->c.tile_scr_bytes * 4) != GB_OK) return GB_ERR_OOM;
    } else if (where == 21) {  // output pool
      ctx->c.cap_factor *= 2;
    } else {
      return set_err(ctx, GB_ERR_OOM, "work arena too small for this operation");
    }
  }
  gb_clear_status(ctx);
  return e;
}

int gb_run_retry(gb_context* ctx, const std::function<int()>& body) { return run_retry(ctx, body); }

// ======================================================================= connectivity
// Grid for candidate pairs of a one-cell raw layer: about 32 boxes per tile.
static int pair_grid(gb_context* ctx, gb_layer* L, long long n) {
  DLayer d = read_desc(ctx, L);
  int4 bb;
  cudaMemcpy(&bb, d.cbox, 16, cudaMemcpyDeviceToHost);
  const double W = (double)bb.z - bb.x + 1, H = (double)bb.w - bb.y + 1;
  const double cell = std::sqrt(W * H * 32.0 / (double)(n > 0 ? n : 1));
  int g = 4;
  while (g < 30 && (double)(1ll << g) < cell) ++g;
  return g;
}

extern "C" int gb_components(gb_context* ctx, const c_box* boxes, unsigned long long n,
                             long long* ncomp, long long* labels) {
  if (!ctx || !ncomp) return GB_ERR_ARG;
  if (n == 0) { *ncomp = 0; return GB_OK; }
  if (n > 0x7fffffffull) return set_err(ctx, GB_ERR_ARG, "too many boxes for int32 indices");
  GbCtx& c = ctx->c;
  gb_layer* L = nullptr;
  int e = gb_layer_from_host(ctx, boxes, n, nullptr, 1, &L);
  if (e) return e;
  e = gb_sync(ctx, nullptr);
  if (e) { gb_layer_free(ctx, L); return e; }
  const int g = pair_grid(ctx, L, (long long)n);
  int* parent = nullptr;
  unsigned char* touched = nullptr;
  long long* lab = nullptr;
  long long* map = nullptr;
  int* flag = nullptr;
  long long* nc = nullptr;
  cudaMalloc(&parent, n * 4);
  cudaMalloc(&touched, n);
  cudaMalloc(&lab, n * 8);
  cudaMalloc(&map, n * 8);
  cudaMalloc(&flag, n * 4);
  cudaMalloc(&nc, 8);
  if (!parent || !touched || !lab || !map || !flag || !nc) {
    e = set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in gb_components");
  } else {
    e = run_retry(ctx, [&]() -> int {
      gb_layer* B = new_arena_layer(ctx, 1, g);
      if (!B) return GB_ERR_CAPACITY;
      gb_launch_bin_index(c, L->d, B->d, 1, g);
      gb_launch_components(c, L->d, B->d, parent, touched, lab, (long long)n, nc, flag, map);
      return GB_OK;
    });
    if (e == GB_OK) {
      cudaMemcpy(ncomp, nc, 8, cudaMemcpyDeviceToHost);
      if (labels) cudaMemcpy(labels, lab, n * 8, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(parent); cudaFree(touched); cudaFree(lab); cudaFree(map); cudaFree(flag); cudaFree(nc);
  gb_layer_free(ctx, L);
  return e;
}

// ComputeInteractions / FindSingletons (pnummerge.f90:388-562) and
// CertifyHealing (design_impl.f90:35-56) on the GPU.
extern "C" int gb_interactions(gb_context* ctx, const c_box* boxes, unsigned long long n, long long* strict_pairs,
                               long long* singletons, unsigned char* is_singleton) {
  if (!ctx || (n && !boxes)) return GB_ERR_ARG;
  if (n > 0x7fffffffull) return set_err(ctx, GB_ERR_ARG, "too many boxes for int32 indices");
  if (n == 0) {
    if (strict_pairs) *strict_pairs = 0;
    if (singletons) *singletons = 0;
    return GB_OK;
  }
  GbCtx& c = ctx->c;
  gb_layer* L = nullptr;
  int e = gb_layer_from_host(ctx, boxes, n, nullptr, 1, &L);
  if (e) return e;
  e = gb_sync(ctx, nullptr);
  if (e) { gb_layer_free(ctx, L); return e; }
  const int g = pair_grid(ctx, L, (long long)n);
  unsigned char* touched = nullptr;
  unsigned char* mask = nullptr;
  unsigned long long* cnt = nullptr;
  cudaMalloc(&touched, n);
  cudaMalloc(&cnt, 16);
  if (is_singleton) cudaMalloc(&mask, n);
  if (!touched || !cnt || (is_singleton && !mask)) {
    e = set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in gb_interactions");
  } else {
    e = run_retry(ctx, [&]() -> int {
      gb_layer* B = new_arena_layer(ctx, 1, g);
      if (!B) return GB_ERR_CAPACITY;
      gb_launch_bin_index(c, L->d, B->d, 1, g);
      gb_launch_pair_stats(c, L->d, B->d, g, touched, (long long)n, cnt, cnt + 1, mask);
      return GB_OK;
    });
    if (e == GB_OK) {
      unsigned long long h[2];
      cudaMemcpy(h, cnt, 16, cudaMemcpyDeviceToHost);
      if (strict_pairs) *strict_pairs = (long long)h[0];
      if (singletons) *singletons = (long long)h[1];
      if (is_singleton) cudaMemcpy(is_singleton, mask, n, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(touched); cudaFree(mask); cudaFree(cnt);
  gb_layer_free(ctx, L);
  return e;
}

extern "C" int gb_certify_healing(gb_context* ctx, const c_box* boxes, unsigned long long n, int* healed) {
  if (!ctx || !healed) return GB_ERR_ARG;
  if (n < 2) { *healed = 1; return GB_OK; }
  long long pairs = 0;
  const int e = gb_interactions(ctx, boxes, n, &pairs, nullptr, nullptr);
  if (!e) *healed = pairs == 0 ? 1 : 0;
  return e;
}

__global__ void k_label_keys(const long long* lab, long long n, unsigned long long* keys, unsigned* vals) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    keys[i] = (unsigned long long)lab[i];
    vals[i] = (unsigned)i;
  }
}

// off[l] = first position of label l in the label-sorted keys, off[R+1] = n
// (labels 1..R all occur; label 0 may not).
__global__ void k_label_offsets(const unsigned long long* keys, long long n, long long R, long long* off) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long prev = i == 0 ? -1 : (long long)keys[i - 1];
    const long long cur = i == n ? R + 1 : (long long)keys[i];
    for (long long l = prev + 1; l <= cur; ++l) off[l] = i;
  }
}

// Union area per PNUM component (calculate_union_area_by_polygon,
// design.f90:854-935): the boxes are grouped by component label on the
// device (labels of gb_components, radix-sorted), each group becomes one cell
// of a layer, and the per-cell union area is the component's area; cell 0
// holds the singletons, whose boxes are disjoint.
extern "C" int gb_component_areas(gb_context* ctx, const c_box* boxes, unsigned long long n, long long* areas,
                                  unsigned long long cap, long long* nlabels) {
  if (!ctx || !nlabels || (n && !boxes)) return GB_ERR_ARG;
  if (n > 0x7fffffffull) return set_err(ctx, GB_ERR_ARG, "too many boxes for int32 indices");
  if (n == 0) {
    *nlabels = 1;
    if (cap < 1) return GB_ERR_CAPACITY;
    if (areas) areas[0] = 0;
    return GB_OK;
  }
  GbCtx& c = ctx->c;
  gb_layer* L = nullptr;
  int e = gb_layer_from_host(ctx, boxes, n, nullptr, 1, &L);
  if (e) return e;
  e = gb_sync(ctx, nullptr);
  if (e) { gb_layer_free(ctx, L); return e; }
  const int g = pair_grid(ctx, L, (long long)n);
  int* parent = nullptr;
  unsigned char* touched = nullptr;
  long long *lab = nullptr, *map = nullptr, *nc = nullptr, *off = nullptr;
  int* flag = nullptr;
  unsigned long long *keys = nullptr, *kt = nullptr;
  unsigned *vals = nullptr, *vt = nullptr;
  int4* sorted = nullptr;
  cudaMalloc(&parent, n * 4);
  cudaMalloc(&touched, n);
  cudaMalloc(&lab, n * 8);
  cudaMalloc(&map, n * 8);
  cudaMalloc(&flag, n * 4);
  cudaMalloc(&nc, 8);
  cudaMalloc(&keys, n * 8);
  cudaMalloc(&kt, n * 8);
  cudaMalloc(&vals, n * 4);
  cudaMalloc(&vt, n * 4);
  cudaMalloc(&sorted, n * 16);
  gb_layer* G = nullptr;
  if (!parent || !touched || !lab || !map || !flag || !nc || !keys || !kt || !vals || !vt || !sorted) {
    e = set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in gb_component_areas");
  } else {
    e = run_retry(ctx, [&]() -> int {
      gb_layer* B = new_arena_layer(ctx, 1, g);
      if (!B) return GB_ERR_CAPACITY;
      gb_launch_bin_index(c, L->d, B->d, 1, g);
      gb_launch_components(c, L->d, B->d, parent, touched, lab, (long long)n, nc, flag, map);
      return GB_OK;
    });
  }
  long long R = 0;
  if (e == GB_OK) {
    long long ncomp = 0, nsingle = 0;
    cudaMemcpy(&ncomp, nc, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(&nsingle, c.dscal + 4, 8, cudaMemcpyDeviceToHost);
    R = ncomp - nsingle;
    *nlabels = R + 1;
    if (cap < (unsigned long long)(R + 1)) e = GB_ERR_CAPACITY;
  }
  if (e == GB_OK) {
    cudaMalloc(&off, (size_t)(R + 2) * 8);
    if (!off) e = set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in gb_component_areas");
  }
  if (e == GB_OK) {
    int bits = 1;
    while (bits < 63 && (R >> bits)) ++bits;
    k_label_keys<<<c.work_blocks, 256, 0, c.stream>>>(lab, (long long)n, keys, vals);
    if (gb_radix_sort_pairs(c, keys, vals, (long long)n, bits, kt, vt) < 0)
      e = set_err(ctx, GB_ERR_INTERNAL, "radix sort setup failed");
  }
  if (e == GB_OK) {
    k_gather_boxes<<<c.work_blocks, 256, 0, c.stream>>>((const int4*)L->own_boxes, vals, sorted, (long long)n);
    k_label_offsets<<<c.work_blocks, 256, 0, c.stream>>>(keys, (long long)n, R, off);
    c.launches += 3;
    e = gb_sync(ctx, nullptr);
    if (!e) e = gb_layer_from_device(ctx, (const c_box*)sorted, n, off, (int)(R + 1), &G);
    if (!e) e = areas ? gb_op_area(ctx, G, areas) : GB_OK;
  }
  if (G) gb_layer_free(ctx, G);
  cudaFree(parent); cudaFree(touched); cudaFree(lab); cudaFree(map); cudaFree(flag); cudaFree(nc);
  cudaFree(keys); cudaFree(kt); cudaFree(vals); cudaFree(vt); cudaFree(sorted); cudaFree(off);
  gb_layer_free(ctx, L);
  return e;
}

// ======================================================================= sorts
// Sorts keys with their payloads over the key bits that differ.  d_span, when
// given, already holds the OR of every key with the first key (computed where
// the keys were made); otherwise one pass over the keys computes it.
static int sort_keys_perm(gb_context* ctx, unsigned long long* dkeys, unsigned* dvals, long long n,
                          unsigned long long* d_span = nullptr) {
  GbCtx& c = ctx->c;
  unsigned long long* orx = d_span;
  if (!orx) {
    cudaMalloc(&orx, 8);
    cudaMemsetAsync(orx, 0, 8, c.stream);
    k_key_span<<<c.work_blocks, 256, 0, c.stream>>>(dkeys, n, orx);
  }
  unsigned long long span = 0;
  cudaMemcpyAsync(&span, orx, 8, cudaMemcpyDeviceToHost, c.stream);
  cudaStreamSynchronize(c.stream);
  if (!d_span) cudaFree(orx);
  int bits = 0;
  while (bits < 64 && (span >> bits)) ++bits;
  if (bits == 0) return GB_OK;
  unsigned long long* kt = nullptr;
  unsigned* vt = nullptr;
  if (cudaMalloc(&kt, (size_t)n * 8) != cudaSuccess || cudaMalloc(&vt, (size_t)n * 4) != cudaSuccess) {
    if (kt) cudaFree(kt);
    return set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in sort");
  }
  int p = gb_radix_sort_pairs(c, dkeys, dvals, n, bits, kt, vt);
  cudaStreamSynchronize(c.stream);
  cudaFree(kt);
  cudaFree(vt);
  return p < 0 ? set_err(ctx, GB_ERR_INTERNAL, "radix sort setup failed") : gb_sync(ctx, nullptr);
}

static bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static int morton_sort_impl(gb_context* ctx, c_box* boxes, long long n, int sort_boxes,
                            unsigned long long* keys_out, long long* perm_out, long long perm_add,
                            bool dev_io) {
  GbCtx& c = ctx->c;
  if (n <= 0) return GB_OK;
  int4* db = nullptr;
  int4* db2 = nullptr;
  unsigned long long* dk = nullptr;
  unsigned* dv = nullptr;
  int e = GB_OK;
  if (dev_io) db = (int4*)boxes;
  else if (cudaMalloc(&db, (size_t)n * 16) != cudaSuccess) return GB_ERR_OOM;
  // keys, then one word for their span
  if (cudaMalloc(&dk, (size_t)(n + 1) * 8) != cudaSuccess || cudaMalloc(&dv, (size_t)n * 4) != cudaSuccess) {
    e = GB_ERR_OOM;
    goto done;
  }
  if (!dev_io) cudaMemcpyAsync(db, boxes, (size_t)n * 16, cudaMemcpyHostToDevice, c.stream);
  cudaMemsetAsync(dk + n, 0, 8, c.stream);
  k_morton_keys<<<c.work_blocks, 256, 0, c.stream>>>(db, n, dk, dv, dk + n);
  e = sort_keys_perm(ctx, dk, dv, n, dk + n);
  if (e) goto done;
  if (keys_out) cudaMemcpy(keys_out, dk, (size_t)n * 8, dev_io ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
  if (perm_out) {
    long long* dp = nullptr;
    if (dev_io) dp = perm_out;
    else if (cudaMalloc(&dp, (size_t)n * 8) != cudaSuccess) { e = GB_ERR_OOM; goto done; }
    k_perm_out<<<c.work_blocks, 256, 0, c.stream>>>(dv, dp, n, perm_add);
    if (!dev_io) {
      cudaMemcpyAsync(perm_out, dp, (size_t)n * 8, cudaMemcpyDeviceToHost, c.stream);
      cudaStreamSynchronize(c.stream);
      cudaFree(dp);
    }
  }
  if (sort_boxes) {
    if (cudaMalloc(&db2, (size_t)n * 16) != cudaSuccess) { e = GB_ERR_OOM; goto done; }
    k_gather_boxes<<<c.work_blocks, 256, 0, c.stream>>>(db, dv, db2, n);
    cudaMemcpyAsync(boxes, db2, (size_t)n * 16, dev_io ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                    c.stream);
  }
  cudaStreamSynchronize(c.stream);
done:
  if (!dev_io && db) cudaFree(db);
  if (db2) cudaFree(db2);
  if (dk) cudaFree(dk);
  if (dv) cudaFree(dv);
  return e;
}

extern "C" int gb_morton_sort(gb_context* ctx, c_box* boxes, long long n, int sort_boxes,
                              unsigned long long* keys_out, long long* perm) {
  if (!ctx || (n > 0 && !boxes)) return GB_ERR_ARG;
  if (n > 0xffffffffll) return GB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return morton_sort_impl(ctx, boxes, n, sort_boxes, keys_out, perm, 0, false);
}

extern "C" int gb_canonical_sort(gb_context* ctx, c_box* boxes, long long n) {
  if (!ctx || (n > 0 && !boxes)) return GB_ERR_ARG;
  if (n <= 1) return GB_OK;
  GbCtx& c = ctx->c;
  int4 *db = nullptr, *db2 = nullptr;
  unsigned long long* dk = nullptr;
  unsigned* dv = nullptr;
  int e = GB_OK;
  if (cudaMalloc(&db, (size_t)n * 16) || cudaMalloc(&db2, (size_t)n * 16) || cudaMalloc(&dk, (size_t)n * 8) ||
      cudaMalloc(&dv, (size_t)n * 4)) {
    e = GB_ERR_OOM;
  } else {
    cudaMemcpyAsync(db, boxes, (size_t)n * 16, cudaMemcpyHostToDevice, c.stream);
    // LSD over the two 64-bit halves: first (x2, y2), then (x1, y1), both stable.
    k_canon_keys<<<c.work_blocks, 256, 0, c.stream>>>(db, n, dk, 1);
    k_iota<<<c.work_blocks, 256, 0, c.stream>>>(dv, n);
    e = sort_keys_perm(ctx, dk, dv, n);
    if (!e) {
      k_canon_keys_perm<<<c.work_blocks, 256, 0, c.stream>>>(db, dv, n, dk);
      e = sort_keys_perm(ctx, dk, dv, n);
    }
    if (!e) {
      k_gather_boxes<<<c.work_blocks, 256, 0, c.stream>>>(db, dv, db2, n);
      cudaMemcpyAsync(boxes, db2, (size_t)n * 16, cudaMemcpyDeviceToHost, c.stream);
      cudaStreamSynchronize(c.stream);
    }
  }
  cudaFree(db); cudaFree(db2); cudaFree(dk); cudaFree(dv);
  return e;
}

extern "C" int32_t gb_um_to_dbu(double r) { return (int32_t)(1000.0 * r); }

extern "C" int gb_radix_sort_device(gb_context* ctx, unsigned long long* d_keys, unsigned* d_vals, long long n,
                                    int bits, unsigned long long* d_keys_tmp, unsigned* d_vals_tmp) {
  if (!ctx || n < 0 || bits < 1 || bits > 64 || (n > 1 && (!d_keys || !d_vals || !d_keys_tmp || !d_vals_tmp)))
    return -GB_ERR_ARG;
  const int p = gb_radix_sort_pairs(ctx->c, d_keys, d_vals, n, bits, d_keys_tmp, d_vals_tmp);
  if (p == -2) return -set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in radix sort");
  return p < 0 ? -set_err(ctx, GB_ERR_INTERNAL, "radix sort setup failed") : p;
}

extern "C" int gb_radix_sort_device_cfg(gb_context* ctx, unsigned long long* d_keys, unsigned* d_vals, long long n,
                                        int bits, unsigned long long* d_keys_tmp, unsigned* d_vals_tmp, int passes,
                                        int tile) {
  if (!ctx || n < 0 || bits < 1 || bits > 64 || (n > 1 && (!d_keys || !d_vals || !d_keys_tmp || !d_vals_tmp)))
    return -GB_ERR_ARG;
  const int p = gb_radix_sort_pairs(ctx->c, d_keys, d_vals, n, bits, d_keys_tmp, d_vals_tmp, passes, tile);
  if (p == -2) return -set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in radix sort");
  return p < 0 ? -set_err(ctx, GB_ERR_ARG, "radix sort configuration not available") : p;
}

extern "C" int gb_radix_autotune(gb_context* ctx, const unsigned long long* d_keys, const unsigned* d_vals,
                                 long long n, int bits, int* passes, int* tile, float* ms) {
  if (!ctx || n < 2 || bits < 1 || bits > 64 || !d_keys || !d_vals) return GB_ERR_ARG;
  const int r = gb_radix_tune(ctx->c, d_keys, d_vals, n, bits, passes, tile, ms);
  if (r == -2) return set_err(ctx, GB_ERR_OOM, "cudaMalloc failed in radix autotune");
  if (r < 0) return set_err(ctx, GB_ERR_INTERNAL, "radix autotune found no configuration");
  return gb_sync(ctx, nullptr);
}

extern "C" void gb_radix_tuning_reset(void) { gb_radix_forget_tuning(); }

extern "C" int gb_morton_keys_device(gb_context* ctx, const c_box* d_boxes, long long n, unsigned long long* d_keys,
                                     unsigned* d_vals) {
  if (!ctx || n < 0 || (n > 0 && (!d_boxes || !d_keys || !d_vals))) return GB_ERR_ARG;
  k_morton_keys<<<ctx->c.work_blocks, 256, 0, ctx->c.stream>>>((const int4*)d_boxes, n, d_keys, d_vals);
  return GB_OK;
}

// ======================================================================= drop-ins
static int host_bool(gb_context* ctx, int control, long value, const c_box* A, unsigned long AN,
                     const c_box* B, unsigned long BN, std::vector<c_box>& res) {
  gb_layer* LA = nullptr;
  gb_layer* LB = nullptr;
  int e = gb_layer_from_host(ctx, A, AN, nullptr, 1, &LA);
  if (!e) e = gb_layer_from_host(ctx, B, BN, nullptr, 1, &LB);
  if (e) {
    if (LA) gb_layer_free(ctx, LA);
    return e;
  }
  e = run_retry(ctx, [&]() -> int {
    gb_layer* O = nullptr;
    int r;
    if (control == GB_OP_SIZE) r = gb_op_size(ctx, LA, (int32_t)value, &O);
    else if (control == GB_OP_MERGE) r = gb_op_bool(ctx, GB_OP_MERGE, LA, nullptr, &O);
    else r = gb_op_bool(ctx, (int)control, LA, LB, &O);
    if (r) return r;
    unsigned long long n = 0;
    r = gb_layer_to_host(ctx, O, nullptr, 0, &n, nullptr);
    if (r && r != GB_ERR_CAPACITY) return r;
    res.resize(n);
    return gb_layer_to_host(ctx, O, res.data(), n, &n, nullptr);
  });
  gb_layer_free(ctx, LA);
  gb_layer_free(ctx, LB);
  return e;
}

extern "C" void PerformBoostPolygonOperation(const struct c_box* input_A, unsigned long AN,
                                             const struct c_box* input_B, unsigned long BN,
                                             struct c_box* output, unsigned long* outN,
                                             unsigned long control_parameter, long control_value) {
  if (!outN) return;
  *outN = 0;
  if (AN == 0 && BN == 0) return;  // boost_polygon_api.cpp:107-110
  if (control_parameter > 5) return;  // unknown control: outN = 0 (:138-140)
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_context* ctx = default_ctx();
  if (!ctx) {
    fprintf(stderr, "PerformBoostPolygonOperation: no CUDA context\n");
    return;
  }
  std::vector<c_box> res;
  int e = host_bool(ctx, (int)control_parameter, control_value, input_A, AN, input_B, BN, res);
  if (e) {
    fprintf(stderr, "PerformBoostPolygonOperation: status %d (%s)\n", e, gb_last_error(ctx));
    return;
  }
  const unsigned long mx = std::max(AN, BN);
  const unsigned long cap = control_parameter == GB_OP_AND ? 10 * mx : 4 * mx;
  if (res.size() > cap) {
    fprintf(stderr, "PerformBoostPolygonOperation: result has %zu boxes, caller buffer holds %lu\n",
            res.size(), cap);
    return;
  }
  if (!res.empty()) memcpy(output, res.data(), res.size() * sizeof(c_box));
  *outN = (unsigned long)res.size();
}

extern "C" void PerformBoostPolygonMerge(const struct c_box* input, unsigned long N,
                                         struct c_box* output, unsigned long* outN) {
  if (!outN) return;
  *outN = 0;
  if (N == 0) return;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_context* ctx = default_ctx();
  if (!ctx) return;
  std::vector<c_box> res;
  int e = host_bool(ctx, GB_OP_MERGE, 0, input, N, nullptr, 0, res);
  if (e) {
    fprintf(stderr, "PerformBoostPolygonMerge: status %d (%s)\n", e, gb_last_error(ctx));
    return;
  }
  if (res.size() > 2 * N) {
    fprintf(stderr, "PerformBoostPolygonMerge: result has %zu boxes, caller buffer holds %lu\n",
            res.size(), 2 * N);
    return;
  }
  if (!res.empty()) memcpy(output, res.data(), res.size() * sizeof(c_box));
  *outN = (unsigned long)res.size();
}

extern "C" void thrust_sort_boxes_direct(struct c_box* boxes, int64_t n) {
  if (n <= 1 || !boxes) return;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_context* ctx = default_ctx();
  if (!ctx) return;
  int e = morton_sort_impl(ctx, boxes, n, 1, nullptr, nullptr, 0, is_device_ptr(boxes));
  if (e) fprintf(stderr, "thrust_sort_boxes_direct: status %d\n", e);
}

extern "C" void thrust_sort_boxes_indirect(struct c_box* boxes, int64_t* indices, int64_t n) {
  if (n <= 1 || !boxes || !indices) return;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_context* ctx = default_ctx();
  if (!ctx) return;
  const bool dev = is_device_ptr(boxes);
  int e = morton_sort_impl(ctx, boxes, n, 0, nullptr, (long long*)indices, 1, dev);
  if (e) fprintf(stderr, "thrust_sort_boxes_indirect: status %d\n", e);
}

extern "C" void device_event_sort(struct XYTracker* arr, int64_t n) {
  if (n <= 1 || !arr) return;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_context* ctx = default_ctx();
  if (!ctx) return;
  GbCtx& c = ctx->c;
  const bool dev = is_device_ptr(arr);
  XYTracker *dt = nullptr, *dt2 = nullptr;
  unsigned long long* dk = nullptr;
  unsigned* dv = nullptr;
  if (dev) dt = arr;
  else cudaMalloc(&dt, (size_t)n * sizeof(XYTracker));
  cudaMalloc(&dt2, (size_t)n * sizeof(XYTracker));
  cudaMalloc(&dk, (size_t)n * 8);
  cudaMalloc(&dv, (size_t)n * 4);
  if (dt && dt2 && dk && dv) {
    if (!dev) cudaMemcpyAsync(dt, arr, (size_t)n * sizeof(XYTracker), cudaMemcpyHostToDevice, c.stream);
    k_tracker_keys<<<c.work_blocks, 256, 0, c.stream>>>(dt, n, dk, dv);
    if (sort_keys_perm(ctx, dk, dv, n) == GB_OK) {
      k_gather_trackers<<<c.work_blocks, 256, 0, c.stream>>>(dt, dv, dt2, n);
      cudaMemcpyAsync(arr, dt2, (size_t)n * sizeof(XYTracker),
                      dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c.stream);
      cudaStreamSynchronize(c.stream);
    } else {
      fprintf(stderr, "device_event_sort: sort failed (%s)\n", gb_last_error(ctx));
    }
  } else {
    fprintf(stderr, "device_event_sort: cudaMalloc failed\n");
  }
  if (!dev && dt) cudaFree(dt);
  if (dt2) cudaFree(dt2);
  if (dk) cudaFree(dk);
  if (dv) cudaFree(dv);
}
