// gb_deck.cu -- deck-level execution: the OP1 ring-check chain on device
// layers, CUDA-graph capture of operator chains, and kernel profiling.
//
// OP1 (op_template.m4:14-22, the README ring check):
//   t1:P_1 = d1:P GROW t1:nothing a a a a
//   t1:P_2 = d1:P SIZE t1:nothing -a
//   t1:P_outer_ring = t1:P_1 ~ d1:P
//   t1:P_inner_ring = d1:P ~ t1:P_2
//   t1:P_ring_and1 = t1:P_outer_ring * d1:P
//   t1:P_ring_intersection = t1:P_outer_ring * t1:P_inner_ring
//   ASSERT_ZERO on the last two
// Every operator works on all cells of a layer at once, so a batch of
// independent cells is one launch per kernel, and the whole chain has no
// host round trip: it can be captured once and replayed as a CUDA graph.
#include <cstring>
#include <vector>

#include "gbool.h"
#include <algorithm>

#include "gb_internal.h"

#define GB_GRID_TUNE_MIN 13  // smallest tile grid (log2 dbu) the slab-height tuner tries

using namespace gbi;

struct gb_graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  unsigned long long arena_off = 0;
  long long kernels = 0;
};

__global__ void k_zero_prof(long long* ctr) {
  ctr[8] = 0;
  ctr[9] = 0;
}
__global__ void k_arena_to(DStatus* st, unsigned long long off) { st->arena_off = off; }

// on = 1: start a profiling window (event pairs and byte counters reset);
// on = 2: reset only the byte counters (keeps event pairs captured in a graph);
// on = 0: stop recording events.
extern "C" int gb_profile(gb_context* ctx, int on) {
  if (!ctx) return GB_ERR_ARG;
  if (on != 2) {
    ctx->c.prof = on != 0;
    ctx->c.prof_used = 0;
  }
  k_zero_prof<<<1, 1, 0, ctx->c.stream>>>(ctx->c.tile_counter);
  return GB_OK;
}

extern "C" int gb_profile_read(gb_context* ctx, double* ms_total, long long* launches,
                               long long* bytes_in, long long* bytes_out) {
  if (!ctx) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  cudaStreamSynchronize(c.stream);
  double ms = 0;
  long long n = 0;
  for (size_t i = 0; i + 1 < c.prof_used; i += 2) {
    float t = 0;
    if (cudaEventElapsedTime(&t, c.prof_ev[i], c.prof_ev[i + 1]) == cudaSuccess) {
      ms += t;
      ++n;
    }
  }
  cudaGetLastError();
  long long ctr[10];
  cudaMemcpy(ctr, c.tile_counter, sizeof(ctr), cudaMemcpyDeviceToHost);
  if (ms_total) *ms_total = ms;
  if (launches) *launches = n;
  if (bytes_in) *bytes_in = ctr[8];
  if (bytes_out) *bytes_out = ctr[9];
  return GB_OK;
}

// Per-phase cycle counters of the scanline kernel (diagnostics): on != 0
// enables them; gb_tile_timing_read returns [cycA, cycB, cycC, cycD, tiles,
// pieces, sub-bands, strip pieces] summed over CTAs since enabling, the
// sub-band step counters, per sub-band-count bucket the tiles and their
// phase-C cycles, and the sub-bands with and without spilled column words and
// their cycles (40 values).
__global__ void k_zero_timing(long long* ctr) {
  for (int i = 16; i < 56; ++i) ctr[i] = 0;
}
extern "C" int gb_tile_timing(gb_context* ctx, int on) {
  if (!ctx) return GB_ERR_ARG;
  ctx->c.timing = on != 0;
  k_zero_timing<<<1, 1, 0, ctx->c.stream>>>(ctx->c.tile_counter);
  return GB_OK;
}
extern "C" int gb_tile_timing_read(gb_context* ctx, long long* out8) {
  if (!ctx || !out8) return GB_ERR_ARG;
  cudaStreamSynchronize(ctx->c.stream);
  cudaMemcpy(out8, ctx->c.tile_counter + 16, 40 * sizeof(long long), cudaMemcpyDeviceToHost);
  return GB_OK;
}

extern "C" long long gb_launch_count(gb_context* ctx) { return ctx ? ctx->c.launches : 0; }

extern "C" int gb_graph_begin(gb_context* ctx) {
  if (!ctx) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  DStatus s = read_status(ctx);
  ctx->graph_arena_off = s.arena_off;
  if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return set_err(ctx, GB_ERR_CUDA, "cudaStreamBeginCapture failed");
  // every replay starts allocating from the same arena offset
  k_arena_to<<<1, 1, 0, c.stream>>>(c.st, s.arena_off);
  return GB_OK;
}

extern "C" int gb_graph_end(gb_context* ctx, gb_graph** out) {
  if (!ctx || !out) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  gb_graph* G = new gb_graph();
  G->arena_off = ctx->graph_arena_off;
  if (cudaStreamEndCapture(c.stream, &G->g) != cudaSuccess) {
    delete G;
    cudaGetLastError();
    return set_err(ctx, GB_ERR_CUDA, "cudaStreamEndCapture failed");
  }
  if (cudaGraphInstantiate(&G->ex, G->g, 0) != cudaSuccess) {
    cudaGraphDestroy(G->g);
    delete G;
    cudaGetLastError();
    return set_err(ctx, GB_ERR_CUDA, "cudaGraphInstantiate failed");
  }
  size_t nn = 0;
  cudaGraphGetNodes(G->g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) cudaGraphGetNodes(G->g, nodes.data(), &nn);
  for (auto& n : nodes) {
    cudaGraphNodeType t;
    cudaGraphNodeGetType(n, &t);
    if (t == cudaGraphNodeTypeKernel) ++G->kernels;
  }
  *out = G;
  return GB_OK;
}

extern "C" int gb_graph_launch(gb_context* ctx, gb_graph* G) {
  if (!ctx || !G) return GB_ERR_ARG;
  return cudaGraphLaunch(G->ex, ctx->c.stream) == cudaSuccess ? GB_OK
                                                               : set_err(ctx, GB_ERR_CUDA, "cudaGraphLaunch failed");
}

extern "C" long long gb_graph_kernels(gb_graph* G) { return G ? G->kernels : 0; }

extern "C" void gb_graph_destroy(gb_graph* G) {
  if (!G) return;
  if (G->ex) cudaGraphExecDestroy(G->ex);
  if (G->g) cudaGraphDestroy(G->g);
  delete G;
}

// The OP1 chain (op_template.m4:14-22) on every cell of P, one scanline pass
// per operator.  *F / *Q (optional) receive the erosion's frame and complement.
static int op1_chain(gb_context* ctx, gb_layer* P, int32_t a, gb_layer** outs, gb_layer** F, gb_layer** Q) {
  gb_layer* p1 = a >= 0 ? op_grow(ctx, P, a, a, a, a, true) : op_erode(ctx, P, -a);
  gb_layer* p2 = a > 0 ? op_erode(ctx, P, a, F, Q)
                       : (a == 0 ? op_bool(ctx, GB_OP_MERGE, P, nullptr, 0) : op_grow(ctx, P, -a, -a, -a, -a, true));
  if (!p1 || !p2) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
  gb_layer* outer = op_bool(ctx, GB_OP_NOT, p1, P, 0);
  gb_layer* inner = op_bool(ctx, GB_OP_NOT, P, p2, 0);
  if (!outer || !inner) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
  gb_layer* and1 = op_bool(ctx, GB_OP_AND, outer, P, 0);
  gb_layer* inter = op_bool(ctx, GB_OP_AND, outer, inner, 0);
  if (!and1 || !inter) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
  outs[0] = p1; outs[1] = p2; outs[2] = outer; outs[3] = inner; outs[4] = and1; outs[5] = inter;
  return GB_OK;
}

extern "C" int gb_op1(gb_context* ctx, gb_layer* P, int32_t a, gb_layer** outs) {
  if (!ctx || !P || !outs || P->dead) return GB_ERR_ARG;
  return op1_chain(ctx, P, a, outs, nullptr, nullptr);
}

// Union area of P per cell from the erosion's complement: the frame F of a
// cell contains P, so area(P) = area(F) - area(F \ P), and the tile kernel
// has already summed area(F \ P) per cell.
__global__ void k_area_from_frame(const DLayer* F, const DLayer* Q, long long* out, int ncell, DStatus* st) {
  if (st->err) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
    const int4 f = F->boxes[k];
    out[k] = (long long)(f.z - f.x) * (long long)(f.w - f.y) - Q->cell_area[k];
  }
}

__global__ void k_copy_area(const DLayer* A, long long* out, int ncell, DStatus* st) {
  if (st->err) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) out[k] = A->cell_area[k];
}

// The OP1 chain plus the union area of P per cell into d_area (device, ncell
// entries).  With a > 0 the area falls out of the erosion (no extra pass over
// P); otherwise it is a count-mode union of P.  Asynchronous, capturable.
extern "C" int gb_op1_area(gb_context* ctx, gb_layer* P, int32_t a, gb_layer** outs, long long* d_area) {
  if (!ctx || !P || !outs || !d_area || P->dead) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  gb_layer* F = nullptr;
  gb_layer* Q = nullptr;
  const int e = op1_chain(ctx, P, a, outs, &F, &Q);
  if (e) return e;
  const int nb = (P->ncell + 255) / 256;
  if (F && Q) {
    k_area_from_frame<<<nb, 256, 0, c.stream>>>(F->d, Q->d, d_area, P->ncell, c.st);
  } else {
    gb_layer* M = op_bool(ctx, GB_OP_MERGE, P, nullptr, 1);
    if (!M) return set_err(ctx, GB_ERR_CAPACITY, "descriptor pool exhausted");
    k_copy_area<<<nb, 256, 0, c.stream>>>(M->d, d_area, P->ncell, c.st);
  }
  ++c.launches;
  return GB_OK;
}

__global__ void k_gather_counts(const DLayer* const* L, int nl, int ncell, long long* out,
                                const DLayer* area_layer, long long* area_out, DStatus* st) {
  if (st->err) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x) {
    for (int j = 0; j < nl; ++j) out[(long long)k * nl + j] = L[j]->cell_count ? L[j]->cell_count[k] : -1;
    if (area_out) area_out[k] = area_layer->cell_area ? area_layer->cell_area[k] : -1;
  }
}

// The deck through host buffers.  The boxes go to a device staging buffer
// kept by the context (grown when needed) on a copy stream, in two halves
// split at a cell boundary when the layer is large; each half's deck starts
// when its copy has landed, so the second copy overlaps the first half's
// work.  Counts and areas come back with one copy each at the end.
static int op1_host_impl(gb_context* ctx, const c_box* boxes, unsigned long long n,
                         const long long* cell_offsets, int ncell, int32_t a, long long* counts,
                         long long* area, unsigned long long* digests, int* assert_failures) {
  if (!ctx || (!boxes && n) || ncell < 1) return GB_ERR_ARG;
  if (!cell_offsets) ncell = 1;
  GbCtx& c = ctx->c;
  std::vector<long long> off(ncell + 1);
  if (cell_offsets) {
    std::copy(cell_offsets, cell_offsets + ncell + 1, off.begin());
    for (int k = 0; k < ncell; ++k)
      if (off[k] > off[k + 1] || off[k] < 0) return set_err(ctx, GB_ERR_ARG, "cell offsets must not decrease");
    if (off[ncell] > (long long)n) return set_err(ctx, GB_ERR_ARG, "cell offsets past the boxes");
  } else {
    off[0] = 0;
    off[1] = (long long)n;
  }
  const size_t bytes = std::max<size_t>(16, (size_t)n * 16);
  if (c.io_cap < bytes) {
    if (c.io_buf) cudaFree(c.io_buf);
    c.io_buf = nullptr;
    c.io_cap = 0;
    if (cudaMalloc(&c.io_buf, bytes) != cudaSuccess) return set_err(ctx, GB_ERR_OOM, "input staging buffer");
    c.io_cap = bytes;
  }
  if (!c.copy_stream && cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return set_err(ctx, GB_ERR_CUDA, "copy stream");
  // groups of cells: two halves of the boxes when there are enough of them
  std::vector<int> cut{0};
  if (ncell > 1 && n >= (1ull << 22)) {
    const int k = (int)(std::lower_bound(off.begin(), off.end(), (long long)(n / 2)) - off.begin());
    if (k > 0 && k < ncell) cut.push_back(k);
  }
  cut.push_back(ncell);
  const int ng = (int)cut.size() - 1;
  std::vector<cudaEvent_t> ev(ng);
  char* dbox = (char*)c.io_buf;
  // the copy stream starts after the work already queued on the context stream (earlier users of the buffer)
  cudaEvent_t ready;
  cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  cudaEventRecord(ready, c.stream);
  cudaStreamWaitEvent(c.copy_stream, ready, 0);
  for (int g = 0; g < ng; ++g) {
    cudaEventCreateWithFlags(&ev[g], cudaEventDisableTiming);
    const long long b0 = off[cut[g]], b1 = off[cut[g + 1]];
    if (b1 > b0)
      cudaMemcpyAsync(dbox + b0 * 16, boxes + b0, (size_t)(b1 - b0) * 16, cudaMemcpyHostToDevice, c.copy_stream);
    cudaEventRecord(ev[g], c.copy_stream);
  }
  long long* dcounts = nullptr;
  long long* darea = nullptr;
  unsigned long long* ddig = nullptr;
  DLayer** dl = nullptr;
  int e = GB_OK;
  if (cudaMalloc(&dcounts, (size_t)ncell * 6 * 8) != cudaSuccess || cudaMalloc(&darea, (size_t)ncell * 8) != cudaSuccess ||
      cudaMalloc(&dl, 8 * sizeof(DLayer*)) != cudaSuccess ||
      (digests && cudaMalloc(&ddig, (size_t)ncell * 6 * 8) != cudaSuccess))
    e = set_err(ctx, GB_ERR_OOM, "deck result buffers");
  for (int g = 0; g < ng && !e; ++g) {
    const int k0 = cut[g], k1 = cut[g + 1];
    const long long b0 = off[k0];
    std::vector<long long> goff(off.begin() + k0, off.begin() + k1 + 1);
    for (long long& v : goff) v -= b0;
    cudaStreamWaitEvent(c.stream, ev[g], 0);
    gb_layer* P = nullptr;
    e = gbi::layer_over_device(ctx, dbox + b0 * 16, off[k1] - b0, goff.data(), k1 - k0, &P);
    if (e) break;
    const int gn = k1 - k0;
    e = gb_run_retry(ctx, [&]() -> int {
      gb_layer* outs[6];
      int r = gb_op1_area(ctx, P, a, outs, darea + k0);
      if (r) return r;
      DLayer* hl[6];
      for (int j = 0; j < 6; ++j) hl[j] = outs[j]->d;
      cudaMemcpyAsync(dl, hl, sizeof(hl), cudaMemcpyHostToDevice, c.stream);
      k_gather_counts<<<(gn + 255) / 256, 256, 0, c.stream>>>(dl, 6, gn, dcounts + (size_t)k0 * 6, nullptr, nullptr,
                                                             c.st);
      if (ddig) {  // per-cell strip digests of the six layers, [cell][layer]
        cudaMemsetAsync(ddig + (size_t)k0 * 6, 0, (size_t)gn * 6 * 8, c.stream);
        for (int j = 0; j < 6; ++j) gb_launch_digest(c, outs[j]->d, ddig + (size_t)k0 * 6 + j, 6);
      }
      return GB_OK;
    });
    gb_layer_free(ctx, P);
  }
  cudaStreamSynchronize(c.copy_stream);  // no copy may outlive the call
  std::vector<long long> hc((size_t)ncell * 6), ha(ncell);
  if (!e) {
    cudaMemcpy(hc.data(), dcounts, hc.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(ha.data(), darea, ha.size() * 8, cudaMemcpyDeviceToHost);
    int fails = 0;
    for (int k = 0; k < ncell; ++k) fails += (hc[(size_t)k * 6 + 4] > 0) + (hc[(size_t)k * 6 + 5] > 0);
    if (assert_failures) *assert_failures = fails;
    if (counts) memcpy(counts, hc.data(), hc.size() * 8);
    if (area) memcpy(area, ha.data(), ha.size() * 8);
    if (digests) cudaMemcpy(digests, ddig, (size_t)ncell * 6 * 8, cudaMemcpyDeviceToHost);
  }
  for (cudaEvent_t x : ev) cudaEventDestroy(x);
  cudaEventDestroy(ready);
  if (dcounts) cudaFree(dcounts);
  if (darea) cudaFree(darea);
  if (ddig) cudaFree(ddig);
  if (dl) cudaFree(dl);
  return e;
}

extern "C" int gb_op1_host(gb_context* ctx, const c_box* boxes, unsigned long long n,
                           const long long* cell_offsets, int ncell, int32_t a, long long* counts,
                           long long* area, int* assert_failures) {
  return op1_host_impl(ctx, boxes, n, cell_offsets, ncell, a, counts, area, nullptr, assert_failures);
}

extern "C" int gb_op1_host_digest(gb_context* ctx, const c_box* boxes, unsigned long long n,
                                  const long long* cell_offsets, int ncell, int32_t a, long long* counts,
                                  long long* area, unsigned long long* digests, int* assert_failures) {
  if (!digests) return GB_ERR_ARG;
  return op1_host_impl(ctx, boxes, n, cell_offsets, ncell, a, counts, area, digests, assert_failures);
}

// Slab height of the operators: the OP1 chain with the union area runs on P
// once untimed and once timed (CUDA events on the context stream) at each
// tile grid 2^13 .. 2^16 dbu, and the fastest grid stays set on the context.
// Results differ between grids only in where strips are cut (the point sets
// are the same).  ms_out (4 entries, may be NULL): the times, -1 for a grid
// that did not run.
extern "C" int gb_grid_autotune(gb_context* ctx, gb_layer* P, int32_t a, int* best_g, float* ms_out) {
  if (!ctx || !P || P->dead || !best_g) return GB_ERR_ARG;
  GbCtx& c = ctx->c;
  long long* d_area = nullptr;
  if (cudaMalloc(&d_area, (size_t)P->ncell * 8) != cudaSuccess) return set_err(ctx, GB_ERR_OOM, "grid tuning buffer");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int old = c.grid;
  float best = 0.f;
  int bg = -1;
  for (int g = GB_GRID_TUNE_MIN; g <= 16; ++g) {
    c.grid = g;
    float ms = -1.f;
    for (int rep = 0; rep < 2; ++rep) {
      const int r = gb_run_retry(ctx, [&]() -> int {
        gb_layer* outs[6];
        cudaEventRecord(e0, c.stream);
        const int q = gb_op1_area(ctx, P, a, outs, d_area);
        cudaEventRecord(e1, c.stream);
        return q;
      });
      if (r) {
        ms = -1.f;
        break;
      }
      if (rep) cudaEventElapsedTime(&ms, e0, e1);
    }
    if (ms_out) ms_out[g - GB_GRID_TUNE_MIN] = ms;
    if (ms > 0.f && (bg < 0 || ms < best)) {
      best = ms;
      bg = g;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_area);
  c.grid = bg < 0 ? old : bg;
  *best_g = c.grid;
  return bg < 0 ? set_err(ctx, GB_ERR_CAPACITY, "the deck ran on no grid") : GB_OK;
}

extern "C" int gb_debug_lookback_timeout(gb_context* ctx, int spin_limit) {
  if (!ctx || spin_limit < 1) return GB_ERR_ARG;
  gb_clear_status(ctx);
  if (gb_radix_lookback_timeout_probe(ctx->c, spin_limit)) return GB_ERR_CUDA;
  const int e = gb_sync(ctx, nullptr);
  gb_clear_status(ctx);
  return e;
}
