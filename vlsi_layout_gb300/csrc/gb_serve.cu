// gb_serve.cu -- a request loop for Boolean operators on layers resident in HBM.
//
// Layers are added once and binned into a long-lived context.  Requests
// (AND / NOT / OR / XOR / GROW / SIZE on one or two resident layers) arrive on
// a schedule; the loop admits an arrived request as soon as an execution slot
// is free and the estimated device memory of all requests in flight fits the
// budget, runs it asynchronously on the slot's own stream and arena (so the
// work of concurrent requests overlaps on the GPU), and retires requests as
// their completion events fire.  Requests that arrive while others run are
// admitted as slots and memory free up: batching is continuous, not a queue
// drained in rounds.  Latency = completion - arrival, on the host clock.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "gbool.h"
#include "gb_internal.h"

using namespace gbi;

struct gb_server_slot {
  gb_context* ctx = nullptr;
  cudaEvent_t done = nullptr;
  int req = -1;
  unsigned long long mark = 0;
  long long est = 0;
  gb_layer* out = nullptr;
  long long* dcount = nullptr;  // device: strips of the result
  long long* hcount = nullptr;  // pinned host copy
};

struct gb_server {
  int device = 0;
  unsigned long long budget = 0;
  gb_context* home = nullptr;  // owns the resident (binned) layers
  std::vector<gb_layer*> raw, binned;
  std::vector<long long> nbox;
  std::vector<gb_server_slot> slots;
  std::vector<std::vector<c_box>> kept;  // results copied out when requested
};

namespace {

__global__ void k_copy_count(const DLayer* L, long long* out) {
  *out = L->cell_count ? L->cell_count[0] : -1;
}

long long estimate(const gb_server* S, const gb_request& r) {
  long long n = S->nbox[r.a] + (r.op <= GB_OP_NOT ? S->nbox[r.b] : 0);
  if (r.op == GB_REQ_SIZE && r.amount < 0) n *= 3;  // erosion runs two Booleans on the complement
  return 48ll * n + (4ll << 20);
}

gb_layer* issue(gb_server* S, gb_server_slot& sl, const gb_request& r, int* status) {
  gb_layer* O = nullptr;
  int e = GB_ERR_ARG;
  gb_layer* A = S->binned[r.a];
  switch (r.op) {
    case GB_OP_XOR:
    case GB_OP_OR:
    case GB_OP_AND:
    case GB_OP_NOT:
      e = gb_op_bool(sl.ctx, r.op, A, S->binned[r.b], &O);
      break;
    case GB_REQ_GROW:
      e = gb_op_grow(sl.ctx, A, r.amount, r.amount, r.amount, r.amount, &O);
      break;
    case GB_REQ_SIZE:
      e = gb_op_size(sl.ctx, A, r.amount, &O);
      break;
    default:
      break;
  }
  *status = e;
  return e ? nullptr : O;
}

}  // namespace

extern "C" int gb_serve_create(int device, unsigned long long budget_bytes, int slots,
                               unsigned long long slot_arena_bytes, gb_server** out) {
  if (!out || slots < 1 || slots > 64) return GB_ERR_ARG;
  gb_server* S = new gb_server();
  S->device = device;
  S->budget = budget_bytes;
  int e = gb_context_create(device, slot_arena_bytes, &S->home);
  if (e) { delete S; return e; }
  for (int i = 0; i < slots; ++i) {
    gb_server_slot sl;
    e = gb_context_create(device, slot_arena_bytes, &sl.ctx);
    if (!e) e = gb_set_tile_scratch(sl.ctx, 4ull << 20);
    if (e) break;
    cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    cudaMalloc(&sl.dcount, 8);
    cudaMallocHost(&sl.hcount, 8);
    S->slots.push_back(sl);
  }
  if (e) { gb_serve_destroy(S); return e; }
  *out = S;
  return GB_OK;
}

extern "C" int gb_serve_add_layer(gb_server* S, const c_box* boxes, unsigned long long n, int* id) {
  if (!S || !id) return GB_ERR_ARG;
  gb_layer* L = nullptr;
  int e = gb_layer_from_host(S->home, boxes, n, nullptr, 1, &L);
  if (e) return e;
  // bin once; the binned form lives in the home context's arena for the server's lifetime
  gb_layer* B = binned_of(S->home, L, 16);
  if (!B) {
    gb_layer_free(S->home, L);  // not recorded: gb_serve_destroy would never free it
    return GB_ERR_CAPACITY;
  }
  e = gb_sync(S->home, nullptr);
  if (e) {
    gb_layer_free(S->home, B);
    gb_layer_free(S->home, L);
    return e;
  }
  *id = (int)S->raw.size();
  S->raw.push_back(L);
  S->binned.push_back(B);
  S->nbox.push_back((long long)n);
  return GB_OK;
}

extern "C" int gb_serve_run(gb_server* S, const gb_request* reqs, int nreq, gb_result* res, int keep_outputs) {
  if (!S || (nreq && (!reqs || !res))) return GB_ERR_ARG;
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  auto now_s = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
  if (keep_outputs) S->kept.assign(nreq, {});
  for (int i = 0; i < nreq; ++i) {
    res[i] = gb_result{};
    res[i].status = -1;
    if (reqs[i].a < 0 || reqs[i].a >= (int)S->raw.size() ||
        (reqs[i].op <= GB_OP_NOT && (reqs[i].b < 0 || reqs[i].b >= (int)S->raw.size())))
      res[i].status = GB_ERR_ARG;
  }
  std::deque<int> waiting;
  int next = 0, done = 0;
  long long inflight = 0;
  while (done < nreq) {
    const double t = now_s();
    while (next < nreq && reqs[next].arrival_s <= t) waiting.push_back(next++);
    // retire finished requests
    for (gb_server_slot& sl : S->slots) {
      if (sl.req < 0 || cudaEventQuery(sl.done) != cudaSuccess) continue;
      const int i = sl.req;
      long long need = 0;
      int e = gb_sync(sl.ctx, &need);
      res[i].status = e;
      res[i].count = *sl.hcount;
      if (!e && keep_outputs && sl.out) {
        unsigned long long n = 0;
        gb_layer_to_host(sl.ctx, sl.out, nullptr, 0, &n, nullptr);
        S->kept[i].resize(n);
        gb_layer_to_host(sl.ctx, sl.out, S->kept[i].data(), n, &n, nullptr);
      }
      res[i].end_s = now_s();
      res[i].latency_ms = (res[i].end_s - reqs[i].arrival_s) * 1e3;
      if (e) gb_clear_status(sl.ctx);
      gb_arena_release(sl.ctx, sl.mark);
      inflight -= sl.est;
      sl.req = -1;
      sl.out = nullptr;
      ++done;
    }
    // admit arrived requests in order while a slot is free and the budget allows
    while (!waiting.empty()) {
      const int i = waiting.front();
      if (res[i].status == GB_ERR_ARG) {
        waiting.pop_front();
        res[i].end_s = now_s();
        ++done;
        continue;
      }
      const long long est = estimate(S, reqs[i]);
      if (est > (long long)S->budget) {  // can never fit: refuse
        waiting.pop_front();
        res[i].status = GB_ERR_CAPACITY;
        res[i].end_s = now_s();
        ++done;
        continue;
      }
      gb_server_slot* free_slot = nullptr;
      for (gb_server_slot& sl : S->slots)
        if (sl.req < 0) { free_slot = &sl; break; }
      if (!free_slot || inflight + est > (long long)S->budget) break;
      waiting.pop_front();
      gb_server_slot& sl = *free_slot;
      sl.mark = gb_arena_mark(sl.ctx);
      res[i].start_s = now_s();
      int st = 0;
      sl.out = issue(S, sl, reqs[i], &st);
      if (!sl.out) {
        res[i].status = st;
        res[i].end_s = now_s();
        gb_arena_release(sl.ctx, sl.mark);
        ++done;
        continue;
      }
      k_copy_count<<<1, 1, 0, sl.ctx->c.stream>>>(sl.out->d, sl.dcount);
      cudaMemcpyAsync(sl.hcount, sl.dcount, 8, cudaMemcpyDeviceToHost, sl.ctx->c.stream);
      cudaEventRecord(sl.done, sl.ctx->c.stream);
      sl.req = i;
      sl.est = est;
      inflight += est;
    }
    if (done < nreq) {
      bool busy = false;
      for (gb_server_slot& sl : S->slots) busy |= sl.req >= 0;
      if (!busy && waiting.empty() && next < nreq) {
        const double wait = reqs[next].arrival_s - now_s();
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.001)));
      } else {
        std::this_thread::yield();
      }
    }
  }
  return GB_OK;
}

extern "C" int gb_serve_result_boxes(gb_server* S, int i, c_box* out, unsigned long long cap,
                                     unsigned long long* n) {
  if (!S || !n || i < 0 || i >= (int)S->kept.size()) return GB_ERR_ARG;
  *n = S->kept[i].size();
  if (*n > cap) return GB_ERR_CAPACITY;
  if (*n && out) memcpy(out, S->kept[i].data(), *n * sizeof(c_box));
  return GB_OK;
}

extern "C" void gb_serve_destroy(gb_server* S) {
  if (!S) return;
  for (gb_server_slot& sl : S->slots) {
    if (sl.ctx) gb_sync(sl.ctx, nullptr);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.dcount) cudaFree(sl.dcount);
    if (sl.hcount) cudaFreeHost(sl.hcount);
    if (sl.ctx) gb_context_destroy(sl.ctx);
  }
  for (gb_layer* L : S->raw) gb_layer_free(S->home, L);
  if (S->home) gb_context_destroy(S->home);
  delete S;
}
