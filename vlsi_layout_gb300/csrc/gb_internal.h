// gb_internal.h -- host-side context and kernel launchers shared by the
// engine's translation units.  Not part of the public C-ABI (include/gbool.h).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include <functional>
#include <mutex>
#include "gb_common.cuh"

struct c_box;  // include/gbool.h

#define GB_SCAN_BLOCKS 256
#define GB_SCAN_THREADS 512
#define GB_TILE_THREADS 384
#define GB_NDESC 8192

struct GbCtx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int nsm = 0;
  int work_blocks = 0;     // persistent grid of streaming kernels
  int tile_blocks = 0;     // persistent grid of the tile kernel (1 CTA / SM)
  size_t tile_smem = 0;
  DStatus* st = nullptr;   // device
  char* arena = nullptr;   // work arena (device bump allocation)
  unsigned long long arena_cap = 0;
  long long* scan_part = nullptr;    // [GB_SCAN_BLOCKS + 1]
  long long* dscal = nullptr;        // device scalar scratch [64]
  long long* tile_counter = nullptr; // [64] persistent-kernel work counters
  char* tile_scratch = nullptr;      // per-CTA scratch of the tile kernel
  size_t tile_scr_bytes = 0;         // bytes per CTA
  DLayer* desc = nullptr;            // descriptor pool [GB_NDESC] in device memory
  std::vector<int> desc_free;
  int cap_factor = 2;                // output pool pieces per input piece of a Boolean op
  std::string last_error;
  // profiling: CUDA events around every tile-kernel launch
  bool prof = false;
  std::vector<cudaEvent_t> prof_ev;  // pairs (start, stop)
  size_t prof_used = 0;
  unsigned prof_flags = 0;
  bool timing = false;               // per-phase clock64 counters in the tile kernel
  long long launches = 0;            // kernels issued by the engine (host-side count)
  void* rs = nullptr;                // radix sort state (histograms, look-back status), gb_radix.cu
  int grid = 16;                     // tile grid log2 (slab height 2^grid dbu) of the operators
  void* io_buf = nullptr;            // device staging of host inputs (gb_op1_host), grow-only
  size_t io_cap = 0;
  cudaStream_t copy_stream = nullptr;  // host-to-device copies that overlap the compute stream
};

struct gb_layer {
  int slot = -1;
  DLayer* d = nullptr;  // descriptor in device memory
  int ncell = 1;
  int g = 16;
  int binned = 0;
  int counted = 0;      // cell_count holds exact strip counts
  int arena_owned = 0;  // arrays live in the work arena
  unsigned long long seq = 0;  // creation sequence (arena layers)
  bool dead = false;
  void* own_boxes = nullptr;  // raw layers: cudaMalloc'd arrays
  void* own_coff = nullptr;
  void* own_cell = nullptr;
  gb_layer* bin_cache = nullptr;
  long long nbox_host = 0;
};

struct gb_context {
  GbCtx c;
  std::mutex mu;
  unsigned long long seq = 0;
  std::vector<gb_layer*> arena_layers;
  std::vector<std::pair<unsigned long long, unsigned long long>> marks;  // (device off, seq)
  unsigned long long graph_arena_off = 0;
};


// host helpers shared by gb_api.cu and gb_deck.cu
namespace gbi {
int set_err(gb_context* ctx, int code, const char* msg);
gb_layer* new_arena_layer(gb_context* ctx, int ncell, int g);
gb_layer* binned_of(gb_context* ctx, gb_layer* L, int g);
DStatus read_status(gb_context* ctx);
DLayer read_desc(gb_context* ctx, gb_layer* L);
// A raw layer over n boxes already in device memory (not copied; the caller
// keeps them alive while the layer is used), cells given by host offsets.
int layer_over_device(gb_context* ctx, const void* d_boxes, long long n, const long long* h_offsets, int ncell,
                      gb_layer** out);
// The layer's boxes in device memory: a raw layer's array, or a binned layer
// exported into the work arena.
int layer_device_boxes(gb_context* ctx, gb_layer* L, const c_box** d_boxes, long long* n);
}
gb_layer* op_bool(gb_context* ctx, int op, gb_layer* A, gb_layer* B, int mode);
gb_layer* op_grow(gb_context* ctx, gb_layer* A, int E, int N, int W, int S, bool merge);
// Erosion of P by the square [-t,t]^2.  frame_out / comp_out (optional)
// receive the frame F (bbox of each cell grown by t, one box per cell) and
// the complement Q = F \ P computed on the way.
gb_layer* op_erode(gb_context* ctx, gb_layer* P, int t, gb_layer** frame_out = nullptr,
                   gb_layer** comp_out = nullptr);
int sync_where(gb_context* ctx, int* where, long long* need);
// Run a host-synchronous device sequence; on a capacity error enlarge the
// failing resource (tile scratch, output slots) and run it again.
int gb_run_retry(gb_context* ctx, const std::function<int()>& body);

// ---- kernels / launchers (gb_bin.cu)
// Exclusive scan of an int array into int64 starts.  The array pointers are
// read on the device from the given descriptor fields, and the length from
// n_dev, so sizes decided on the device need no host round trip.
void gb_launch_scan_i32(GbCtx& c, int* const* in_field, long long* const* out_field,
                        const long long* n_dev, long long* total_dev);
void gb_launch_arena_reset(GbCtx& c, unsigned long long mark);
// Build the binned form of `src` (raw or binned) after growing every box by
// (E,N,W,S) on grid g.  out must be a descriptor with ncell set by the host.
void gb_launch_rebin(GbCtx& c, const DLayer* src, int src_binned, DLayer* out, int ncell, int g,
                     int E, int N, int W, int S);
// Closed-tile index binning for connectivity (pcs holds int box indices).
void gb_launch_bin_index(GbCtx& c, const DLayer* src, DLayer* out, int ncell, int g);
// Output window / slot capacities of a Boolean op.
// alloc_slots = 0: count / area only (no output slots).
void gb_launch_bool_setup(GbCtx& c, int op, const DLayer* A, const DLayer* B, DLayer* O,
                          int ncell, int g, int alloc_slots);
// Export a binned layer to global-coordinate int4 boxes (tile order).
// offsets [ntiles+1] and the out buffer are allocated from the arena; the
// device pointer to the box array and the total land in *dscal-slots.
void gb_launch_export(GbCtx& c, const DLayer* L, int4** out_ptr_dev, long long* total_dev);
void gb_launch_cell_bbox_fill(GbCtx& c, DLayer* L, int ncell);
// Per-cell strip digests of a binned layer, added to out[cell * stride]
// (out zeroed by the caller).
void gb_launch_digest(GbCtx& c, const DLayer* L, unsigned long long* out, int stride);

// ---- tile kernel (gb_tile.cu)
void gb_tile_setup(GbCtx& c);
// mode: 0 = emit strips, 1 = count + area only
void gb_launch_tile_bool(GbCtx& c, int op, const DLayer* A, const DLayer* B, DLayer* O, int g,
                         int mode);

// ---- connectivity (gb_uf.cu)
void gb_launch_components(GbCtx& c, const DLayer* raw, DLayer* binidx, int* parent,
                          unsigned char* touched, long long* labels, long long n,
                          long long* out_ncomp_dev, int* flag_tmp, long long* map_tmp);

// Overlap statistics of one layer: pairs overlapping with positive area
// (*strict_dev) and boxes meeting no other box (*single_dev, mask_dev
// optional).  binidx: closed-range index binning on grid g.
void gb_launch_pair_stats(GbCtx& c, const DLayer* raw, DLayer* binidx, int g, unsigned char* touched,
                          long long n, unsigned long long* strict_dev, unsigned long long* single_dev,
                          unsigned char* mask_dev);

// ---- radix sort (gb_radix.cu)
// Sorts n (key, value) pairs by the low `bits` bits of the 64-bit keys.
// tmp buffers must hold n entries each.  Stable.  passes / items (keys per
// thread: 12, 16 or 20) <= 0 take the tuned or default choice.  Returns
// the pass count, or < 0 when the configuration is not available.
int gb_radix_sort_pairs(GbCtx& c, unsigned long long* keys, unsigned* vals, long long n, int bits,
                        unsigned long long* keys_tmp, unsigned* vals_tmp, int passes = 0, int items = 0);
int gb_radix_tune(GbCtx& c, const unsigned long long* keys, const unsigned* vals, long long n, int bits,
                      int* best_passes, int* best_items, float* best_ms);
void gb_radix_default(int bits, int* passes, int* items);
void gb_radix_forget_tuning();
void gb_radix_free(GbCtx& c);

int gb_radix_lookback_timeout_probe(GbCtx& c, int spin_limit);

// helpers
inline int gb_cuda_check(GbCtx& c, cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    c.last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GB_ERR_CUDA;
  }
  return GB_OK;
}
