/*
 * gbool.h -- C-ABI of the GB300 Manhattan box-Boolean engine (libgbool.so).
 *
 * Two groups of entry points:
 *
 *  1. Drop-in replacements that keep the reference's exact symbol names and
 *     signatures, so the Fortran layer binds them unchanged:
 *       PerformBoostPolygonOperation / PerformBoostPolygonMerge
 *         replace src/boost_polygon_api.h:26-37 (impl boost_polygon_api.cpp:
 *         41-156; Fortran binding boost_polygon_apif.f90:12-38);
 *       thrust_sort_boxes_direct / thrust_sort_boxes_indirect
 *         replace src/gpu_morton.cu:149-187 (binding gpu_morton_sort.f90:41-55);
 *       device_event_sort
 *         replaces src/event_sorter.cu:64-81 (binding event_sorter_apif.f90:17-23).
 *
 *  2. gb_* entry points in the bind(c)-by-value style of event_sorter_apif.f90,
 *     each returning a GB_* status: device-resident layers (SoA boxes in HBM,
 *     binned to a fixed 2^g-dbu tile grid), the MAGPARSER operators on them,
 *     Klee's-measure area, PNUM connectivity, Morton/tracker sorts, and the
 *     control-deck runner.
 *
 * Result form: a Boolean / sizing result is the canonical strip decomposition
 * of its point set: the plane is cut by the fixed grid of 2^g-dbu tiles
 * (default g = 16) and inside each tile the region is given as maximal
 * vertical strips (at every x the maximal y-intervals, merged along x while
 * unchanged), the form heal_boxes emits (polygon_fracture.f90:805-1004).
 * Coordinates are int32 dbu, areas int64.  No floating point touches results.
 */
#ifndef GBOOL_H
#define GBOOL_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes */
#define GB_OK 0
#define GB_ERR_CAPACITY 1     /* a capacity was too small; retried internally where possible */
#define GB_ERR_INVALID_BOX 2  /* an input (or grown) box has x1 >= x2 or y1 >= y2 */
#define GB_ERR_OOM 3
#define GB_ERR_TIMEOUT 4      /* a bounded device wait gave up */
#define GB_ERR_CUDA 5
#define GB_ERR_ARG 6
#define GB_ERR_INTERNAL 7
#define GB_ERR_CORRUPT 8       /* a SNAP stream or file is malformed (codec desync, bad Snappy element) */

/* ---- Boolean opcodes (the reference's control parameter, boost_polygon_api.cpp:116-137) */
#define GB_OP_XOR 0
#define GB_OP_OR 1
#define GB_OP_AND 2
#define GB_OP_NOT 3   /* A - B */
#define GB_OP_MERGE 4 /* union of A */
#define GB_OP_SIZE 5  /* PerformBoostPolygonOperation only: resize by control_value */
#define GB_OP_OVERLAP 7 /* single-layer AND (CalculateSingleLayerAND, design_impl.f90:385-498):
                           the area covered by at least two boxes of A; B unused */

/* AoS box, identical to c_box of boost_polygon_api.h:16-23 and Fortran type(Box). */
struct c_box {
  int32_t x1;
  int32_t y1;
  int32_t x2;
  int32_t y2;
};
typedef struct c_box c_box;

/* Tracker event of event_sorter.cu:15-19 (12 bytes with padding). */
struct XYTracker {
  int32_t X;
  int32_t Y;
  int8_t polygonNumber;
};
typedef struct XYTracker XYTracker;

/* =====================================================================
 * 1. Drop-in replacements (reference symbols)
 * ===================================================================== */

/* boost_polygon_api.h:29-36.  control 0 XOR, 1 OR, 2 AND, 3 NOT (A-B),
 * 4 MERGE (A), 5 SIZE (A resized by control_value dbu).  Host pointers.  The
 * caller's buffer convention is kept: `output` holds at least 4*max(AN,BN)
 * boxes, or 10*max(AN,BN) for AND (boost_polygon_apif.f90:59-71).  Where the
 * reference wrote past that buffer unchecked, this version prints the needed
 * size to stderr, writes nothing and sets *outN = 0.  Re-entrant (calls are
 * serialised on the default context). */
void PerformBoostPolygonOperation(const struct c_box* input_A, unsigned long AN,
                                  const struct c_box* input_B, unsigned long BN,
                                  struct c_box* output, unsigned long* outN,
                                  unsigned long control_parameter, long control_value);

/* boost_polygon_api.cpp:41-70 (binding boost_polygon_apif.f90:14-25): union
 * of N boxes; `output` holds at least 2*N boxes (boost_polygon_apif.f90:95). */
void PerformBoostPolygonMerge(const struct c_box* input, unsigned long N, struct c_box* output,
                              unsigned long* outN);

/* gpu_morton.cu:149-164: sort boxes in place by the 64-bit Morton key of the
 * box centre.  Host or device pointer. */
void thrust_sort_boxes_direct(struct c_box* boxes, int64_t n);

/* gpu_morton.cu:169-187: write the 1-based permutation that sorts the boxes
 * by Morton key into indices[0..n); boxes are not moved. */
void thrust_sort_boxes_indirect(struct c_box* boxes, int64_t* indices, int64_t n);

/* event_sorter.cu:64-81: sort trackers by (X, Y) in place. */
void device_event_sort(struct XYTracker* arr, int64_t n);

/* =====================================================================
 * 2. Native API
 * ===================================================================== */
typedef struct gb_context gb_context;
typedef struct gb_layer gb_layer;

/* Create a context on `device` with a device work arena of arena_bytes
 * (0 = a default sized to the free memory).  Operators allocate their
 * results from the arena on the device, so they need no host round trip. */
int gb_context_create(int device, unsigned long long arena_bytes, gb_context** out);
int gb_context_destroy(gb_context* ctx);
/* Run all work of the context on this cudaStream_t (NULL = the context's own). */
int gb_set_stream(gb_context* ctx, void* stream);
const char* gb_last_error(gb_context* ctx);
/* Synchronise the stream and return the first device-side status (GB_*). */
int gb_sync(gb_context* ctx, long long* need);
void gb_clear_status(gb_context* ctx);
/* Arena marks: layers created after a mark are invalid after releasing it. */
unsigned long long gb_arena_mark(gb_context* ctx);
int gb_arena_release(gb_context* ctx, unsigned long long mark);
/* Output pool of a Boolean op, in pieces per input piece (default 2; doubled
 * and retried automatically by the host-synchronous entry points). */
int gb_set_capacity_factor(gb_context* ctx, int factor);
/* Per-CTA scratch of the tile kernel in bytes (default 8 MiB; at least 64 KiB,
 * rounded up to a multiple of 512). */
int gb_set_tile_scratch(gb_context* ctx, unsigned long long bytes);

/* A layer of n boxes (host pointer), grouped into ncell independent cells by
 * cell_offsets[ncell+1] (NULL: one cell).  The boxes are copied to HBM. */
int gb_layer_from_host(gb_context* ctx, const c_box* boxes, unsigned long long n,
                       const long long* cell_offsets, int ncell, gb_layer** out);
/* Same with device pointers (copied on the device). */
int gb_layer_from_device(gb_context* ctx, const c_box* d_boxes, unsigned long long n,
                         const long long* d_cell_offsets, int ncell, gb_layer** out);
int gb_layer_ncell(gb_layer* L);
/* Box (strip) count, total and per cell (per_cell may be NULL).  Syncs. */
int gb_layer_count(gb_context* ctx, gb_layer* L, long long* total, long long* per_cell);
/* Per-cell digest of a Boolean result (a binned layer): out[ncell] (host)
 * gets, per cell, the sum mod 2^64 of gb_strip_hash(x1, y1, x2, y2) over its
 * strips in global dbu -- the MurmurHash3 fmix64 finaliser of
 * (x1<<32|y1) ^ fmix64((x2<<32|y2) + 0x9e3779b97f4a7c15), coordinates taken
 * as uint32.  Order-independent: two layers with the same strips per cell
 * have the same digests.  A raw (input) layer gives GB_ERR_ARG. */
int gb_layer_digest(gb_context* ctx, gb_layer* L, unsigned long long* out);
/* Copy a layer to the host in tile order (cell-major).  cap is the capacity
 * of out in boxes; *n receives the count (GB_ERR_CAPACITY if cap < count).
 * cell_offsets (ncell+1 entries, may be NULL) receives the per-cell ranges. */
int gb_layer_to_host(gb_context* ctx, gb_layer* L, c_box* out, unsigned long long cap,
                     unsigned long long* n, long long* cell_offsets);
void gb_layer_free(gb_context* ctx, gb_layer* L);

/* Operators (device-resident, asynchronous on the context stream).
 * gb_op_bool: op GB_OP_XOR/OR/AND/NOT need B; GB_OP_MERGE and GB_OP_OVERLAP
 * take A alone (B ignored). */
int gb_op_bool(gb_context* ctx, int op, gb_layer* A, gb_layer* B, gb_layer** out);
int gb_op_grow(gb_context* ctx, gb_layer* A, int32_t E, int32_t N, int32_t W, int32_t S,
               gb_layer** out);
int gb_op_size(gb_context* ctx, gb_layer* A, int32_t s, gb_layer** out);
/* Union area per cell (Klee's measure, int64).  Syncs. */
int gb_op_area(gb_context* ctx, gb_layer* A, long long* area_per_cell);

/* PNUM connectivity (pnummerge.f90:279-385) of n host boxes: component count
 * and, when labels is not NULL, per-box labels (0 singleton, else 1..R with
 * roots numbered in index order). */
int gb_components(gb_context* ctx, const c_box* boxes, unsigned long long n, long long* ncomp,
                  long long* labels);

/* Overlap statistics of n host boxes (ComputeInteractionsCPU and
 * FindSingletonsCPU, pnummerge.f90:388-562): *strict_pairs = pairs i<k whose
 * boxes overlap with positive area; *singletons = boxes that no other box
 * touches or overlaps (closed bounds); is_singleton (optional, n bytes) gets
 * the mask.  Either count pointer may be NULL.  Synchronous. */
int gb_interactions(gb_context* ctx, const c_box* boxes, unsigned long long n, long long* strict_pairs,
                    long long* singletons, unsigned char* is_singleton);
/* CertifyHealing (design_impl.f90:35-56): *healed = 1 when n < 2 or no two
 * boxes overlap with positive area, else 0. */
int gb_certify_healing(gb_context* ctx, const c_box* boxes, unsigned long long n, int* healed);
/* Union area per PNUM component (calculate_union_area_by_polygon,
 * design.f90:854-935): areas[0] = total area of the singletons, areas[k] =
 * union area of component k (labels as gb_components), k = 1..R.  *nlabels
 * receives R + 1; GB_ERR_CAPACITY when cap < R + 1 (areas may then be NULL
 * to size the call).  Their sum is the union area of the layer. */
int gb_component_areas(gb_context* ctx, const c_box* boxes, unsigned long long n, long long* areas,
                       unsigned long long cap, long long* nlabels);

/* Morton-key sort of n host boxes: keys_out (optional) and perm (optional,
 * 0-based) receive the sorted keys and the permutation; boxes are sorted in
 * place when sort_boxes != 0. */
int gb_morton_sort(gb_context* ctx, c_box* boxes, long long n, int sort_boxes,
                   unsigned long long* keys_out, long long* perm);

/* Device-resident LSD radix sort of (key, value) pairs by the low `bits`
 * key bits, stable; the *_tmp buffers hold n entries.  The sorted pairs end
 * in d_keys / d_vals.  The pass count and keys per thread come from the
 * autotuner's table when it holds this device, bit width and size class,
 * else from the default (digits of at most 7 bits, an even pass count when
 * that costs no extra pass of bytes, tiles of 8192 keys).  n < 2^32.  Returns the number
 * of passes (>= 0) or minus a GB_ERR_* status.  Asynchronous on the context stream.
 * Replaces the Thrust radix sorts of gpu_morton.cu:149-187 and
 * event_sorter.cu:64-81 on device-resident data. */
int gb_radix_sort_device(gb_context* ctx, unsigned long long* d_keys, unsigned* d_vals, long long n, int bits,
                         unsigned long long* d_keys_tmp, unsigned* d_vals_tmp);
/* The same with an explicit configuration: `passes` passes splitting the
 * bits as evenly as possible (digits of 1..10 bits) and CTA tiles of `tile`
 * keys (3072, 4096, 5120 on 256 threads; 6144, 8192 on 512 threads).
 * -GB_ERR_ARG when the configuration is not built.  No counterpart in the
 * reference. */
int gb_radix_sort_device_cfg(gb_context* ctx, unsigned long long* d_keys, unsigned* d_vals, long long n, int bits,
                             unsigned long long* d_keys_tmp, unsigned* d_vals_tmp, int passes, int tile);
/* Autotuner: times every built (passes, tile) pair near the fewest passes on
 * a device copy of the given pairs (inputs untouched; needs 2 x 12 n bytes of
 * device memory), keeps the fastest in a process-wide table keyed by device,
 * bit width and power-of-two size class, and returns it.  Synchronous.  No
 * counterpart in the reference. */
int gb_radix_autotune(gb_context* ctx, const unsigned long long* d_keys, const unsigned* d_vals, long long n,
                      int bits, int* passes, int* tile, float* ms);
/* Clear the autotuner's table (later sorts use the default again). */
void gb_radix_tuning_reset(void);
/* The plan (pass count, keys per tile) the device sort takes for `bits`
 * significant key bits and n keys on `device`: the tuned one for that bit
 * width and size class, else the default (fewest passes of at most 7 bits,
 * rounded up to an even count; 8192-key tiles).  For byte accounting. */
int gb_radix_plan(int device, int bits, long long n, int* passes, int* tile);
/* Morton keys of device boxes (gpu_morton.cu:113-144) and the identity
 * permutation, on the device. */
int gb_morton_keys_device(gb_context* ctx, const c_box* d_boxes, long long n, unsigned long long* d_keys,
                          unsigned* d_vals);

/* Canonical order: sort n host boxes by (x1, y1, x2, y2). */
int gb_canonical_sort(gb_context* ctx, c_box* boxes, long long n);

/* Convert um to dbu exactly as the interpreter does: int(1000*r), truncating
 * toward zero (controlparser.f90:146,568-576). */
int32_t gb_um_to_dbu(double r);

/* ---- no-allocation Boolean (no counterpart in the reference)
 * For callers that cannot allocate device memory on their call path: a
 * serving loop that reserved its whole device budget up front, a host that
 * must avoid the allocator's implicit device synchronisation, or a Fortran /
 * C caller that owns only the buffers it passes.  Computes the canonical
 * strips of pred(A, B) (op 0..4; MERGE reads A only) for device boxes
 * d_A[nA], d_B[nB] that all lie in one 65536-dbu tile, into d_out[out_cap];
 * *d_count (device) gets the strip count, *d_area (device, may be NULL) the
 * strip area.  Works only in storage reserved statically in the library
 * (each GPU that loads it holds ~9 MB until exit): nA + nB <= 16384 and at
 * most 65536 strips, else GB_ERR_CAPACITY; a result larger than out_cap is
 * GB_ERR_CAPACITY too.  Boxes outside the first box's tile give
 * GB_ERR_INVALID_BOX.  On every status other than GB_OK, *d_count (and
 * *d_area) is -1.  The first call on a device sets up the static storage
 * (cudaGetSymbolAddress).  All calls share that storage: calls whose GPU
 * work overlaps race.  Every call waits for `stream` (a cudaStream_t, NULL =
 * default) to finish and returns the status. */
int gb_bool_tile_noalloc(int op, const c_box* d_A, int nA, const c_box* d_B, int nB, c_box* d_out,
                         long long out_cap, long long* d_count, long long* d_area, void* stream);

/* ---- control decks */
/* Run a MAGPARSER control deck (controlparser.f90 syntax; the README's
 * RUN_LOOP(`OP1', ...) macro line is expanded in place) on the GPU engine.
 * log (may be NULL) receives the interpreter's report; *assert_failures
 * counts failed ASSERT_ZEROs.  Returns GB_OK or the first failing status. */
int gb_run_deck(const char* path, char* log, unsigned long long log_cap, int* assert_failures);

/* ---- serving loop: Boolean requests on layers resident in HBM */
#define GB_REQ_SIZE 5 /* request op: SIZE by `amount` dbu (ops 0..3 are the Booleans) */
#define GB_REQ_GROW 6 /* request op: GROW all four sides by `amount` dbu */
typedef struct gb_server gb_server;
typedef struct gb_request {
  int op;           /* GB_OP_XOR/OR/AND/NOT, GB_REQ_SIZE or GB_REQ_GROW */
  int a, b;         /* resident layer ids (b unused by SIZE / GROW) */
  int amount;       /* dbu for SIZE / GROW */
  double arrival_s; /* arrival time, seconds after the start of gb_serve_run */
} gb_request;
typedef struct gb_result {
  int status;       /* GB_* of the request */
  int pad;
  long long count;  /* strips in the result */
  double start_s, end_s, latency_ms; /* admission, completion, completion - arrival */
} gb_result;
/* A server with `slots` concurrent execution slots (each its own stream and
 * work arena of slot_arena_bytes) admitting requests while the estimated
 * device memory of those in flight stays within budget_bytes. */
int gb_serve_create(int device, unsigned long long budget_bytes, int slots,
                    unsigned long long slot_arena_bytes, gb_server** out);
/* Add a resident layer (copied to HBM and binned once). */
int gb_serve_add_layer(gb_server* s, const c_box* boxes, unsigned long long n, int* id);
/* Serve requests in arrival order on the host clock (requests sorted by
 * arrival_s); a request is admitted when it has arrived, a slot is free and
 * the memory budget allows; results[i] gets its status, strip count and
 * latency.  keep_outputs != 0 keeps every result for gb_serve_result_boxes. */
int gb_serve_run(gb_server* s, const gb_request* reqs, int nreq, gb_result* results, int keep_outputs);
int gb_serve_result_boxes(gb_server* s, int index, c_box* out, unsigned long long cap, unsigned long long* n);
void gb_serve_destroy(gb_server* s);

/* ---- deck-level execution */
/* OP1 ring-check chain (op_template.m4:14-22) on all cells of P with amount a
 * dbu: outs[0..5] = P_1 (GROW a), P_2 (SIZE -a), outer ring (P_1 ~ P),
 * inner ring (P ~ P_2), ring_and1 (outer * P), ring_intersection
 * (outer * inner).  Asynchronous; capturable into a CUDA graph. */
int gb_op1(gb_context* ctx, gb_layer* P, int32_t a, gb_layer** outs);
/* The same chain plus the deck's Klee union area of P per cell, written to
 * d_area (device memory, one int64 per cell).  With a > 0 the area comes out
 * of the erosion's complement (area(frame) - area(frame \ P)) with no extra
 * pass; otherwise from a count-mode union of P.  Asynchronous, capturable. */
int gb_op1_area(gb_context* ctx, gb_layer* P, int32_t a, gb_layer** outs, long long* d_area);
/* The same deck through host buffers: boxes are copied in, the chain runs,
 * and per cell the six layer counts (counts[ncell*6], may be NULL) and the
 * union area of P (area[ncell], may be NULL) are copied out.  Layers of 4M
 * boxes or more run as two groups of cells whose uploads overlap the first
 * group's work (pinned host memory makes the copies asynchronous); the
 * device staging buffer stays with the context until it is destroyed.
 * *assert_failures receives the number of failing ASSERT_ZEROs. */
int gb_op1_host(gb_context* ctx, const c_box* boxes, unsigned long long n,
                const long long* cell_offsets, int ncell, int32_t a, long long* counts,
                long long* area, int* assert_failures);
/* gb_op1_host plus, per cell, a digest of each of the six result layers
 * (digests[ncell*6], [cell][layer]): the sum mod 2^64 of a 64-bit hash of
 * every strip (x1, y1, x2, y2 in global dbu), so equal canonical strips give
 * equal digests in any order (the same function as gb_layer_digest). */
int gb_op1_host_digest(gb_context* ctx, const c_box* boxes, unsigned long long n,
                       const long long* cell_offsets, int ncell, int32_t a, long long* counts,
                       long long* area, unsigned long long* digests, int* assert_failures);

/* ---- SNAP layer streams (box_codec.f90, serialization.f90, snappy_api.cpp)
 * A stream is the layer's boxes cut into chunks of 65536; each chunk is the
 * box codec's byte stream (infobyte, zigzag varint anchor deltas, width /
 * height dictionaries by first appearance: CompressBoxesUsingCodec,
 * box_codec.f90:616-698), compressed with method 1 (Snappy raw format, as
 * snappy_compress_buffer, box_codec.f90:732-734) or stored as is with
 * method 0.  ZLIB (2) and ZSTD (3) are refused with GB_ERR_ARG.
 * chunk_meta holds three int64 per chunk, as the chunk header of a .snap
 * file: num_boxes, raw_byte_size, compressed_size.  Synchronous. */
/* Bound of the device bytes a stream of n boxes can take. */
int gb_snap_max_bytes(long long n, long long* bytes);
/* CompressBoxesToStream (box_codec.f90:675-760) on n device boxes (16-byte
 * aligned).  The chunks' data go back to back into d_out (cap bytes;
 * GB_ERR_CAPACITY when short); chunk_meta (host, 3 * ceil(n / 65536)) and
 * *total (bytes used) are filled. */
int gb_compress_boxes_to_stream(gb_context* ctx, const c_box* d_boxes, long long n, int method,
                                unsigned char* d_out, long long cap, long long* chunk_meta, long long* total);
/* DecompressStreamToBoxes (box_codec.f90:765-880): num_chunks chunks whose
 * data lie back to back at d_data (device), described by chunk_meta (host),
 * into d_boxes (device, sum of num_boxes entries).  A malformed stream (codec
 * desync, bad Snappy element, sizes that disagree with the header) gives
 * GB_ERR_CORRUPT; the reference stops there. */
int gb_decompress_stream_to_boxes(gb_context* ctx, const unsigned char* d_data, const long long* chunk_meta,
                                  long long num_chunks, int method, c_box* d_boxes);
/* SaveLayerToSnap + SaveCompressedStreamToDisk (diskdesign_impl.f90:59-82,
 * serialization.f90:15-50): the .snap file of n device boxes.  pnum (host,
 * n int64, may be NULL) is stored after the header and sets the PNUM bit (4)
 * of layer_properties; without it the bit is cleared; the R-tree bit (8) is
 * never saved. */
int gb_save_layer_to_snap(gb_context* ctx, const char* path, const c_box* d_boxes, long long n, int method,
                          int layer_properties, const long long* pnum);
/* Header of a .snap file (an empty file is an empty layer). */
int gb_snap_file_info(const char* path, long long* total_boxes, long long* num_chunks, int* method,
                      int* layer_properties);
/* RestoreSnapToLayer (diskdesign_impl.f90:84-113): the file's boxes into
 * d_boxes (device, cap entries; *n receives the count, GB_ERR_CAPACITY when
 * cap is short) and, when pnum is not NULL and the file holds one, its PNUM
 * table (host, n int64). */
int gb_restore_snap_to_layer(gb_context* ctx, const char* path, c_box* d_boxes, long long cap, long long* n,
                             long long* pnum);

/* Tile grid of the operators on this context: slab height 2^g dbu,
 * 10 <= g <= 16 (default 16).  Results on two grids hold the same point set
 * and differ only in where strips are cut at tile edges. */
int gb_set_grid(gb_context* ctx, int g);
int gb_get_grid(gb_context* ctx);
/* Slab-height autotuner: runs the OP1 chain with the union area
 * (gb_op1_area) on P with amount a once untimed and once timed at each grid
 * g = 13..16 and leaves the fastest set on the context (*best_g).  ms_out
 * (4 floats, may be NULL) receives the times in ms, -1 for a grid that did
 * not run.  Synchronous. */
int gb_grid_autotune(gb_context* ctx, gb_layer* P, int32_t a, int* best_g, float* ms_out);

/* CUDA-graph capture of an operator chain on the context stream.  Every
 * replay restarts the work arena at the offset it had at gb_graph_begin. */
typedef struct gb_graph gb_graph;
int gb_graph_begin(gb_context* ctx);
int gb_graph_end(gb_context* ctx, gb_graph** out);
int gb_graph_launch(gb_context* ctx, gb_graph* g);
long long gb_graph_kernels(gb_graph* g);
void gb_graph_destroy(gb_graph* g);

/* Profiling: when on, every scanline-kernel launch is bracketed by CUDA
 * events; gb_profile_read returns their summed time, the launch count and
 * the algorithmic bytes the kernel read (pieces) and wrote (strips) since
 * gb_profile(ctx, 1).  on = 2 resets only the byte counters (event pairs
 * captured in a graph stay valid); on = 0 stops recording. */
int gb_profile(gb_context* ctx, int on);
int gb_profile_read(gb_context* ctx, double* ms_total, long long* launches, long long* bytes_in,
                    long long* bytes_out);
long long gb_launch_count(gb_context* ctx);
/* Diagnostics: per-phase cycle counters of the scanline kernel.  out8 (40
 * entries) gets cycles of phases A (ranks), B (sub-band lists), C (sub-band
 * sweeps), D (stitch/emit) summed over CTAs; tiles, pieces, sub-bands, strip
 * pieces; then 16 per-warp counters of the sub-band steps (compress,
 * rasterise, scan, count, write, transpose cycles, members, columns); then
 * per sub-band-count bucket (1, 2-3, 4-7, 8-15, 16-31, 32+) the tiles and
 * their phase-C cycles; the sub-bands whose column words spilled to scratch
 * and their cycles, the others and theirs; all since gb_tile_timing(ctx, 1). */
int gb_tile_timing(gb_context* ctx, int on);
/* Diagnostics: runs one radix pass whose only CTA waits for a predecessor
 * tile that never publishes; returns the status it reports (GB_ERR_TIMEOUT
 * when the bounded wait works) with the context status cleared again. */
int gb_debug_lookback_timeout(gb_context* ctx, int spin_limit);
int gb_tile_timing_read(gb_context* ctx, long long* out8);

#ifdef __cplusplus
}
#endif
#endif
