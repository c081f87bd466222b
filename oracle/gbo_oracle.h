/*
 * gbo_oracle.h -- CPU oracle for the Manhattan box-Boolean path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker (or the timed CPU baseline), never as the product path.
 *
 * It restates, in plain C++17 + OpenMP, the algorithms the reference runs on
 * the CPU for this path (file:line citations are relative to the reference
 * project, skoranne/VLSI_LAYOUT):
 *   - box validity / grow / clip          src/geometry.f90:66-70,184-215
 *   - um -> dbu truncation int(1000*r)     src/controlparser.f90:146,568-576
 *   - heal sweep (corner tokens, lap sum,  src/polygon_fracture.f90:805-1004
 *     prev/curr region merge-join)         (generalised to two owners with a
 *                                          Boolean predicate on the laps, the
 *                                          pattern of src/pboolean.f90:110-112)
 *   - Klee union area (segment tree)       src/geometry.f90:1840-1972
 *   - PNUM union-find (closed overlap,     src/pnummerge.f90:279-385,
 *     min-index root, relabel 1..R)        src/datastructures.f90:90-215
 *   - Morton key of the box centre         src/gpu_morton.cu:113-144
 *   - tracker key (X^sign)<<32|(Y^sign)    src/event_sorter.cu:48-59
 *
 * Canonical form.  The reference back ends return different rectangle lists
 * for the same point set (Boost re-tiles at 100000 dbu, FRAME cuts at its
 * tiles, heal_boxes emits maximal vertical strips).  Parity is therefore
 * defined on a canonical decomposition of the point set: the plane is cut by
 * a fixed grid of G = 2^grid_log2 dbu tiles (tile (i,j) = [iG,(i+1)G) x
 * [jG,(j+1)G)), and inside each tile the region is the heal_boxes strip form
 * (at every x the maximal y-intervals, merged along x while unchanged).  The
 * list is sorted by (x1, y1).  With a single tile this is exactly what
 * heal_boxes emits.
 */
#ifndef GBO_ORACLE_H
#define GBO_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int32_t x1, y1, x2, y2; } orc_box;

enum { ORC_XOR = 0, ORC_OR = 1, ORC_AND = 2, ORC_NOT = 3, ORC_MERGE = 4, ORC_OVERLAP = 7 };
/* ORC_OVERLAP: single-layer AND, the area covered by at least two boxes of A
 * (B unused). */

/* Canonical strips of pred(A, B) (op as above).  *out is malloc'd (free with
 * orc_free).  Returns the strip count, or -1 on invalid input boxes. */
int64_t orc_boolean(const orc_box* A, int64_t nA, const orc_box* B, int64_t nB,
                    int op, int grid_log2, orc_box** out);
/* GROW: box_grow_directional(E,N,W,S) on every box, then heal (union). */
int64_t orc_grow(const orc_box* A, int64_t n, int32_t E, int32_t N, int32_t W,
                 int32_t S, int grid_log2, orc_box** out);
/* SIZE(s): Minkowski dilation (s>0) / erosion (s<0) of the union by the
 * square [-|s|,|s|]^2; s == 0 is the union. */
int64_t orc_size(const orc_box* A, int64_t n, int32_t s, int grid_log2, orc_box** out);
/* Union area as int64 (calculate_union_area_fast). */
int64_t orc_union_area(const orc_box* A, int64_t n);
/* PNUM connectivity.  labels (optional, n entries): 0 for singletons, else
 * 1..R with roots numbered in index order.  Returns the component count
 * (non-singleton components + singletons). */
int64_t orc_components(const orc_box* A, int64_t n, int64_t* labels);
/* Overlap statistics of one layer: *pairs = pairs i<k whose boxes overlap
 * with positive area (ComputeInteractionsCPU, pnummerge.f90:483-562);
 * *singletons = boxes with no other box touching or overlapping them
 * (closed bounds, FindSingletonsCPU, pnummerge.f90:388-482); is_singleton
 * (optional, n entries) gets the mask. */
void orc_interactions(const orc_box* A, int64_t n, int64_t* pairs, int64_t* singletons,
                      uint8_t* is_singleton);
/* Union area per PNUM component (calculate_union_area_by_polygon,
 * design.f90:854-935): areas[0] = total area of the singletons, areas[k] =
 * union area of component k (labels of orc_components).  Returns R, the
 * number of non-singleton components (areas holds R + 1 entries; pass
 * areas = NULL to size it). */
int64_t orc_component_areas(const orc_box* A, int64_t n, int64_t* areas);
uint64_t orc_morton_key(const orc_box* b);
uint64_t orc_tracker_key(int32_t X, int32_t Y);
int32_t orc_um_to_dbu(double r);
/* Sort boxes by (x1, y1, x2, y2) in place. */
void orc_canonical_sort(orc_box* A, int64_t n);
/* OP1 ring-check deck on one layer (op_template.m4:14-22): returns the box
 * counts of the two ASSERT_ZERO layers and every intermediate layer, plus
 * the union area.  counts[8]: poly_1, poly_2, outer, inner, and1, inter,
 * merged(poly), unused. */
void orc_op1(const orc_box* A, int64_t n, int32_t amount, int grid_log2,
             int64_t* counts, int64_t* area);
/* orc_op1 plus the strip digests of its seven layers (digests[7]: poly_1,
 * poly_2, outer, inner, and1, inter, merged); one layer, every operator
 * parallel over its tiles. */
void orc_op1_digest(const orc_box* A, int64_t n, int32_t amount, int grid_log2,
                    int64_t* counts, int64_t* area, uint64_t* digests);
/* orc_op1 over ncell cells (off[ncell+1]), cells in parallel: counts[8*k..]. */
void orc_op1_cells(const orc_box* A, const int64_t* off, int64_t ncell, int32_t amount, int grid_log2,
                   int64_t* counts, int64_t* area);
/* orc_op1_cells plus per-cell strip digests digests[7*k..]: poly_1, poly_2,
 * outer, inner, and1, inter, merged(P) (orc_strip_digest of each layer). */
void orc_op1_cells_digest(const orc_box* A, const int64_t* off, int64_t ncell, int32_t amount, int grid_log2,
                          int64_t* counts, int64_t* area, uint64_t* digests);
/* 64-bit hash of one strip: fmix64((x1<<32|y1) ^ fmix64((x2<<32|y2) +
 * 0x9e3779b97f4a7c15)), coordinates as uint32 (MurmurHash3's finaliser). */
uint64_t orc_strip_hash(int32_t x1, int32_t y1, int32_t x2, int32_t y2);
/* Sum mod 2^64 of orc_strip_hash over a strip list: independent of order. */
uint64_t orc_strip_digest(const orc_box* A, int64_t n);
/* The reference's CPU path for the OP1 deck, restated (gbo_refpath.cpp): the
 * timed CPU baseline.  counts[6*k..] per cell: boxes of poly_1, poly_2,
 * outer, inner, and1, inter in the reference's own decompositions (FRAME
 * tiles, pairwise AND clips), area[k] the union area; cells in parallel. */
void orc_refpath_op1_cells(const orc_box* A, const int64_t* off, int64_t ncell, int32_t amount, int64_t* counts,
                           int64_t* area);
/* One of those six layers (which = 0..5) of one cell; *out malloc'd. */
int64_t orc_refpath_op1_layer(const orc_box* A, int64_t n, int32_t amount, int which, orc_box** out);
/* SubtractBox (boolean_ops_rtree.f90:139-186): subject minus clip as up to
 * four pieces written to out4; returns their count. */
int64_t orc_refpath_subtract(const orc_box* subject, const orc_box* clip, orc_box* out4);
void orc_free(void* p);
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
