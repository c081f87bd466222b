// gbo_refpath.cpp -- the reference's CPU path for the OP1 deck, restated.
//
// TEST INFRASTRUCTURE ONLY (see gbo_oracle.h): this is the timed CPU baseline
// (bench.py's cpu_baseline and --impl reference arm), never the product path.
//
// It follows the operators the reference's control language runs on the CPU
// (file:line citations relative to skoranne/VLSI_LAYOUT), with Boost.Polygon
// (absent here, unpinned) replaced by the reference's own CPU routines: the
// heal_boxes sweep for MERGE, CalculateNOTRTree's fracture for NOT:
//   - GROW: CalculateGROWLayer (design_impl.f90:571-586): grow every box, build
//     the tree (sort), MergeHealLayer (design_impl.f90:1318-1341): heal_boxes
//     below K_FRAME_THRESHOLD boxes, else FRAME merge per K x K tile
//     (CalculateFrameFunction1) with no re-heal across tiles;
//   - SIZE: one whole-layer Minkowski operation (CalculateBoostOperation,
//     design_impl.f90:931-951); the erosion is the oracle's own definition;
//   - `~` FRAME-NOT: CalculateFrameFunction2 (design_impl.f90:993-1129): heal
//     both operands when needed, K = int(nodes^(1/4)) with nodes =
//     CalculateTotalNodes(max(NA,NB), 16) (rtree.f90:19-35), the balanced
//     K x K grid over MBR(A) (CreateGrid, design_impl.f90:159-275), per tile
//     FilterLayer (design_impl.f90:99-143: R-tree query, clip, drop empty) of
//     A and B and A \ B by the reference's own CPU NOT, CalculateNOTRTree
//     (boolean_ops_rtree.f90:26-136: each box of A fractured iteratively by
//     the boxes of B its R-tree query returns, SubtractBox,
//     boolean_ops_rtree.f90:139-186), then the tiles' outputs concatenated,
//     the tree built and the result healed again;
//   - `*` AND: CalculateAND (design.f90:1131-1235): every box of A queries B's
//     R-tree and emits a (*) b for every interacting b whose clip has positive
//     area (the reference's output is these pairwise clips, unhealed);
//   - the R-tree: boxes sorted by the device Morton key of their centre
//     (gpu_morton.cu:113-144), packed bottom-up with 16 entries per node
//     (BuildRTree, rtree.f90:55-130; K_LEAF_CAPACITY, commonmodule.f90:8),
//     searched with closed overlap (SearchTreeRecursive, rtree.f90:134-193);
//   - box_interact (geometry.f90:102-118): closed overlap, except a single
//     common point.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gbo_internal.h"
#include "gbo_oracle.h"

namespace {

using gbo::Box;
using gbo::Piece;

constexpr int64_t K_LEAF = 16;              // K_LEAF_CAPACITY, commonmodule.f90:8
constexpr int64_t K_FRAME_THRESHOLD = 1024;  // commonmodule.f90:23

inline bool valid(const Box& b) { return b.x1 < b.x2 && b.y1 < b.y2; }

// box_interact (geometry.f90:102-118): the closed boxes meet, and not in a
// single point.
inline bool interact(const Box& a, const Box& b) {
  if (a.x1 > b.x2 || a.y1 > b.y2 || a.x2 < b.x1 || a.y2 < b.y1) return false;
  const int32_t x1 = std::max(a.x1, b.x1), y1 = std::max(a.y1, b.y1);
  const int32_t x2 = std::min(a.x2, b.x2), y2 = std::min(a.y2, b.y2);
  return !(x1 == x2 && y1 == y2);
}

inline Box clip(const Box& a, const Box& b) {
  return {std::max(a.x1, b.x1), std::max(a.y1, b.y1), std::min(a.x2, b.x2), std::min(a.y2, b.y2)};
}

Box mbr(const std::vector<Box>& v) {
  Box m{INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN};
  for (const Box& b : v) {
    m.x1 = std::min(m.x1, b.x1); m.y1 = std::min(m.y1, b.y1);
    m.x2 = std::max(m.x2, b.x2); m.y2 = std::max(m.y2, b.y2);
  }
  return m;
}

// Packed R-tree: level 0 holds the MBR of every K_LEAF consecutive boxes,
// each higher level the MBR of K_LEAF consecutive nodes of the level below.
struct RTree {
  std::vector<std::vector<Box>> lv;
};

struct RLayer {
  std::vector<Box> b;
  bool healed = false;
  bool treed = false;
  RTree t;
};

// BuildTree (diskdesign_impl.f90:40-57): sort, then BuildRTree.
void build_tree(RLayer& L) {
  if (L.treed) return;
  std::vector<std::pair<uint64_t, Box>> k(L.b.size());
  for (size_t i = 0; i < L.b.size(); ++i) k[i] = {orc_morton_key((const orc_box*)&L.b[i]), L.b[i]};
  std::stable_sort(k.begin(), k.end(), [](const auto& a, const auto& c) { return a.first < c.first; });
  for (size_t i = 0; i < k.size(); ++i) L.b[i] = k[i].second;
  L.t.lv.clear();
  std::vector<Box> cur;
  for (size_t i = 0; i < L.b.size(); i += K_LEAF) {
    std::vector<Box> part(L.b.begin() + i, L.b.begin() + std::min(L.b.size(), i + (size_t)K_LEAF));
    cur.push_back(mbr(part));
  }
  while (!cur.empty()) {
    L.t.lv.push_back(cur);
    if (cur.size() == 1) break;
    std::vector<Box> up;
    for (size_t i = 0; i < cur.size(); i += K_LEAF) {
      std::vector<Box> part(cur.begin() + i, cur.begin() + std::min(cur.size(), i + (size_t)K_LEAF));
      up.push_back(mbr(part));
    }
    cur.swap(up);
  }
  L.treed = true;
}

inline bool node_overlap(const Box& n, const Box& q) {
  return std::max(n.x1, q.x1) <= std::min(n.x2, q.x2) && std::max(n.y1, q.y1) <= std::min(n.y2, q.y2);
}

// SearchTreeRecursive: the first box index of every leaf whose MBR meets q.
void search(const RTree& t, int level, size_t node, const Box& q, std::vector<int64_t>& leaves) {
  if (!node_overlap(t.lv[level][node], q)) return;
  if (level == 0) {
    leaves.push_back((int64_t)node * K_LEAF);
    return;
  }
  const size_t c0 = node * K_LEAF, c1 = std::min(t.lv[level - 1].size(), c0 + (size_t)K_LEAF);
  for (size_t c = c0; c < c1; ++c) search(t, level - 1, c, q, leaves);
}
void search_tree(const RTree& t, const Box& q, std::vector<int64_t>& leaves) {
  leaves.clear();
  if (t.lv.empty()) return;
  search(t, (int)t.lv.size() - 1, 0, q, leaves);
}

// FilterLayer: L's boxes meeting the window, clipped to it, empty clips dropped.
void filter_layer(const RLayer& L, const Box& w, std::vector<Piece>& out, uint8_t owner) {
  std::vector<int64_t> leaves;
  search_tree(L.t, w, leaves);
  for (int64_t s : leaves)
    for (int64_t k = s; k < std::min<int64_t>(s + K_LEAF, (int64_t)L.b.size()); ++k)
      if (interact(w, L.b[k])) {
        const Box c = clip(w, L.b[k]);
        if (valid(c)) out.push_back({c, owner});
      }
}

int64_t total_nodes(int64_t n) {  // CalculateTotalNodes(n, 16)
  if (n == 0) return 0;
  int64_t cur = (n + K_LEAF - 1) / K_LEAF, tot = cur;
  while (cur > 1) {
    cur = (cur + K_LEAF - 1) / K_LEAF;
    tot += cur;
  }
  return tot;
}

int frame_k(int64_t n) {  // K_GRID = int(sqrt(sqrt(real(nodes))))
  return std::max(1, (int)std::sqrt(std::sqrt((double)total_nodes(n))));
}

// CreateGrid with GridOverlap 0: rows x cols tiles over the MBR, remainders
// given to the first rows / columns.
std::vector<Box> create_grid(const Box& m, int rows, int cols) {
  const int32_t fw = m.x2 - m.x1, fh = m.y2 - m.y1;
  const int32_t cw = fw / cols, ew = fw % cols, rh = fh / rows, eh = fh % rows;
  std::vector<Box> g;
  for (int i = 1; i <= rows; ++i) {
    const int32_t y0 = m.y1 + (i - 1) * rh + std::min(i - 1, eh), y1 = m.y1 + i * rh + std::min(i, eh);
    for (int j = 1; j <= cols; ++j) {
      const int32_t x0 = m.x1 + (j - 1) * cw + std::min(j - 1, ew), x1 = m.x1 + j * cw + std::min(j, ew);
      g.push_back({x0, y0, x1, y1});
    }
  }
  return g;
}

// heal_boxes on the whole layer.
void heal_boxes(RLayer& L) {
  std::vector<Piece> p(L.b.size());
  for (size_t i = 0; i < L.b.size(); ++i) p[i] = {L.b[i], 0};
  std::vector<Box> out;
  gbo::sweep_tile(p, ORC_MERGE, out);
  L.b.swap(out);
  L.healed = true;
  L.treed = false;
}

// SubtractBox (boolean_ops_rtree.f90:139-186): subject minus clip as up to
// four disjoint pieces (left, right, bottom-middle, top-middle).
int subtract_box(const Box& s, const Box& c, Box* o) {
  if (s.x2 <= c.x1 || s.x1 >= c.x2 || s.y2 <= c.y1 || s.y1 >= c.y2) {
    o[0] = s;
    return 1;
  }
  const int32_t ix1 = std::max(s.x1, c.x1), iy1 = std::max(s.y1, c.y1);
  const int32_t ix2 = std::min(s.x2, c.x2), iy2 = std::min(s.y2, c.y2);
  int k = 0;
  if (s.x1 < ix1) o[k++] = {s.x1, s.y1, ix1, s.y2};
  if (s.x2 > ix2) o[k++] = {ix2, s.y1, s.x2, s.y2};
  if (s.y1 < iy1) o[k++] = {ix1, s.y1, ix2, iy1};
  if (s.y2 > iy2) o[k++] = {ix1, iy2, ix2, s.y2};
  return k;
}

// CalculateNOTRTree (boolean_ops_rtree.f90:26-136): every box of A is
// fractured by the boxes of B that B's R-tree returns for it.
void not_rtree(const std::vector<Box>& A, const std::vector<Box>& Bv, std::vector<Box>& out) {
  RLayer B;
  B.b = Bv;
  build_tree(B);
  std::vector<int64_t> leaves;
  std::vector<Box> frag, next;
  Box f4[4];
  for (const Box& a : A) {
    search_tree(B.t, a, leaves);
    frag.assign(1, a);
    for (int64_t s : leaves) {
      for (int64_t k = s; k < std::min<int64_t>(s + K_LEAF, (int64_t)B.b.size()) && !frag.empty(); ++k) {
        next.clear();
        for (const Box& f : frag) {
          const int nf = subtract_box(f, B.b[k], f4);
          next.insert(next.end(), f4, f4 + nf);
        }
        frag.swap(next);
      }
      if (frag.empty()) break;
    }
    out.insert(out.end(), frag.begin(), frag.end());
  }
}

// The tiled FRAME computation: op on the pieces of A (and B) inside each tile
// (NOT by fracture, MERGE by the heal_boxes sweep).
void frame_tiles(RLayer& A, RLayer* B, int op, int K, std::vector<Box>& out) {
  build_tree(A);
  if (B) build_tree(*B);
  const std::vector<Box> grid = create_grid(mbr(A.b), K, K);
  std::vector<std::vector<Box>> part(grid.size());
  for (size_t t = 0; t < grid.size(); ++t) {
    std::vector<Piece> pa, pb;
    filter_layer(A, grid[t], pa, 0);
    if (op == ORC_NOT) {
      filter_layer(*B, grid[t], pb, 1);
      std::vector<Box> a(pa.size()), b(pb.size());
      for (size_t i = 0; i < pa.size(); ++i) a[i] = pa[i].b;
      for (size_t i = 0; i < pb.size(); ++i) b[i] = pb[i].b;
      not_rtree(a, b, part[t]);
    } else {
      gbo::sweep_tile(pa, op, part[t]);
    }
  }
  out.clear();
  for (auto& v : part) out.insert(out.end(), v.begin(), v.end());
}

// MergeHealLayer (design_impl.f90:1318-1341).
void merge_heal(RLayer& L) {
  if ((int64_t)L.b.size() < K_FRAME_THRESHOLD) {
    heal_boxes(L);
    return;
  }
  std::vector<Box> out;
  frame_tiles(L, nullptr, ORC_MERGE, frame_k((int64_t)L.b.size()), out);  // CalculateFrameFunction1
  L.b.swap(out);
  L.healed = true;
  L.treed = false;
}

// CalculateGROWLayer.
RLayer grow_layer(const RLayer& P, int32_t e, int32_t n, int32_t w, int32_t s) {
  RLayer G;
  gbo::grow_all(P.b.data(), (int64_t)P.b.size(), e, n, w, s, G.b);
  build_tree(G);
  merge_heal(G);
  return G;
}

// CalculateFrameFunction2 with A \ B per tile.
RLayer frame_not(RLayer& A, RLayer& B) {
  RLayer O;
  if (A.b.empty()) return O;
  if (!A.healed) merge_heal(A);
  if (!B.healed) merge_heal(B);
  frame_tiles(A, &B, ORC_NOT, frame_k((int64_t)std::max(A.b.size(), B.b.size())), O.b);
  build_tree(O);
  merge_heal(O);
  return O;
}

// CalculateAND: pairwise clips of positive area.
RLayer and_layer(RLayer& A, RLayer& B) {
  RLayer O;
  build_tree(A);
  build_tree(B);
  std::vector<int64_t> leaves;
  for (const Box& a : A.b) {
    search_tree(B.t, a, leaves);
    for (int64_t s : leaves)
      for (int64_t k = s; k < std::min<int64_t>(s + K_LEAF, (int64_t)B.b.size()); ++k)
        if (interact(a, B.b[k])) {
          const Box c = clip(a, B.b[k]);
          if ((int64_t)(c.x2 - c.x1) * (int64_t)(c.y2 - c.y1) > 0) O.b.push_back(c);
        }
  }
  O.healed = true;  // disjoint by construction when A and B are healed (design.f90:1230-1232)
  return O;
}

void op1_impl(const orc_box* Ab, int64_t n, int32_t a, std::vector<Box>* layers, int64_t* counts, int64_t* area) {
  RLayer P;
  P.b.assign((const Box*)Ab, (const Box*)Ab + n);
  RLayer p1 = grow_layer(P, a, a, a, a);
  RLayer p2;
  gbo::size_impl(P.b.data(), (int64_t)P.b.size(), -a, 30, p2.b);  // one whole-layer operation
  p2.healed = true;
  RLayer outer = frame_not(p1, P);
  RLayer inner = frame_not(P, p2);
  RLayer and1 = and_layer(outer, P);
  RLayer inter = and_layer(outer, inner);
  const RLayer* L[6] = {&p1, &p2, &outer, &inner, &and1, &inter};
  for (int k = 0; k < 6; ++k) {
    if (counts) counts[k] = (int64_t)L[k]->b.size();
    if (layers) layers[k] = L[k]->b;
  }
  if (area) *area = orc_union_area(Ab, n);  // calculate_union_area_fast
}

}  // namespace

extern "C" {

void orc_refpath_op1_cells(const orc_box* A, const int64_t* off, int64_t ncell, int32_t amount, int64_t* counts,
                           int64_t* area) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ncell; ++k)
    op1_impl(A + off[k], off[k + 1] - off[k], amount, nullptr, counts + 6 * k, area + k);
}

int64_t orc_refpath_op1_layer(const orc_box* A, int64_t n, int32_t amount, int which, orc_box** out) {
  std::vector<Box> layers[6];
  int64_t area = 0;
  if (which < 0 || which > 5) return -1;
  op1_impl(A, n, amount, layers, nullptr, &area);
  const std::vector<Box>& v = layers[which];
  *out = (orc_box*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(orc_box));
  if (!v.empty()) std::memcpy(*out, v.data(), v.size() * sizeof(orc_box));
  return (int64_t)v.size();
}

int64_t orc_refpath_subtract(const orc_box* subject, const orc_box* clip_box, orc_box* out4) {
  return subtract_box(*(const Box*)subject, *(const Box*)clip_box, (Box*)out4);
}

}  // extern "C"
