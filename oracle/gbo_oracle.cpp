// gbo_oracle.cpp -- CPU oracle for the Manhattan box-Boolean path.
//
// TEST INFRASTRUCTURE ONLY (see gbo_oracle.h): the checker the CUDA path is
// compared against, and the CPU baseline that bench.py times.  Nothing in the
// product library links or calls this file.
//
// Build: g++ -O3 -std=c++17 -fopenmp -shared -fPIC gbo_oracle.cpp -o libgbo_oracle.so
#include "gbo_oracle.h"
#include "gbo_internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace gbo {

inline bool valid(const Box& b) { return b.x1 < b.x2 && b.y1 < b.y2; }  // geometry.f90:66-70

// ca, cb: how many boxes of A and of B cover the point
inline bool pred(int op, int32_t ca, int32_t cb) {
  const bool a = ca > 0, b = cb > 0;
  switch (op) {
    case ORC_XOR: return a != b;
    case ORC_OR: return a || b;
    case ORC_AND: return a && b;
    case ORC_NOT: return a && !b;
    case ORC_OVERLAP: return ca >= 2;  // CalculateSingleLayerAND, design_impl.f90:385-498
    default: return a;  // ORC_MERGE
  }
}

inline int32_t tile_of(int32_t v, int g) { return (int32_t)((int64_t)v >> g); }  // floor(v / 2^g)

// One corner token of polygon_fracture.f90:824-833: +1 at (x1,y1) and (x2,y2),
// -1 at (x1,y2) and (x2,y1); the owner selects which lap counter it updates.
struct Tok { int32_t x, y; int8_t s; uint8_t o; };

struct Region { int32_t y1, y2, xs; };

// heal_boxes (polygon_fracture.f90:805-1004) generalised to two owners: the
// skip list of y -> lap_change becomes an ordered map y -> (dA, dB); at every
// new X the y-prefix sums give covA/covB of the slab right of X, the predicate
// selects the covered y-intervals, and the prev/curr merge-join keeps a region
// open while its (y1,y2) is unchanged, emitting [x_start, X] x [y1, y2] when it
// changes (:931-964).
void sweep_tile(const std::vector<Piece>& pcs, int op, std::vector<Box>& out) {
  if (pcs.empty()) return;
  std::vector<Tok> tok;
  tok.reserve(pcs.size() * 4);
  for (const Piece& p : pcs) {
    tok.push_back({p.b.x1, p.b.y1, +1, p.owner});
    tok.push_back({p.b.x1, p.b.y2, -1, p.owner});
    tok.push_back({p.b.x2, p.b.y1, -1, p.owner});
    tok.push_back({p.b.x2, p.b.y2, +1, p.owner});
  }
  std::sort(tok.begin(), tok.end(), [](const Tok& a, const Tok& b) {
    return a.x != b.x ? a.x < b.x : a.y < b.y;
  });
  std::map<int32_t, std::pair<int32_t, int32_t>> lap;
  std::vector<Region> prev, curr;
  size_t i = 0;
  while (i < tok.size()) {
    const int32_t X = tok[i].x;
    for (; i < tok.size() && tok[i].x == X; ++i) {
      auto& d = lap[tok[i].y];
      if (tok[i].o == 0) d.first += tok[i].s; else d.second += tok[i].s;
      if (d.first == 0 && d.second == 0) lap.erase(tok[i].y);
    }
    curr.clear();
    int32_t ca = 0, cb = 0, ys = 0;
    bool in = false;
    for (const auto& kv : lap) {
      ca += kv.second.first;
      cb += kv.second.second;
      const bool now = pred(op, ca, cb);
      if (!in && now) { ys = kv.first; in = true; }
      else if (in && !now) { curr.push_back({ys, kv.first, X}); in = false; }
    }
    size_t p = 0, c = 0;
    while (p < prev.size() && c < curr.size()) {
      if (prev[p].y1 == curr[c].y1 && prev[p].y2 == curr[c].y2) {
        curr[c].xs = prev[p].xs; ++p; ++c;
      } else if (prev[p].y1 < curr[c].y1) {
        if (X > prev[p].xs) out.push_back({prev[p].xs, prev[p].y1, X, prev[p].y2});
        ++p;
      } else if (prev[p].y1 > curr[c].y1) {
        ++c;
      } else {
        if (X > prev[p].xs) out.push_back({prev[p].xs, prev[p].y1, X, prev[p].y2});
        ++p;
      }
    }
    for (; p < prev.size(); ++p)
      if (X > prev[p].xs) out.push_back({prev[p].xs, prev[p].y1, X, prev[p].y2});
    prev.swap(curr);
  }
}

bool cmp_box(const Box& a, const Box& b) {
  if (a.x1 != b.x1) return a.x1 < b.x1;
  if (a.y1 != b.y1) return a.y1 < b.y1;
  if (a.x2 != b.x2) return a.x2 < b.x2;
  return a.y2 < b.y2;
}

// Clip every box to the fixed 2^g grid and run one sweep per tile.
int64_t boolean_impl(const Box* A, int64_t nA, const Box* B, int64_t nB, int op, int g,
                     std::vector<Box>& res) {
  res.clear();
  for (int64_t i = 0; i < nA; ++i) if (!valid(A[i])) return -1;
  for (int64_t i = 0; i < nB; ++i) if (!valid(B[i])) return -1;
  std::unordered_map<int64_t, int64_t> tix;
  std::vector<std::vector<Piece>> tiles;
  auto add = [&](const Box& b, uint8_t owner) {
    const int32_t tx0 = tile_of(b.x1, g), tx1 = tile_of(b.x2 - 1, g);
    const int32_t ty0 = tile_of(b.y1, g), ty1 = tile_of(b.y2 - 1, g);
    for (int32_t ty = ty0; ty <= ty1; ++ty)
      for (int32_t tx = tx0; tx <= tx1; ++tx) {
        const int64_t key = ((int64_t)ty << 32) ^ (int64_t)(uint32_t)tx;
        auto it = tix.find(key);
        int64_t t;
        if (it == tix.end()) { t = (int64_t)tiles.size(); tix.emplace(key, t); tiles.emplace_back(); }
        else t = it->second;
        const int64_t X0 = (int64_t)tx << g, Y0 = (int64_t)ty << g;
        Box c{(int32_t)std::max<int64_t>(b.x1, X0), (int32_t)std::max<int64_t>(b.y1, Y0),
              (int32_t)std::min<int64_t>(b.x2, X0 + (1LL << g)),
              (int32_t)std::min<int64_t>(b.y2, Y0 + (1LL << g))};
        tiles[t].push_back({c, owner});
      }
  };
  for (int64_t i = 0; i < nA; ++i) add(A[i], 0);
  if (op != ORC_MERGE && op != ORC_OVERLAP)
    for (int64_t i = 0; i < nB; ++i) add(B[i], 1);
  const int64_t nt = (int64_t)tiles.size();
  std::vector<std::vector<Box>> outs(nt);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = 0; t < nt; ++t) sweep_tile(tiles[t], op, outs[t]);
  size_t tot = 0;
  for (auto& o : outs) tot += o.size();
  res.reserve(tot);
  for (auto& o : outs) res.insert(res.end(), o.begin(), o.end());
  std::sort(res.begin(), res.end(), cmp_box);
  return (int64_t)res.size();
}

int64_t export_boxes(const std::vector<Box>& v, orc_box** out) {
  if (!out) return (int64_t)v.size();
  *out = (orc_box*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(orc_box));
  if (!v.empty()) std::memcpy(*out, v.data(), v.size() * sizeof(orc_box));
  return (int64_t)v.size();
}

// box_grow_directional (geometry.f90:184-193): x2+=E, y2+=N, x1-=W, y1-=S; the
// grown box must stay valid and inside int32.
bool grow_all(const Box* A, int64_t n, int32_t E, int32_t N, int32_t W, int32_t S,
              std::vector<Box>& g) {
  g.resize(n);
  for (int64_t i = 0; i < n; ++i) {
    if (!valid(A[i])) return false;
    const int64_t x1 = (int64_t)A[i].x1 - W, x2 = (int64_t)A[i].x2 + E;
    const int64_t y1 = (int64_t)A[i].y1 - S, y2 = (int64_t)A[i].y2 + N;
    if (x1 >= x2 || y1 >= y2 || x1 < INT32_MIN || y1 < INT32_MIN || x2 > INT32_MAX || y2 > INT32_MAX)
      return false;
    g[i] = {(int32_t)x1, (int32_t)y1, (int32_t)x2, (int32_t)y2};
  }
  return true;
}

int64_t grow_impl(const Box* A, int64_t n, int32_t E, int32_t N, int32_t W, int32_t S, int g,
                  std::vector<Box>& res) {
  std::vector<Box> grown;
  if (!grow_all(A, n, E, N, W, S, grown)) return -1;
  return boolean_impl(grown.data(), n, nullptr, 0, ORC_MERGE, g, res);
}

// SIZE(-t) = closure(P \ ((F \ P) (+) [-t,t]^2)) with F = bbox(P) grown by t:
// every complement point within L-inf distance t of P lies in F, so this is
// the Minkowski erosion of the union by the square.
int64_t size_impl(const Box* A, int64_t n, int32_t s, int g, std::vector<Box>& res) {
  if (s > 0) return grow_impl(A, n, s, s, s, s, g, res);
  if (s == 0 || n == 0) return boolean_impl(A, n, nullptr, 0, ORC_MERGE, g, res);
  const int32_t t = -s;
  Box bb{INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN};
  for (int64_t i = 0; i < n; ++i) {
    if (!valid(A[i])) return -1;
    bb.x1 = std::min(bb.x1, A[i].x1); bb.y1 = std::min(bb.y1, A[i].y1);
    bb.x2 = std::max(bb.x2, A[i].x2); bb.y2 = std::max(bb.y2, A[i].y2);
  }
  std::vector<Box> frame;
  if (!grow_all(&bb, 1, t, t, t, t, frame)) return -1;
  std::vector<Box> q, d;
  if (boolean_impl(frame.data(), 1, A, n, ORC_NOT, g, q) < 0) return -1;
  if (grow_impl(q.data(), (int64_t)q.size(), t, t, t, t, g, d) < 0) return -1;
  return boolean_impl(A, n, d.data(), (int64_t)d.size(), ORC_NOT, g, res);
}

// ---- Klee's measure: calculate_union_area_fast (geometry.f90:1840-1927) ----
struct Ev { int32_t x, y1, y2; int8_t lap; };

void update_tree(int node, int s, int e, int l, int r, int val, const std::vector<int32_t>& uy,
                 std::vector<int32_t>& cnt, std::vector<int64_t>& len) {  // geometry.f90:1933-1972
  if (l <= s && e <= r) {
    cnt[node] += val;
  } else {
    const int mid = s + (e - s) / 2;
    if (l <= mid) update_tree(2 * node, s, mid, l, r, val, uy, cnt, len);
    if (r > mid) update_tree(2 * node + 1, mid + 1, e, l, r, val, uy, cnt, len);
  }
  if (cnt[node] > 0) len[node] = (int64_t)uy[e + 1] - uy[s];
  else if (s == e) len[node] = 0;
  else len[node] = len[2 * node] + len[2 * node + 1];
}

}  // namespace gbo

using namespace gbo;

extern "C" {

int64_t orc_boolean(const orc_box* A, int64_t nA, const orc_box* B, int64_t nB, int op,
                    int grid_log2, orc_box** out) {
  std::vector<Box> res;
  const int64_t n = boolean_impl((const Box*)A, nA, (const Box*)B, nB, op, grid_log2, res);
  if (n < 0) return -1;
  return export_boxes(res, out);
}

int64_t orc_grow(const orc_box* A, int64_t n, int32_t E, int32_t N, int32_t W, int32_t S,
                 int grid_log2, orc_box** out) {
  std::vector<Box> res;
  if (grow_impl((const Box*)A, n, E, N, W, S, grid_log2, res) < 0) return -1;
  return export_boxes(res, out);
}

int64_t orc_size(const orc_box* A, int64_t n, int32_t s, int grid_log2, orc_box** out) {
  std::vector<Box> res;
  if (size_impl((const Box*)A, n, s, grid_log2, res) < 0) return -1;
  return export_boxes(res, out);
}

int64_t orc_union_area(const orc_box* Ab, int64_t n) {
  const Box* A = (const Box*)Ab;
  if (n <= 0) return 0;
  std::vector<int32_t> yv(2 * n);
  for (int64_t i = 0; i < n; ++i) {
    yv[2 * i] = std::min(A[i].y1, A[i].y2);
    yv[2 * i + 1] = std::max(A[i].y1, A[i].y2);
  }
  std::sort(yv.begin(), yv.end());
  yv.erase(std::unique(yv.begin(), yv.end()), yv.end());
  std::vector<Ev> ev(2 * n);
  for (int64_t i = 0; i < n; ++i) {
    const int32_t y1 = std::min(A[i].y1, A[i].y2), y2 = std::max(A[i].y1, A[i].y2);
    ev[2 * i] = {std::min(A[i].x1, A[i].x2), y1, y2, +1};
    ev[2 * i + 1] = {std::max(A[i].x1, A[i].x2), y1, y2, -1};
  }
  std::sort(ev.begin(), ev.end(), [](const Ev& a, const Ev& b) { return a.x < b.x; });
  const int num_y = (int)yv.size();
  if (num_y < 2) return 0;
  std::vector<int32_t> cnt(4 * (size_t)num_y, 0);
  std::vector<int64_t> len(4 * (size_t)num_y, 0);
  int64_t area = 0, cur = ev[0].x;
  for (const Ev& e : ev) {
    const int64_t dx = (int64_t)e.x - cur;
    if (dx > 0) { area += dx * len[1]; cur = e.x; }
    const int j1 = (int)(std::lower_bound(yv.begin(), yv.end(), e.y1) - yv.begin());
    const int j2 = (int)(std::lower_bound(yv.begin(), yv.end(), e.y2) - yv.begin());
    if (j1 < j2) update_tree(1, 0, num_y - 2, j1, j2 - 1, e.lap, yv, cnt, len);
  }
  return area;
}

// PerformMerge (pnummerge.f90:279-385): every pair i<k whose boxes overlap with
// closed bounds (<=, so edge and corner touches count, :341-342) is an edge;
// UnionFind keeps the smaller index as root (datastructures.f90:90-112) and
// fullreduce numbers the roots 1..R in index order, singletons staying 0
// (:143-171).  The component count is count_roots() + count(arr == 0)
// (magparser.f90:372-373).  Candidate pairs come from an x1-sorted sweep
// instead of the R-tree; the pair set is the same.
int64_t orc_components(const orc_box* Ab, int64_t n, int64_t* labels) {
  const Box* A = (const Box*)Ab;
  if (n <= 0) return 0;
  std::vector<int64_t> ord(n), par(n);
  std::vector<uint8_t> touched(n, 0);
  for (int64_t i = 0; i < n; ++i) { ord[i] = i; par[i] = i; }
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
    return A[a].x1 != A[b].x1 ? A[a].x1 < A[b].x1 : a < b;
  });
  auto find = [&](int64_t x) {
    while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
    return x;
  };
  for (int64_t s = 0; s < n; ++s) {
    const Box& bi = A[ord[s]];
    for (int64_t t = s + 1; t < n && A[ord[t]].x1 <= bi.x2; ++t) {
      const Box& bk = A[ord[t]];
      if (std::max(bi.y1, bk.y1) <= std::min(bi.y2, bk.y2)) {
        touched[ord[s]] = touched[ord[t]] = 1;
        int64_t ra = find(ord[s]), rb = find(ord[t]);
        if (ra != rb) { if (ra < rb) par[rb] = ra; else par[ra] = rb; }
      }
    }
  }
  int64_t next = 1, comps = 0;
  std::vector<int64_t> map(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t r = find(i);
    if (!touched[i]) { ++comps; if (labels) labels[i] = 0; continue; }
    if (r == i) { map[i] = next++; ++comps; }
  }
  if (labels)
    for (int64_t i = 0; i < n; ++i)
      if (touched[i]) labels[i] = map[find(i)];
  return comps;
}

// ComputeInteractionsCPU (pnummerge.f90:483-562) counts the pairs i<k whose
// boxes overlap with strict bounds (<) on both axes; FindSingletonsCPU
// (:388-482) marks a box as a singleton unless another box meets it with
// closed bounds (<=).  Candidates come from an x1-sorted sweep.
void orc_interactions(const orc_box* Ab, int64_t n, int64_t* pairs, int64_t* singletons, uint8_t* is_singleton) {
  const Box* A = (const Box*)Ab;
  int64_t np = 0;
  std::vector<uint8_t> touched(n > 0 ? n : 0, 0);
  if (n > 0) {
    std::vector<int64_t> ord(n);
    for (int64_t i = 0; i < n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
      return A[a].x1 != A[b].x1 ? A[a].x1 < A[b].x1 : a < b;
    });
    for (int64_t s = 0; s < n; ++s) {
      const Box& bi = A[ord[s]];
      for (int64_t t = s + 1; t < n && A[ord[t]].x1 <= bi.x2; ++t) {
        const Box& bk = A[ord[t]];
        if (std::max(bi.y1, bk.y1) <= std::min(bi.y2, bk.y2)) {
          touched[ord[s]] = touched[ord[t]] = 1;
          if (std::max(bi.x1, bk.x1) < std::min(bi.x2, bk.x2) && std::max(bi.y1, bk.y1) < std::min(bi.y2, bk.y2))
            ++np;
        }
      }
    }
  }
  int64_t ns = 0;
  for (int64_t i = 0; i < n; ++i) {
    ns += touched[i] ? 0 : 1;
    if (is_singleton) is_singleton[i] = touched[i] ? 0 : 1;
  }
  if (pairs) *pairs = np;
  if (singletons) *singletons = ns;
}

// calculate_union_area_by_polygon (design.f90:854-935): boxes grouped by PNUM
// number; the singletons (number 0) add their own areas, every other group
// adds the union area of its boxes (calculate_union_area_fast).
int64_t orc_component_areas(const orc_box* A, int64_t n, int64_t* areas) {
  if (n <= 0) {
    if (areas) areas[0] = 0;
    return 0;
  }
  std::vector<int64_t> lab(n);
  orc_components(A, n, lab.data());
  int64_t R = 0;
  for (int64_t i = 0; i < n; ++i) R = std::max(R, lab[i]);
  if (!areas) return R;
  std::vector<std::vector<orc_box>> groups(R + 1);
  for (int64_t i = 0; i < n; ++i) groups[lab[i]].push_back(A[i]);
  areas[0] = 0;
  for (const orc_box& b : groups[0]) areas[0] += (int64_t)(b.x2 - b.x1) * (b.y2 - b.y1);
  for (int64_t k = 1; k <= R; ++k) areas[k] = orc_union_area(groups[k].data(), (int64_t)groups[k].size());
  return R;
}

// ComputeMorton (gpu_morton.cu:113-144): centre = ((int64)x1+x2)/2 truncated,
// sign bit flipped, bits spread, y in the odd and x in the even positions.
uint64_t orc_morton_key(const orc_box* b) {
  const uint32_t cx = (uint32_t)(((int64_t)b->x1 + b->x2) / 2) ^ 0x80000000u;
  const uint32_t cy = (uint32_t)(((int64_t)b->y1 + b->y2) / 2) ^ 0x80000000u;
  auto spread = [](uint64_t m) {
    m = (m | (m << 16)) & 0x0000FFFF0000FFFFULL;
    m = (m | (m << 8)) & 0x00FF00FF00FF00FFULL;
    m = (m | (m << 4)) & 0x0F0F0F0F0F0F0F0FULL;
    m = (m | (m << 2)) & 0x3333333333333333ULL;
    m = (m | (m << 1)) & 0x5555555555555555ULL;
    return m;
  };
  return (spread(cy) << 1) | spread(cx);
}

// PackKeys (event_sorter.cu:48-59).
uint64_t orc_tracker_key(int32_t X, int32_t Y) {
  return ((uint64_t)((uint32_t)X ^ 0x80000000u) << 32) | (uint64_t)((uint32_t)Y ^ 0x80000000u);
}

// int(1000.0_real64 * r) truncates toward zero (controlparser.f90:146,568-570).
int32_t orc_um_to_dbu(double r) { return (int32_t)(1000.0 * r); }

void orc_canonical_sort(orc_box* A, int64_t n) { std::sort((Box*)A, (Box*)A + n, cmp_box); }

// OP1 (op_template.m4:14-22) on one layer with amount a dbu; digests
// (optional, 7 entries): the strip digests of poly_1, poly_2, outer, inner,
// and1, inter and merged(P).
static void op1_impl(const orc_box* Ab, int64_t n, int32_t a, int g, int64_t* counts, int64_t* area,
                     uint64_t* digests) {
  const Box* P = (const Box*)Ab;
  std::vector<Box> p1, p2, outer, inner, and1, inter, merged;
  for (int k = 0; k < 8; ++k) counts[k] = -1;
  if (grow_impl(P, n, a, a, a, a, g, p1) < 0) return;
  if (size_impl(P, n, -a, g, p2) < 0) return;
  boolean_impl(p1.data(), (int64_t)p1.size(), P, n, ORC_NOT, g, outer);
  boolean_impl(P, n, p2.data(), (int64_t)p2.size(), ORC_NOT, g, inner);
  boolean_impl(outer.data(), (int64_t)outer.size(), P, n, ORC_AND, g, and1);
  boolean_impl(outer.data(), (int64_t)outer.size(), inner.data(), (int64_t)inner.size(), ORC_AND, g,
               inter);
  boolean_impl(P, n, nullptr, 0, ORC_MERGE, g, merged);
  counts[0] = (int64_t)p1.size(); counts[1] = (int64_t)p2.size();
  counts[2] = (int64_t)outer.size(); counts[3] = (int64_t)inner.size();
  counts[4] = (int64_t)and1.size(); counts[5] = (int64_t)inter.size();
  counts[6] = (int64_t)merged.size(); counts[7] = 0;
  int64_t s = 0;
  for (const Box& b : merged) s += (int64_t)(b.x2 - b.x1) * (int64_t)(b.y2 - b.y1);
  *area = s;
  if (digests) {
    const std::vector<Box>* L[7] = {&p1, &p2, &outer, &inner, &and1, &inter, &merged};
    for (int k = 0; k < 7; ++k) digests[k] = orc_strip_digest((const orc_box*)L[k]->data(), (int64_t)L[k]->size());
  }
}

void orc_op1(const orc_box* Ab, int64_t n, int32_t a, int g, int64_t* counts, int64_t* area) {
  op1_impl(Ab, n, a, g, counts, area, nullptr);
}

void orc_op1_digest(const orc_box* Ab, int64_t n, int32_t a, int g, int64_t* counts, int64_t* area,
                    uint64_t* digests) {
  op1_impl(Ab, n, a, g, counts, area, digests);
}

// OP1 on every cell of a batched layer, cells in parallel (OpenMP dynamic
// schedule; the per-cell operators run single-threaded inside).
void orc_op1_cells(const orc_box* Ab, const int64_t* off, int64_t ncell, int32_t a, int g,
                   int64_t* counts, int64_t* area) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ncell; ++k) {
    op1_impl(Ab + off[k], off[k + 1] - off[k], a, g, counts + 8 * k, area + k, nullptr);
  }
}

void orc_op1_cells_digest(const orc_box* Ab, const int64_t* off, int64_t ncell, int32_t a, int g,
                          int64_t* counts, int64_t* area, uint64_t* digests) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ncell; ++k) {
    op1_impl(Ab + off[k], off[k + 1] - off[k], a, g, counts + 8 * k, area + k, digests + 7 * k);
  }
}

// Order-independent digest of a strip list: the sum mod 2^64 of a 64-bit hash
// per strip, the MurmurHash3 fmix64 finaliser of the packed corners (the
// device computes the same function).
static inline uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

uint64_t orc_strip_hash(int32_t x1, int32_t y1, int32_t x2, int32_t y2) {
  const uint64_t u = ((uint64_t)(uint32_t)x1 << 32) | (uint32_t)y1;
  const uint64_t v = ((uint64_t)(uint32_t)x2 << 32) | (uint32_t)y2;
  return fmix64(u ^ fmix64(v + 0x9e3779b97f4a7c15ull));
}

uint64_t orc_strip_digest(const orc_box* A, int64_t n) {
  uint64_t h = 0;
  for (int64_t i = 0; i < n; ++i) h += orc_strip_hash(A[i].x1, A[i].y1, A[i].x2, A[i].y2);
  return h;
}

void orc_free(void* p) { std::free(p); }

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
