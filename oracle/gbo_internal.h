// gbo_internal.h -- C++ internals of the CPU oracle shared between its
// translation units (gbo_oracle.cpp, gbo_refpath.cpp).  TEST INFRASTRUCTURE
// ONLY, like the rest of oracle/.
#pragma once
#include <cstdint>
#include <vector>

namespace gbo {

struct Box { int32_t x1, y1, x2, y2; };
struct Piece { Box b; uint8_t owner; };

// The heal_boxes sweep (polygon_fracture.f90:805-1004) over one set of pieces,
// generalised to two owners and a Boolean predicate (op: ORC_*): appends the
// vertical strips of pred(A, B) to out.
void sweep_tile(const std::vector<Piece>& pcs, int op, std::vector<Box>& out);
// box_grow_directional on every box; false if a box is or becomes invalid.
bool grow_all(const Box* A, int64_t n, int32_t E, int32_t N, int32_t W, int32_t S, std::vector<Box>& g);
// SIZE(s) on the oracle's grid of 2^g tiles (canonical strips).
int64_t size_impl(const Box* A, int64_t n, int32_t s, int g, std::vector<Box>& res);

}  // namespace gbo
