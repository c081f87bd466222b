// gb_tile.cu -- the scanline Boolean kernel.
//
// Persistent CTAs (three per SM, 8 warps each) pull output tiles from a
// device work counter.
// For a tile it computes the canonical strips of pred(A, B) inside the tile:
// at every x the maximal y-intervals of the region, merged along x while
// unchanged -- the decomposition heal_boxes emits (polygon_fracture.f90:
// 805-1004), here for any Boolean predicate on the two coverages.
//
// Per tile:
//  A. Ranks.  The distinct x and y values of the tile's pieces are marked in
//     two 2^g+1-bit shared-memory bitmaps; prefix popcounts give every value
//     its rank.  x ranks number the x-slabs (elementary columns of the
//     sweep), y ranks the elementary y-intervals.
//  B. Sub-bands.  The x-slabs are grouped 63 at a time; sub-band s owns
//     slabs [63s, 63s+63) as rows 1..63 of a 64-bit word and sees slab 63s-1
//     as row 0.  Every piece is listed in each sub-band its slab range
//     touches (a counting sort in shared memory).
//  C. One warp per sub-band.  The y ranks of the sub-band's members are
//     compressed again (a bitmap over tile y ranks), and each member ORs its
//     row mask into one 64-bit word per local y column (separately for A and
//     B).  R = pred(A, B) word-wise gives the region for 64 slabs at once.
//     With V = R ^ (R << 1) (the rows where a column changes), a run of R
//     over columns [c1, c2] at row r is unchanged from row r-1 iff
//     V[c1-1 .. c2+1] has bit r clear; a segmented OR-scan along the columns
//     (a linear recurrence F_c = a_c | (b_c & F_{c-1}) evaluated with a warp
//     scan) delivers that OR at each run's last column for all 64 rows at
//     once.  A strip piece starts wherever the run changed; it ends at the
//     next change.  Pieces reaching row 63 are "open", pieces starting at
//     row 1 with no change from row 0 are "continuations".  The scan pass
//     leaves each column's local prefix of the recurrence, the count pass
//     each column's piece starts, so the passes after them do not evaluate
//     it again.  The pieces are dealt to the lanes 32 at a time in (column,
//     row) order, so a column with many pieces does not hold up the warp; a
//     piece's 16-byte record goes to the CTA's record region at its index.
//  D. Stitch.  The records come into shared memory in one bulk copy.  Each
//     continuation is linked to the open piece of the previous sub-band with
//     the same y-interval; every chain head becomes one strip.  The output
//     slots are reserved while the links are made.  Strips are written in
//     (sub-band, column, row) order, so the output of a tile is
//     deterministic.
// No CTA ever waits on another CTA.  The only waits are on the CTA's own
// mbarrier for the bulk copies of phases A and D; each is bounded (a poll
// limit, then GB_ERR_TIMEOUT and the CTA leaves after its copies land).
#include <cstdio>
#include <mutex>

#include "gb_internal.h"
#include "gb_scan.cuh"

#define TK_NW 8
#define TK_NT (TK_NW * 32)
#define TK_WMAX 2049
#define TK_NSBMAX 1042
#define TK_SBS 256
#define TK_MDS 128   // sub-bands whose metadata fits in the bitmap region after phase B
#define TK_MD_INTS (TK_MDS * 4 + (TK_MDS + 2) * 2 + TK_MDS * 2 * 2)  // sbinfo, sbh, sbct, sbol, sbrec
#define TK_LBW 128
#define TK_LVN 256
#define TK_LCN 128
#define TK_MC 128   // sub-band members kept in the per-warp member cache (8 bytes each)
#define TK_MLD 2    // member records loaded per lane before the first is used (per 1024-cell deck: 4 -> 2
                    // records 30.88 -> 30.59 ms)
#define TK_LD 2     // independent global loads in flight per thread in the streaming loops
#define TK_DIRECT 1 // columns of a member painted on its own lane; the rest are spread over the warp
                    // (measured per 1024-cell deck: 0 / 1 / 2 / 3 / 4 / 8 columns -> 35.16 / 34.78 /
                    // 34.91 / 34.85 / 35.02 / 38.13 ms)
#define KID_TILE 20

// A strip piece of one sub-band, 16 bytes, stored downward from the top of
// the CTA scratch.  x: y1 rank | cont << 30 | open << 31; y: y2 rank | low 15
// bits of the head rank << 17; z: first x-slab | high bits of the head rank
// << 17; w: end x-slab.  Ranks and slabs are below 2^17.
struct PieceRec {
  int x, y, z, w;
};
__device__ __forceinline__ int pr_ylo(const PieceRec& p) { return p.x & 0x1ffff; }
__device__ __forceinline__ int pr_yhi(const PieceRec& p) { return p.y & 0x1ffff; }
__device__ __forceinline__ int pr_slo(const PieceRec& p) { return p.z & 0x1ffff; }
__device__ __forceinline__ int pr_shi(const PieceRec& p) { return p.w; }
__device__ __forceinline__ bool pr_cont(const PieceRec& p) { return (p.x >> 30) & 1; }
__device__ __forceinline__ int pr_hrank(const PieceRec& p) {
  return (int)(((unsigned)p.y >> 17) | (((unsigned)p.z >> 17) << 15));
}

// A tile to process: its index, cell and the two operands' pieces.
struct TileRef {
  long long tile;
  const unsigned long long* pa;
  const unsigned long long* pb;
  int nA, nB, cell, pad;
};

struct TileSmem {
  union {  // phases A-B: value bitmaps and their prefix popcounts; phase D: x / y value tables
    struct {
      unsigned xb[TK_WMAX], yb[TK_WMAX];
      unsigned xp[TK_WMAX / 2 + 1], yp[TK_WMAX / 2 + 1];  // prefix popcount per 2 words
    };
    int xyv[2 * TK_WMAX + 2 * (TK_WMAX / 2 + 1)];  // phase D; after the metadata below when it is here
  };
  int sbc_s[TK_SBS + 2];  // per sub-band member counts / cursors (scratch when more sub-bands)
  union {  // phase C: per-warp sweep buffers; phase D: piece records and chain links
    struct {
      unsigned lb[TK_NW][TK_LBW];
      unsigned lp[TK_NW][TK_LBW];
      int lv[TK_NW][TK_LVN];
      unsigned long long ca[TK_NW][TK_LCN];
      unsigned long long cb[TK_NW][TK_LCN];
      // member cache: first row | end row << 7 | owner << 14 | y1 rank << 15, y2 rank << 32 (rows 0..64,
      // ranks below 2^17)
      unsigned long long mc[TK_NW][TK_MC];
      unsigned srow[TK_NW][64][TK_LCN / 32];  // run starts, row-major (transposed)
    };
    unsigned char dbuf[1];
    int4 dbuf_align;  // the region starts on 16 bytes: bulk copies and int4 records land in it
  };
  int sbnext;                            // next sub-band to hand to a warp
  unsigned long long mbar;               // completion of phase D's bulk copies (one phase per tile)
  long long tmp64[33];
  long long tile;
  const unsigned long long* pa;
  const unsigned long long* pb;
  int nA, nB, cell, err;
  int rsplit;  // some sub-band's piece records did not fit the record region (allocated below instead)
  TileRef nx;   // the next tile, reserved and looked up during this tile's phase D
  int have_nx;
  long long obase;
  DStatus* st;
  // up: bytes allocated from the lower half of the scratch; down: strip pieces so far, whose records sit at
  // their piece index in the upper half (the record region)
  unsigned long long up, down;
  int* Xt;
  int* Yt;
  int4* rk;
  int4* mem;  // member records: x1-slab | owner<<31, x2-slab, y1 rank, y2 rank
  int4* sbinfo;  // per sub-band: piece base, piece count, open-list byte offset, open count
  int* sbh;      // heads per sub-band, then their exclusive scan
  int* sbct;     // continuation pieces per sub-band
  int* sbc;      // per sub-band member counts / cursors (sbc_s or scratch)
  int** sbol;    // open list (then continuation list) per sub-band
  PieceRec** sbrec;  // strip pieces per sub-band (global piece index = sbinfo.x + local index)
  unsigned* biglb;
  int* succ;
};
#include <cstddef>
// Bulk asynchronous copies need 16-byte aligned shared-memory addresses, and
// the staged ranks, piece records and sub-band metadata are read as int4.
static_assert(offsetof(TileSmem, dbuf) % 16 == 0, "phase C/D region must start on 16 bytes");
static_assert(offsetof(TileSmem, xyv) % 16 == 0, "value-table region must start on 16 bytes");
static_assert(offsetof(TileSmem, ca) % 16 == 0 && offsetof(TileSmem, srow) % 16 == 0, "per-warp arrays");
static_assert((TK_MD_INTS * 4) % 16 == 0, "value tables after the metadata start on 16 bytes");


__device__ __forceinline__ unsigned long long gb_pred(int op, unsigned long long a, unsigned long long b) {
  switch (op) {
    case GB_OP_XOR: return a ^ b;
    case GB_OP_AND: return a & b;
    case GB_OP_NOT: return a & ~b;
    case GB_OP_OVERLAP: return b;  // b holds the rows covered a second time
    default: return a | b;  // OR, MERGE (B empty)
  }
}

// Single-layer AND: a row bit painted into a column that already had it is
// recorded in the second word array (atomics make the order of two paints of
// the same cell irrelevant), so b ends as the cells covered at least twice.
__device__ __forceinline__ void paint_twice(unsigned* a, unsigned* b, int c, unsigned mlo, unsigned mhi) {
  if (mlo) {
    const unsigned o = atomicOr(&a[2 * c], mlo) & mlo;
    if (o) atomicOr(&b[2 * c], o);
  }
  if (mhi) {
    const unsigned o = atomicOr(&a[2 * c + 1], mhi) & mhi;
    if (o) atomicOr(&b[2 * c + 1], o);
  }
}

__device__ __forceinline__ int bm_rank(const unsigned* bits, const unsigned* pref, int v) {
  const int w = v >> 5;
  return (int)pref[w] + __popc(bits[w] & ((1u << (v & 31)) - 1u));
}
// rank with a prefix stored once per 2 words
__device__ __forceinline__ int bm_rank2(const unsigned* bits, const unsigned* pref2, int v) {
  const int w = v >> 5;
  int r = (int)pref2[w >> 1] + ((w & 1) ? __popc(bits[w - 1]) : 0);
  return r + __popc(bits[w] & ((1u << (v & 31)) - 1u));
}

__device__ __forceinline__ unsigned long long vchg(unsigned long long r) { return (r ^ (r << 1)) & ~1ull; }

// ---- bulk copies of phase D (global scratch -> shared memory, completing on an mbarrier)
#define TK_SPIN_LIMIT (1 << 22)
#define KID_TILE_COPY 22
__device__ __forceinline__ unsigned tk_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void tk_bulk(void* dst, const void* src, unsigned bytes, unsigned mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tk_smem(dst)),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
// bounded wait for the given phase parity; false after `limit` polls
__device__ __forceinline__ bool tk_wait(unsigned mbar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Allocation in the lower half of the CTA's scratch (one thread calls it).
// When a dense tile outgrows it, the allocation spills into the work arena
// (released with the operation); only an exhausted arena is an error.
__device__ __forceinline__ void* sc_up(TileSmem& s, char* base, unsigned long long half,
                                       unsigned long long bytes) {
  const unsigned long long off = atomicAdd(&s.up, (bytes + 15ull) & ~15ull);
  if (off + bytes > half) {
    void* p = s.st ? gb_arena_alloc_atomic(s.st, bytes, KID_TILE) : nullptr;
    if (!p) s.err = 1;
    return p;
  }
  return base + off;
}


// Output tile t: its cell, and where A's and B's pieces of that tile start.  A Boolean result carries a
// descriptor per tile (one load); other callers' layers are looked up through the cell windows.
__device__ __forceinline__ void tile_lookup(int op, const DLayer* A, const DLayer* B, const DLayer* O, long long t,
                                            TileRef& r) {
  r.tile = t;
  r.nA = r.nB = 0;
  r.pa = r.pb = nullptr;
  r.cell = 0;
  if (t >= O->ntiles) return;
  if (O->tdesc) {
    const TileDesc d = O->tdesc[t];
    r.cell = d.cell;
    r.nA = d.nA;
    r.nB = d.nB;
    if (d.nA) r.pa = A->pcs + d.offA;
    if (d.nB) r.pb = B->pcs + d.offB;
    return;
  }
  const int k = gb_find_cell(O->tbase, O->ncell, t);
  const int4 w = O->win[k];
  const long long li = t - O->tbase[k];
  const int tx = w.x + (int)(li % w.z), ty = w.y + (int)(li / w.z);
  r.cell = k;
  const int4 wa = A->win[k];
  if (tx >= wa.x && ty >= wa.y && tx < wa.x + wa.z && ty < wa.y + wa.w) {
    const long long ta = A->tbase[k] + (long long)(ty - wa.y) * wa.z + (tx - wa.x);
    r.nA = A->tcount[ta];
    r.pa = A->pcs + A->tstart[ta];
  }
  if (B && op != GB_OP_MERGE && op != GB_OP_OVERLAP) {
    const int4 wb = B->win[k];
    if (tx >= wb.x && ty >= wb.y && tx < wb.x + wb.z && ty < wb.y + wb.w) {
      const long long tb = B->tbase[k] + (long long)(ty - wb.y) * wb.z + (tx - wb.x);
      r.nB = B->tcount[tb];
      r.pb = B->pcs + B->tstart[tb];
    }
  }
}

// TIMING: the phase counters of gb_tile_timing are compiled in (tctr non-null
// then); the production instance has none of that code.
template <bool TIMING>
__device__ void tile_subband(TileSmem& s, int op, int sb, int nsb, int Ny, int nA, char* base,
                             unsigned long long scr, long long* tctr) {
  if (!TIMING) tctr = nullptr;
  const int lane = gb_lane(), wid = gb_warp();
  long long q0 = tctr ? clock64() : 0;
  const long long qstart = q0;
#define TSTEP(k)                                                           \
  if (tctr && lane == 0) {                                                 \
    const long long q1 = clock64();                                        \
    atomicAdd((unsigned long long*)&tctr[k], (unsigned long long)(q1 - q0)); \
    q0 = q1;                                                               \
  }
  const unsigned long long half = scr >> 1;
  const int beg = sb ? s.sbc[sb - 1] : 0, end = s.sbc[sb];
  const int m = end - beg;
  if (m == 0) {
    if (lane == 0) {
      s.sbinfo[sb] = make_int4(0, 0, 0, 0);
      s.sbh[sb] = 0;
      s.sbct[sb] = 0;
      s.sbol[sb] = nullptr;
      s.sbrec[sb] = nullptr;
    }
    return;
  }
  const int rowbase = 63 * sb - 1;
  const int nwy = ((Ny - 1) >> 5) + 1;
  unsigned* lb = nwy <= TK_LBW ? s.lb[wid] : s.biglb + (size_t)wid * 2 * nwy;
  unsigned* lp = nwy <= TK_LBW ? s.lp[wid] : lb + nwy;
  const bool cache = m <= TK_MC;
  for (int w = lane; w < nwy; w += 32) lb[w] = 0;
  __syncwarp();
  for (int j0 = 0; j0 < m; j0 += 32 * TK_MLD) {
    int4 rr[TK_MLD];
#pragma unroll
    for (int u = 0; u < TK_MLD; ++u) {
      const int j = j0 + u * 32 + lane;
      rr[u] = j < m ? s.mem[beg + j] : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < TK_MLD; ++u) {
      const int j = j0 + u * 32 + lane;
      if (j < m) {
        const int4 r = rr[u];
        if (cache) {
          const unsigned lo = (unsigned)max((r.x & 0x7fffffff) - rowbase, 0), hi = (unsigned)min(r.y - rowbase, 64);
          s.mc[wid][j] = (unsigned long long)(lo | (hi << 7) | (((unsigned)r.x >> 31) << 14) | ((unsigned)r.z << 15)) |
                         ((unsigned long long)(unsigned)r.w << 32);
        }
        atomicOr(&lb[r.z >> 5], 1u << (r.z & 31));
        atomicOr(&lb[r.w >> 5], 1u << (r.w & 31));
      }
    }
  }
  __syncwarp();
  int nl;
  {
    const int per = (nwy + 31) >> 5, w0 = lane * per, w1 = min(nwy, w0 + per);
    int cnt = 0;
    for (int w = w0; w < w1; ++w) cnt += __popc(lb[w]);
    int tot;
    int ex = gb_warp_excl(cnt, &tot);
    for (int w = w0; w < w1; ++w) { lp[w] = ex; ex += __popc(lb[w]); }
    nl = tot;
  }
  const int L = nl - 1;
  TSTEP(0)
  if (tctr && lane == 0) {
    atomicAdd((unsigned long long*)&tctr[6], (unsigned long long)m);
    atomicAdd((unsigned long long*)&tctr[7], (unsigned long long)L);
  }
  int* lv = s.lv[wid];
  unsigned long long* ca = s.ca[wid];
  unsigned long long* cb = s.cb[wid];
  if (nl > TK_LVN || L > TK_LCN) {
    unsigned long long pv = 0, pc = 0;
    if (lane == 0) {
      if (nl > TK_LVN) pv = (unsigned long long)sc_up(s, base, half, (unsigned long long)nl * 4);
      if (L > TK_LCN) pc = (unsigned long long)sc_up(s, base, half, (unsigned long long)L * 16);
    }
    pv = __shfl_sync(0xffffffffu, pv, 0);
    pc = __shfl_sync(0xffffffffu, pc, 0);
    if ((nl > TK_LVN && !pv) || (L > TK_LCN && !pc)) return;  // s.err is set
    if (pv) lv = (int*)pv;
    if (pc) { ca = (unsigned long long*)pc; cb = ca + L; }
  }
  {
    const int per = (nwy + 31) >> 5, w0 = lane * per, w1 = min(nwy, w0 + per);
    for (int w = w0; w < w1; ++w) {
      unsigned bits = lb[w];
      int k = lp[w];
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        lv[k++] = (w << 5) + b;
      }
    }
  }
  // ---- rasterise: one member per lane; each column word is updated as two
  // 32-bit halves with native shared-memory atomicOr
  const int per = (L + 31) >> 5, c0 = min(L, lane * per), c1e = min(L, c0 + per);
  for (int c = c0; c < c1e; ++c) { ca[c] = 0; cb[c] = 0; }
  __syncwarp();
  // 32 members at a time: the (member, column) pairs of the group are spread
  // evenly over the lanes (a warp scan of the spans, then a shuffle search for
  // the member of each pair), so one long member does not serialise a lane.
  long long qa = tctr ? clock64() : 0, qsetup = 0, qpaint = 0;
  for (int jb = 0; jb < m; jb += 32) {
    const int j = jb + lane;
    int lc1 = 0, span = 0, own = 0;
    unsigned long long mk = 0;
    if (j < m) {
      int lo, hi, yz, yw;
      if (cache) {
        const unsigned long long e = s.mc[wid][j];
        const unsigned e0 = (unsigned)e;
        lo = (int)(e0 & 127u);
        hi = (int)((e0 >> 7) & 127u);
        own = (int)((e0 >> 14) & 1u);
        yz = (int)(e0 >> 15);
        yw = (int)(e >> 32);
      } else {
        const int4 r = s.mem[beg + j];
        own = (r.x >> 31) & 1;
        lo = max((r.x & 0x7fffffff) - rowbase, 0);
        hi = min(r.y - rowbase, 64);
        yz = r.z;
        yw = r.w;
      }
      mk = (hi >= 64 ? ~0ull : ((1ull << hi) - 1ull)) & (~0ull << lo);
      lc1 = bm_rank(lb, lp, yz);
      span = bm_rank(lb, lp, yw) - lc1;
    }
    // direct: the first TK_DIRECT columns of every member on its own lane
    {
      unsigned* col = (unsigned*)(own ? cb : ca);
      const unsigned mlo = (unsigned)mk, mhi = (unsigned)(mk >> 32);
      const int d = min(span, TK_DIRECT);
      if (op == GB_OP_OVERLAP) {
        for (int c = lc1; c < lc1 + d; ++c) paint_twice((unsigned*)ca, (unsigned*)cb, c, mlo, mhi);
      } else {
        for (int c = lc1; c < lc1 + d; ++c) {
          if (mlo) atomicOr(&col[2 * c], mlo);
          if (mhi) atomicOr(&col[2 * c + 1], mhi);
        }
      }
    }
    if (tctr) { const long long qb = clock64(); qsetup += qb - qa; qa = qb; }
    // remainder of long members: (member, column) pairs spread over the lanes
    const int rest = max(span - TK_DIRECT, 0);
    if (__any_sync(0xffffffffu, rest > 0)) {
      const int incl = gb_warp_incl(rest);
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      if (tctr && lane == 0) atomicAdd((unsigned long long*)&tctr[12], (unsigned long long)total);
      for (int k0 = 0; k0 < total; k0 += 32) {  // warp-uniform trip count
        const int k = k0 + lane;
        int o = 0;  // owner lane: the first lane whose inclusive prefix exceeds k
#pragma unroll
        for (int st2 = 16; st2 > 0; st2 >>= 1) {
          const int v = __shfl_sync(0xffffffffu, incl, o + st2 - 1);
          if (v <= k) o += st2;
        }
        const int ex_o = __shfl_sync(0xffffffffu, incl - rest, o);
        const int c1_o = __shfl_sync(0xffffffffu, lc1, o);
        const int own_o = __shfl_sync(0xffffffffu, own, o);
        const unsigned long long mk_o = __shfl_sync(0xffffffffu, mk, o);
        if (k < total) {
          unsigned* col = (unsigned*)(own_o ? cb : ca);
          const int c = c1_o + TK_DIRECT + (k - ex_o);
          if (op == GB_OP_OVERLAP) {
            paint_twice((unsigned*)ca, (unsigned*)cb, c, (unsigned)mk_o, (unsigned)(mk_o >> 32));
          } else {
            if ((unsigned)mk_o) atomicOr(&col[2 * c], (unsigned)mk_o);
            if ((unsigned)(mk_o >> 32)) atomicOr(&col[2 * c + 1], (unsigned)(mk_o >> 32));
          }
        }
      }
    }
    if (tctr) { const long long qb = clock64(); qpaint += qb - qa; qa = qb; }
  }
  __syncwarp();
  if (tctr && lane == 0) {
    atomicAdd((unsigned long long*)&tctr[8], (unsigned long long)qsetup);
    atomicAdd((unsigned long long*)&tctr[9], (unsigned long long)qpaint);
  }
  unsigned long long rany = 0;
  for (int c = c0; c < c1e; ++c) {
    const unsigned long long r = gb_pred(op, ca[c], cb[c]);
    ca[c] = r;
    rany |= r;
  }
  // No region in rows 1..63: the sub-band has no strip pieces (row 0 belongs to
  // the previous sub-band, and its runs matter only to continuations here).
  if (!__any_sync(0xffffffffu, (rany & ~1ull) != 0ull)) {
    TSTEP(1)
    if (lane == 0) {
      s.sbinfo[sb] = make_int4(0, 0, 0, 0);
      s.sbh[sb] = 0;
      s.sbct[sb] = 0;
      s.sbol[sb] = nullptr;
      s.sbrec[sb] = nullptr;
    }
    __syncwarp();
    return;
  }
  __syncwarp();
  TSTEP(1)
  // ---- run starts S_c = R_c & ~R_{c-1}, transposed to one column bitmap per row
  const bool tr = L <= TK_LCN;
  if (tr) {
    const int nb = (L + 31) >> 5;
    for (int b = 0; b < nb; ++b) {
      const int c = (b << 5) + lane;
      const unsigned long long Rc = c < L ? ca[c] : 0ull;
      const unsigned long long Rm = (c >= 1 && c - 1 < L) ? ca[c - 1] : 0ull;
      const unsigned long long S = Rc & ~Rm;
      unsigned lo = (unsigned)S, hi = (unsigned)(S >> 32);
#pragma unroll
      for (int j = 16; j > 0; j >>= 1) {
        const unsigned m0 = j == 16 ? 0x0000FFFFu : j == 8 ? 0x00FF00FFu : j == 4 ? 0x0F0F0F0Fu
                          : j == 2 ? 0x33333333u : 0x55555555u;
        const unsigned tlo = __shfl_xor_sync(0xffffffffu, lo, j);
        const unsigned thi = __shfl_xor_sync(0xffffffffu, hi, j);
        if (lane & j) {
          lo = ((tlo & ~m0) >> j) | (lo & ~m0);
          hi = ((thi & ~m0) >> j) | (hi & ~m0);
        } else {
          lo = (lo & m0) | ((tlo & m0) << j);
          hi = (hi & m0) | ((thi & m0) << j);
        }
      }
      s.srow[wid][lane][b] = lo;
      s.srow[wid][32 + lane][b] = hi;
    }
    __syncwarp();
  }
  TSTEP(5)

  // ---- forward segmented OR-scan over the columns (bit-parallel over rows)
  auto R = [&](int c) -> unsigned long long { return (c < 0 || c >= L) ? 0ull : ca[c]; };
  unsigned long long FA = 0ull, FB = ~0ull;
  {
    unsigned long long Rm1 = R(c0 - 1);
    for (int c = c0; c < c1e; ++c) {
      const unsigned long long Rc = ca[c];
      const unsigned long long Sc = Rc & ~Rm1;
      const unsigned long long a = Rc & (vchg(Rc) | (Sc & vchg(Rm1)));
      const unsigned long long b = Rc & Rm1;
      FA = a | (b & FA);
      FB = b & FB;
      cb[c] = FA;  // local prefix: F_c = FA_c | (FB_c & carry-in)
      Rm1 = Rc;
    }
  }
  unsigned long long IA = FA, IB = FB;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long pA = __shfl_up_sync(0xffffffffu, IA, o);
    const unsigned long long pB = __shfl_up_sync(0xffffffffu, IB, o);
    if (lane >= o) { IA = IA | (IB & pA); IB = IB & pB; }
  }
  unsigned long long Fin = __shfl_up_sync(0xffffffffu, IA, 1);
  if (lane == 0) Fin = 0ull;
  const bool last_sb = (sb == nsb - 1);
  TSTEP(2)

  // ---- count pieces / opens / heads
  int np = 0, no = 0, nh = 0, ncn = 0, nz = 0;
  {
    unsigned long long Rm1 = R(c0 - 1), fb = ~0ull;
    for (int c = c0; c < c1e; ++c) {
      const unsigned long long Rc = ca[c], Rp1 = R(c + 1);
      const unsigned long long Ec = Rc & ~Rp1;
      fb &= Rc & Rm1;
      const unsigned long long F = cb[c] | (fb & Fin);
      const unsigned long long Chg = (F | vchg(Rp1)) & Ec;
      const unsigned long long Z = (Chg | 2ull) & Ec & ~1ull;
      cb[c] = Z | ((Chg >> 1) & 1ull);  // bit 0 of Z is always clear
      const int pc = __popcll(Z);
      np += pc;
      if (!last_sb && (Ec >> 63)) ++no;
      const int cont = (sb > 0) && ((Z >> 1) & 1ull) && !((Chg >> 1) & 1ull);
      nh += pc - cont;
      ncn += cont;
      nz += (int)(Ec & 1ull);
      Rm1 = Rc;
    }
  }
  int totP, totO, totH, totC, totZ;
  // runs at row 0 are the runs at row 63 of the previous sub-band, both in y
  // order: a continuation's ordinal among them indexes that sub-band's open list
  int posZ, posP, posO, posH, posC;
  // one 64-bit scan when the fields cannot overflow: pieces and heads (at most 64 x 512 each) in 16 bits,
  // opens, continuations and row-0 ends (at most 512 each) in 10 bits
  if (L <= 512) {
    const unsigned long long v = (unsigned long long)np | ((unsigned long long)nh << 16) |
                                 ((unsigned long long)no << 32) | ((unsigned long long)ncn << 42) |
                                 ((unsigned long long)nz << 52);
    unsigned long long t;
    const unsigned long long e = gb_warp_excl(v, &t);
    posP = (int)(e & 0xffffu);
    posH = (int)((e >> 16) & 0xffffu);
    posO = (int)((e >> 32) & 0x3ffu);
    posC = (int)((e >> 42) & 0x3ffu);
    posZ = (int)((e >> 52) & 0x3ffu);
    totP = (int)(t & 0xffffu);
    totH = (int)((t >> 16) & 0xffffu);
    totO = (int)((t >> 32) & 0x3ffu);
    totC = (int)((t >> 42) & 0x3ffu);
    totZ = (int)((t >> 52) & 0x3ffu);
  } else {
    posZ = gb_warp_excl(nz, &totZ);
    posP = gb_warp_excl(np, &totP);
    posO = gb_warp_excl(no, &totO);
    posH = gb_warp_excl(nh, &totH);
    posC = gb_warp_excl(ncn, &totC);
  }
  int pbase = 0;
  unsigned long long obase = 0, rbase = 0;
  if (lane == 0) {
    pbase = (int)atomicAdd(&s.down, (unsigned long long)totP);
    if (totP > 0) {
      // the record region is the upper half of the scratch, indexed by piece
      const unsigned long long rh = half & ~15ull;
      void* p;
      if ((unsigned long long)(pbase + totP) * sizeof(PieceRec) <= scr - rh) {
        p = base + rh + (size_t)pbase * sizeof(PieceRec);
      } else {
        p = sc_up(s, base, half, (unsigned long long)totP * sizeof(PieceRec));
        s.rsplit = 1;
      }
      rbase = (unsigned long long)p;
      if (!p) pbase = -1;
    }
    if (totO + totC > 0 && pbase >= 0) {
      void* p = sc_up(s, base, half, (unsigned long long)(totO + totC) * 4);
      obase = (unsigned long long)p;
      if (!p) pbase = -1;
    }
  }
  pbase = __shfl_sync(0xffffffffu, pbase, 0);
  obase = __shfl_sync(0xffffffffu, obase, 0);
  rbase = __shfl_sync(0xffffffffu, rbase, 0);
  if (pbase < 0) return;
  PieceRec* recs = (PieceRec*)rbase;
  int* olist = (int*)obase;  // open pieces, then continuation pieces, each in y order
  TSTEP(3)

  // ---- write pieces, dealt to the lanes 32 at a time in (column, row) order: piece k's lane is found by a
  // shuffle search over the lanes' piece counts, its column by a walk over that lane's columns, its row as
  // its rank among the column's piece starts
  {
    const int inclP = posP + np;
    for (int k0 = 0; k0 < totP; k0 += 32) {  // warp-uniform trip count
      const int k = k0 + lane;
      int ow = 0;  // owner lane: the first lane whose inclusive piece prefix exceeds k
#pragma unroll
      for (int st2 = 16; st2 > 0; st2 >>= 1) {
        const int v = __shfl_sync(0xffffffffu, inclP, ow + st2 - 1);
        if (v <= k) ow += st2;
      }
      const int oP = __shfl_sync(0xffffffffu, posP, ow), oO = __shfl_sync(0xffffffffu, posO, ow);
      const int oH = __shfl_sync(0xffffffffu, posH, ow), oC = __shfl_sync(0xffffffffu, posC, ow);
      const int oZ = __shfl_sync(0xffffffffu, posZ, ow);
      if (k < totP) {
        int j = k - oP, o = oO, h = oH, q = oC, z = oZ;
        int c = min(L, ow * per);
        unsigned long long zs, Z, Ec;
        int contc;
        for (;;) {  // the owner's columns before the piece's own: their pieces, opens, continuations, row-0 ends
          zs = cb[c];
          Z = zs & ~1ull;
          Ec = ca[c] & ~R(c + 1);
          contc = (sb > 0) && ((Z >> 1) & 1ull) && !(zs & 1ull);
          const int pc = __popcll(Z);
          if (j < pc) break;
          j -= pc;
          h += pc - contc;
          q += contc;
          o += (!last_sb && (Ec >> 63)) ? 1 : 0;
          z += (int)(Ec & 1ull);
          ++c;
        }
        unsigned long long Zr = Z;
        for (int i = 0; i < j; ++i) Zr &= Zr - 1;
        const int r = __ffsll((long long)Zr) - 1;
        h += j - ((contc && r > 1) ? 1 : 0);  // the column's continuation (row 1) is not a head
        const unsigned long long above = (r >= 63) ? 0ull : ((Z | ~Ec) & (~0ull << (r + 1)));
        const int rend = above ? (__ffsll((long long)above) - 1) : 64;
        int cs = c;
        if (tr) {
          int b = c >> 5;
          unsigned mk = s.srow[wid][r][b] & (0xFFFFFFFFu >> (31 - (c & 31)));
          while (!mk && b > 0) mk = s.srow[wid][r][--b];
          cs = (b << 5) + 31 - __clz(mk);
        } else {
          while (cs > 0) {
            const unsigned long long S2 = ca[cs] & ~ca[cs - 1];
            if ((S2 >> r) & 1ull) break;
            --cs;
          }
        }
        const int cont = (r == 1) && contc;
        const int open = (rend == 64) && !last_sb;
        const int p = pbase + k;
        PieceRec pr;
        const unsigned hr = cont ? (unsigned)z : (unsigned)h;  // continuations keep their row-0 ordinal
        pr.x = lv[cs] | (cont << 30) | (open << 31);
        pr.y = lv[c + 1] | (int)((hr & 0x7fffu) << 17);
        pr.z = (rowbase + r) | (int)((hr >> 15) << 17);
        pr.w = rowbase + rend;
        recs[k] = pr;
        if (open) olist[o] = p;
        if (cont) olist[totO + q] = p;
      }
    }
  }
  TSTEP(4)
  if (tctr && lane == 0) {  // sub-bands whose column words spilled to scratch: count and cycles
    const long long q1 = clock64();
    atomicAdd((unsigned long long*)&tctr[28 + (L > TK_LCN ? 0 : 2)], 1ull);
    atomicAdd((unsigned long long*)&tctr[29 + (L > TK_LCN ? 0 : 2)], (unsigned long long)(q1 - qstart));
  }
  if (lane == 0) {
    s.sbinfo[sb] = make_int4(pbase, totP, totO, 0);
    s.sbol[sb] = (int*)obase;
    s.sbrec[sb] = recs;
    s.sbh[sb] = totH;
    s.sbct[sb] = totC;
  }
#undef TSTEP
}

template <bool TIMING>
__global__ void __launch_bounds__(TK_NT, 3)
k_tile(int op, const DLayer* A, const DLayer* B, DLayer* O, int g, int mode, char* scratch,
       unsigned long long scr, long long* counter, DStatus* st) {
  extern __shared__ __align__(16) unsigned char smraw[];
  TileSmem& s = *reinterpret_cast<TileSmem*>(smraw);
  const int tid = threadIdx.x;
  char* base = scratch + (size_t)blockIdx.x * scr;
  const unsigned long long half = scr >> 1;
  const int W = ((1 << g) >> 5) + 1;
  const bool timing = TIMING && (mode & 4) != 0;
  mode &= 3;
  long long tA = 0, tB = 0, tC = 0, tD = 0, t0 = 0;
  const unsigned mbar = tk_smem(&s.mbar);
  unsigned mph = 0;  // parity of the mbarrier phase the next bulk copies complete
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s.have_nx = 0;
  }
  for (;;) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // before this tile's bulk copies
    __syncthreads();
    if (tid == 0) {
      s.st = st;
      TileRef r;
      if (s.have_nx) r = s.nx;
      else tile_lookup(op, A, B, O, st->err ? (1ll << 62) : (long long)atomicAdd((unsigned long long*)counter, 1ull), r);
      s.have_nx = 0;
      if (st->err) r.tile = 1ll << 62;  // an error stops the CTA, a reserved tile too
      s.tile = r.tile;
      s.nA = r.nA;
      s.nB = r.nB;
      s.pa = r.pa;
      s.pb = r.pb;
      s.cell = r.cell;
      s.up = 0;
      s.down = 0;
      s.err = 0;
      s.rsplit = 0;
    }
    __syncthreads();
    const long long t = s.tile;
    if (t >= O->ntiles) break;
    const int nA = s.nA, nB = s.nB, P = nA + nB;
    if (P == 0) {
      if (tid == 0) { O->tcount[t] = 0; O->tstart[t] = 0; }
      continue;
    }
    if (timing) t0 = clock64();
    // ---- A: tile ranks
    // Pieces of a tile with at most ~2000 pieces are staged in the (still unused) phase C/D region by
    // bulk copies, their ranks kept next to them; each operand starts at the source's offset modulo 16
    // bytes so both ends of the copy are 16-byte aligned, a leading / trailing odd piece is loaded plainly.
    constexpr int DB = (int)(sizeof(s.lb) + sizeof(s.lp) + sizeof(s.lv) + sizeof(s.ca) + sizeof(s.cb) +
                             sizeof(s.mc) + sizeof(s.srow));
    const unsigned long long* pa = s.pa;
    const unsigned long long* pb = s.pb;
    // A pieces at sp + offA, B pieces at sp + offB: offsets of the parity of the source addresses' 8-byte
    // index, so a piece and its copy agree modulo 16 bytes
    const int offA = nA ? (int)(((uintptr_t)pa >> 3) & 1) : 0;
    const int pbit = nB ? (int)(((uintptr_t)pb >> 3) & 1) : 0;
    const int offB = offA + nA + (((offA + nA) & 1) != pbit ? 1 : 0);
    const int rkoff = ((offB + nB) * 8 + 15) & ~15;  // bytes
    const bool pst = rkoff + P * 16 <= DB;
    unsigned long long* sp = reinterpret_cast<unsigned long long*>(s.dbuf);
    int4* srk = reinterpret_cast<int4*>(s.dbuf + rkoff);
    if (pst) {
      // bulk parts [a0, a1) of A and [b0, b1) of B: even counts of pieces starting on 16-byte addresses
      const int a0 = offA & 1, a1 = nA > a0 ? a0 + ((nA - a0) & ~1) : a0;
      const int b0 = pbit, b1 = nB > b0 ? b0 + ((nB - b0) & ~1) : b0;
      if (tid == 0) {
        const unsigned bytes = (unsigned)(a1 - a0 + b1 - b0) * 8u;
        asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(mbar),
                     "r"(bytes)
                     : "memory");
        if (a1 > a0) tk_bulk(sp + offA + a0, pa + a0, (unsigned)(a1 - a0) * 8u, mbar);
        if (b1 > b0) tk_bulk(sp + offB + b0, pb + b0, (unsigned)(b1 - b0) * 8u, mbar);
      }
      // the first / last piece of an operand when it lies outside the bulk part
      if (tid < 4) {
        const int i = (tid & 1) ? ((tid < 2 ? nA : nB) - 1) : 0;
        if (tid < 2 && nA && (i < a0 || i >= a1)) sp[offA + i] = pa[i];
        if (tid >= 2 && nB && (i < b0 || i >= b1)) sp[offB + i] = pb[i];
      }
    }
    for (int w = tid; w < W; w += TK_NT) { s.xb[w] = 0; s.yb[w] = 0; }
    if (pst) {
      const bool ok = tk_wait(mbar, mph, TK_SPIN_LIMIT);
      mph ^= 1u;
      if (__syncthreads_or(!ok)) {
        if (tid == 0) gb_set_error(st, GB_ERR_TIMEOUT, KID_TILE_COPY, t);
        tk_wait(mbar, mph ^ 1u, TK_SPIN_LIMIT);  // let copies in flight land before the CTA exits
        return;
      }
      pa = sp + offA;
      pb = sp + offB;
    } else {
      __syncthreads();
    }
    // pieces are read TK_LD at a time per thread, so their loads overlap
    for (int i0 = tid; i0 < P; i0 += TK_LD * TK_NT) {
      unsigned long long pk[TK_LD];
#pragma unroll
      for (int u = 0; u < TK_LD; ++u) {
        const int i = i0 + u * TK_NT;
        pk[u] = i < P ? (i < nA ? pa[i] : pb[i - nA]) : 0ull;
      }
#pragma unroll
      for (int u = 0; u < TK_LD; ++u) {
        if (i0 + u * TK_NT < P) {
          int x1, y1, x2, y2;
          gb_unpack(pk[u], x1, y1, x2, y2);
          atomicOr(&s.xb[x1 >> 5], 1u << (x1 & 31));
          atomicOr(&s.xb[x2 >> 5], 1u << (x2 & 31));
          atomicOr(&s.yb[y1 >> 5], 1u << (y1 & 31));
          atomicOr(&s.yb[y2 >> 5], 1u << (y2 & 31));
        }
      }
    }
    __syncthreads();
    int Nx, Ny;
    {
      const int per = ((W + TK_NT - 1) / TK_NT) | 1, w0 = min(W, tid * per), w1 = min(W, w0 + per);
      long long cx = 0, cy = 0;
      for (int w = w0; w < w1; ++w) { cx += __popc(s.xb[w]); cy += __popc(s.yb[w]); }
      long long tot;
      const long long ex = gb_block_excl(cx | (cy << 32), s.tmp64, &tot);
      unsigned ox = (unsigned)(ex & 0xffffffffll), oy = (unsigned)(ex >> 32);
      for (int w = w0; w < w1; ++w) {
        if ((w & 1) == 0) { s.xp[w >> 1] = ox; s.yp[w >> 1] = oy; }
        ox += __popc(s.xb[w]);
        oy += __popc(s.yb[w]);
      }
      Nx = (int)(tot & 0xffffffffll);
      Ny = (int)(tot >> 32);
      if (tid == 0) {
        s.Xt = (int*)sc_up(s, base, half, (unsigned long long)Nx * 4);
        s.Yt = (int*)sc_up(s, base, half, (unsigned long long)Ny * 4);
        s.rk = pst ? srk : (int4*)sc_up(s, base, half, (unsigned long long)P * 16);
      }
      __syncthreads();
      if (!s.err) {
        // value tables, one word per thread in turn (set bits are spread, so
        // the threads stay balanced); the rank of a word's first bit comes
        // from the per-2-word prefix
        int* xt = s.Xt;
        int* yt = s.Yt;
        for (int w = tid; w < W; w += TK_NT) {
          unsigned bx = s.xb[w], by = s.yb[w];
          if (bx) {
            int k = (int)s.xp[w >> 1] + ((w & 1) ? __popc(s.xb[w - 1]) : 0);
            while (bx) { const int b = __ffs(bx) - 1; bx &= bx - 1; xt[k++] = (w << 5) + b; }
          }
          if (by) {
            int k = (int)s.yp[w >> 1] + ((w & 1) ? __popc(s.yb[w - 1]) : 0);
            while (by) { const int b = __ffs(by) - 1; by &= by - 1; yt[k++] = (w << 5) + b; }
          }
        }
      }
    }
    const int nslab = Nx - 1;
    const int nsb = (nslab + 62) / 63;
    if (timing) { __syncthreads(); const long long t1 = clock64(); tA += t1 - t0; t0 = t1; }
    // ---- B: sub-band membership (counting sort in shared memory)
    if (tid == 0) s.sbc = nsb <= TK_SBS ? s.sbc_s : (int*)sc_up(s, base, half, (unsigned long long)(nsb + 2) * 4);
    __syncthreads();
    if (!s.sbc) s.sbc = s.sbc_s;  // only after an error (s.err set); the tile is then abandoned
    for (int i = tid; i <= min(nsb, s.sbc == s.sbc_s ? TK_SBS : nsb); i += TK_NT) s.sbc[i] = 0;
    __syncthreads();
    if (!s.err) {
      // warp-uniform trip count: the loop body uses warp-wide match / shuffles
      for (int wb = tid & ~31; wb < P; wb += TK_LD * TK_NT) {
        const int i0 = wb + gb_lane();
        unsigned long long pk[TK_LD];
#pragma unroll
        for (int u = 0; u < TK_LD; ++u) {
          const int i = i0 + u * TK_NT;
          pk[u] = i < P ? (i < nA ? pa[i] : pb[i - nA]) : 0ull;
        }
#pragma unroll
        for (int u = 0; u < TK_LD; ++u) {
          const int i = i0 + u * TK_NT;
          if (i < P) {
            int x1, y1, x2, y2;
            gb_unpack(pk[u], x1, y1, x2, y2);
            const int r1 = bm_rank2(s.xb, s.xp, x1), r2 = bm_rank2(s.xb, s.xp, x2);
            const int c1 = bm_rank2(s.yb, s.yp, y1), c2 = bm_rank2(s.yb, s.yp, y2);
            s.rk[i] = make_int4(r1, r2, c1, c2);
            const int lo = r1 / 63, hi = min(nsb - 1, r2 / 63);
            for (int q = lo; q <= hi; ++q) atomicAdd(&s.sbc[q], 1);
          }
        }
      }
    }
    __syncthreads();
    int M = 0;
    {
      long long carry = 0;
      const int nsbv = s.err ? 0 : nsb;  // after an error the counters are not valid
      for (int b0 = 0; b0 < nsbv; b0 += TK_NT) {
        const int q = b0 + tid;
        const long long v = q < nsbv ? s.sbc[q] : 0;
        long long tot;
        const long long ex = gb_block_excl(v, s.tmp64, &tot);
        if (q < nsbv) s.sbc[q] = (int)(carry + ex);
        carry += tot;
      }
      M = (int)carry;
    }
    if (tid == 0) {
      const int nwy = ((Ny - 1) >> 5) + 1;
      s.mem = (int4*)sc_up(s, base, half, (unsigned long long)M * 16);
      if (nsb <= TK_MDS) {  // the value bitmaps are dead now: keep the metadata on chip
        char* q = reinterpret_cast<char*>(s.xyv);
        s.sbinfo = (int4*)q; q += TK_MDS * 16;
        s.sbol = (int**)q; q += TK_MDS * 8;
        s.sbrec = (PieceRec**)q; q += TK_MDS * 8;
        s.sbh = (int*)q; q += (TK_MDS + 2) * 4;
        s.sbct = (int*)q;
      } else {
        s.sbinfo = (int4*)sc_up(s, base, half, (unsigned long long)nsb * 16);
        s.sbh = (int*)sc_up(s, base, half, (unsigned long long)nsb * 4 + 4);
        s.sbct = (int*)sc_up(s, base, half, (unsigned long long)nsb * 4 + 4);
        s.sbol = (int**)sc_up(s, base, half, (unsigned long long)nsb * 8 + 8);
        s.sbrec = (PieceRec**)sc_up(s, base, half, (unsigned long long)nsb * 8 + 8);
      }
      s.biglb = nwy > TK_LBW ? (unsigned*)sc_up(s, base, half, (unsigned long long)TK_NW * 2 * nwy * 4)
                             : nullptr;
    }
    __syncthreads();
    if (!s.err) {
      const int4* rkp = s.rk;
      int4* memp = s.mem;
      for (int wb = tid & ~31; wb < P; wb += TK_LD * TK_NT) {  // warp-uniform trip count
        const int i0 = wb + gb_lane();
        int4 rr[TK_LD];
#pragma unroll
        for (int u = 0; u < TK_LD; ++u) {
          const int i = i0 + u * TK_NT;
          rr[u] = i < P ? rkp[i] : make_int4(0, -1, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < TK_LD; ++u) {
          const int i = i0 + u * TK_NT;
          if (i < P) {
            const int4 r = rr[u];
            const int lo = r.x / 63, hi = min(nsb - 1, r.y / 63);
            const int4 rec = make_int4(r.x | (i >= nA ? (int)0x80000000 : 0), r.y, r.z, r.w);
            for (int q = lo; q <= hi; ++q) memp[atomicAdd(&s.sbc[q], 1)] = rec;
          }
        }
      }
    }
    __syncthreads();
    if (timing) { const long long t1 = clock64(); tB += t1 - t0; t0 = t1; }
    // ---- C: one warp per sub-band, handed out dynamically, the ones with the most members first
    // (longest processing time first: the phase ends with the last sub-band, so the large ones must
    // not come last).  The order lives in the value-table region, unused until phase D.
    int* const ord = s.xyv + TK_MD_INTS;
    const bool lpt = !s.err && nsb > TK_NW && nsb <= TK_SBS;
    if (lpt) {
      for (int q = tid; q < nsb; q += TK_NT) {
        const int mq = s.sbc[q] - (q ? s.sbc[q - 1] : 0);
        int r = 0;
        for (int j = 0; j < nsb; ++j) {
          const int mj = s.sbc[j] - (j ? s.sbc[j - 1] : 0);
          r += (mj > mq) || (mj == mq && j < q);
        }
        ord[r] = q;
      }
    }
    if (tid == 0) s.sbnext = 0;
    __syncthreads();
    if (!s.err) {
      for (;;) {
        int k = 0;
        if (gb_lane() == 0) k = atomicAdd(&s.sbnext, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= nsb) break;
        tile_subband<TIMING>(s, op, lpt ? ord[k] : k, nsb, Ny, nA, base, scr, timing ? counter + 24 : nullptr);
      }
    }
    // the bulk copies of phase D (async proxy) read the records written above and overwrite shared
    // memory written in phases A-C (generic proxy)
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (timing) {
      const long long t1 = clock64();
      tC += t1 - t0;
      if (tid == 0) {  // phase C per tile, by the tile's sub-band count: 1, 2-3, 4-7, 8-15, 16-31, 32+
        const int bk = nsb <= 1 ? 0 : nsb <= 3 ? 1 : nsb <= 7 ? 2 : nsb <= 15 ? 3 : nsb <= 31 ? 4 : 5;
        atomicAdd((unsigned long long*)&counter[40 + bk], 1ull);
        atomicAdd((unsigned long long*)&counter[46 + bk], (unsigned long long)(t1 - t0));
      }
      t0 = t1;
    }
    // ---- D: stitch and emit.  Piece records, chain links and the x / y value
    // tables are staged in shared memory that phases A-C no longer use.
    const int NP = (int)s.down;
    constexpr int DBYTES = (int)(sizeof(s.lb) + sizeof(s.lp) + sizeof(s.lv) + sizeof(s.ca) + sizeof(s.cb) +
                                 sizeof(s.mc) + sizeof(s.srow));
    const bool prs = (long long)NP * 20 <= DBYTES;
    const int xyoff = nsb <= TK_MDS ? TK_MD_INTS : 0;  // metadata occupies the front of the region
    const int nx4 = (Nx + 3) & ~3, ny4 = (Ny + 3) & ~3;  // tables start on 16-byte boundaries
    const bool xys = nx4 + ny4 + xyoff <= 2 * TK_WMAX + 2 * (TK_WMAX / 2 + 1);
    if (tid == 0 && !s.err && !prs) s.succ = (int*)sc_up(s, base, half, (unsigned long long)NP * 4 + 4);
    __syncthreads();
    if (s.err) {
      if (tid == 0) {
        O->tcount[t] = 0;
        O->tstart[t] = 0;
        gb_set_error(st, GB_ERR_CAPACITY, KID_TILE, (long long)scr * 2);
      }
      continue;
    }
    // the next tile's reservation (the work counter) and its descriptor load run on the last thread while
    // the bulk copies below land
    if (tid == TK_NT - 1 && !st->err) {
      tile_lookup(op, A, B, O, (long long)atomicAdd((unsigned long long*)counter, 1ull), s.nx);
      s.have_nx = 1;
    }
    PieceRec* PR = prs ? reinterpret_cast<PieceRec*>(s.dbuf) : nullptr;
    int* succ = prs ? reinterpret_cast<int*>(s.dbuf + (size_t)NP * 16) : s.succ;
    const int* Xv = xys ? s.xyv + xyoff : s.Xt;
    const int* Yv = xys ? s.xyv + xyoff + nx4 : s.Yt;
    // record of global piece q, which belongs to sub-band sb
    auto REC = [&](int sb, int q) -> PieceRec { return prs ? PR[q] : s.sbrec[sb][q - s.sbinfo[sb].x]; };
    const int wid = gb_warp(), lane = gb_lane();
    // piece records of every sub-band and the x / y value tables into shared memory by bulk copies
    // (all 16-byte aligned: records are 16 bytes, scratch allocations are rounded to 16 bytes)
    if ((prs && NP > 0) || xys) {
      if (tid == 0) {
        const unsigned bytes = (prs ? (unsigned)NP * 16u : 0u) + (xys ? (unsigned)(nx4 + ny4) * 4u : 0u);
        asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(mbar),
                     "r"(bytes)
                     : "memory");
        if (xys) {
          if (nx4) tk_bulk(s.xyv + xyoff, s.Xt, (unsigned)nx4 * 4u, mbar);
          if (ny4) tk_bulk(s.xyv + xyoff + nx4, s.Yt, (unsigned)ny4 * 4u, mbar);
        }
      }
      if (prs && !s.rsplit) {
        if (tid == 0 && NP > 0) tk_bulk(PR, base + (half & ~15ull), (unsigned)NP * 16u, mbar);
      } else if (prs && wid == 0) {
        for (int sb = lane; sb < nsb; sb += 32) {
          const int4 inf = s.sbinfo[sb];
          if (inf.y > 0) tk_bulk(PR + inf.x, s.sbrec[sb], (unsigned)inf.y * 16u, mbar);
        }
      }
      const bool ok = tk_wait(mbar, mph, TK_SPIN_LIMIT);
      mph ^= 1u;
      if (__syncthreads_or(!ok)) {
        if (tid == 0) gb_set_error(st, GB_ERR_TIMEOUT, KID_TILE_COPY, t);
        tk_wait(mbar, mph ^ 1u, TK_SPIN_LIMIT);  // let copies in flight land before the CTA exits
        return;
      }
    }
    for (int p = tid; p < NP; p += TK_NT) succ[p] = -1;
    int H = 0;
    {
      long long carry = 0;
      for (int b0 = 0; b0 < nsb; b0 += TK_NT) {
        const int q = b0 + tid;
        const long long v = q < nsb ? s.sbh[q] : 0;
        long long tot;
        const long long ex = gb_block_excl(v, s.tmp64, &tot);
        if (q < nsb) s.sbh[q] = (int)(carry + ex);
        carry += tot;
      }
      H = (int)carry;
    }
    __syncthreads();
    if (tid == TK_NT - 32) {  // read after the links' barrier
      s.obase = -1;
      if (mode == 0 && H > 0) {
        atomicAdd((unsigned long long*)&O->ntot, (unsigned long long)H);
        const long long o = (long long)atomicAdd((unsigned long long*)&O->nused, (unsigned long long)H);
        if (o + H <= O->npcs) {
          s.obase = o;
        } else {
          unsigned long long* p =
              (unsigned long long*)gb_arena_alloc_atomic(st, (unsigned long long)H * 8ull, KID_TILE + 1);
          if (p) s.obase = (long long)(p - O->pcs);
        }
      }
    }
    // link every continuation piece to the open piece of the previous
    // sub-band: its row-0 ordinal indexes that sub-band's open list directly
    for (int sb = 1 + wid; sb < nsb; sb += TK_NW) {
      const int nc = s.sbct[sb];
      if (!nc) continue;
      const int* cl = s.sbol[sb] + s.sbinfo[sb].z;
      const int4 pinf = s.sbinfo[sb - 1];
      const int* ol = s.sbol[sb - 1];
      for (int k = lane; k < nc; k += 32) {
        const int p = cl[k];
        const int ord = pr_hrank(REC(sb, p));
        if (ord < pinf.z) succ[ol[ord]] = p;
        else gb_set_error(st, GB_ERR_INTERNAL, KID_TILE, t);
      }
    }
    __syncthreads();
    const long long obase = s.obase;
    unsigned long long* outp = obase >= 0 ? O->pcs + obase : nullptr;
    long long area = 0;
    if (prs) {
      // records on chip: every thread takes pieces in turn; a piece's sub-band is its first slab / 63
      // (its first row is 1..63 of that sub-band)
      for (int p = tid; p < NP; p += TK_NT) {
        const PieceRec pr = PR[p];
        if (pr_cont(pr)) continue;
        int q = p, guard = 0;
        while (succ[q] >= 0 && guard++ <= nsb) q = succ[q];
        const int shi = q == p ? pr_shi(pr) : pr_shi(PR[q]);
        const int slo = pr_slo(pr);
        const int xs = Xv[slo], xe = Xv[shi], ylo = Yv[pr_ylo(pr)], yhi = Yv[pr_yhi(pr)];
        const int pos = s.sbh[slo / 63] + pr_hrank(pr);
        if (outp) outp[pos] = gb_pack(xs, ylo, xe, yhi);
        area += (long long)(xe - xs) * (long long)(yhi - ylo);
      }
    } else {
      for (int sb = wid; sb < nsb; sb += TK_NW) {
        const int4 inf = s.sbinfo[sb];
        for (int j = lane; j < inf.y; j += 32) {
          const int p = inf.x + j;
          const PieceRec pr = REC(sb, p);
          if (pr_cont(pr)) continue;
          int q = p, sq = sb, guard = 0;
          while (succ[q] >= 0 && guard++ <= nsb) { q = succ[q]; ++sq; }
          const int shi = q == p ? pr_shi(pr) : pr_shi(REC(sq, q));
          const int slo = pr_slo(pr);
          const int xs = Xv[slo], xe = Xv[shi], ylo = Yv[pr_ylo(pr)], yhi = Yv[pr_yhi(pr)];
          const int pos = s.sbh[sb] + pr_hrank(pr);
          if (outp) outp[pos] = gb_pack(xs, ylo, xe, yhi);
          area += (long long)(xe - xs) * (long long)(yhi - ylo);
        }
      }
    }
    area = gb_block_sum(area, s.tmp64);
    if (tid == 0) {
      if (mode == 0) {
        O->tcount[t] = obase >= 0 ? H : 0;
        O->tstart[t] = obase >= 0 ? obase : 0;
      } else {
        O->tcount[t] = H;
      }
      atomicAdd((unsigned long long*)&O->cell_area[s.cell], (unsigned long long)area);
      atomicAdd((unsigned long long*)&O->cell_count[s.cell], (unsigned long long)H);
      if (timing) {
        const long long t1 = clock64();
        tD += t1 - t0;
        atomicAdd((unsigned long long*)&counter[20], 1ull);
        atomicAdd((unsigned long long*)&counter[21], (unsigned long long)P);
        atomicAdd((unsigned long long*)&counter[22], (unsigned long long)nsb);
        atomicAdd((unsigned long long*)&counter[23], (unsigned long long)NP);
      }
      atomicAdd((unsigned long long*)&counter[8], (unsigned long long)P * 8ull);
      atomicAdd((unsigned long long*)&counter[9], (unsigned long long)(mode == 0 ? H : 0) * 8ull);
    }
  }
  if (timing && threadIdx.x == 0) {
    atomicAdd((unsigned long long*)&counter[16], (unsigned long long)tA);
    atomicAdd((unsigned long long*)&counter[17], (unsigned long long)tB);
    atomicAdd((unsigned long long*)&counter[18], (unsigned long long)tC);
    atomicAdd((unsigned long long*)&counter[19], (unsigned long long)tD);
  }
}

void gb_tile_setup(GbCtx& c) {
  c.tile_smem = sizeof(TileSmem);
  cudaFuncSetAttribute(k_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.tile_smem);
  cudaFuncSetAttribute(k_tile<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.tile_smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<false>, TK_NT, c.tile_smem);
  c.tile_blocks = c.nsm * (per_sm > 0 ? per_sm : 1);
}

__global__ void k_zero_counter(long long* ctr) { *ctr = 0; }

// The output pool is sized for the worst case (cap_factor x input pieces) and
// tiles reserve exactly what they emit.  When nothing was allocated in the
// arena after the pool (no overflow, no scratch spill), the unused tail goes
// back to the arena, so a chain of operators keeps only what it produced.
__global__ void k_pool_trim(DLayer* O, DStatus* st) {
  if (st->err || !O->pcs) return;
  const unsigned long long start = (unsigned long long)((char*)O->pcs - st->arena_base);
  const unsigned long long end = start + (((unsigned long long)O->npcs * 8ull + 255ull) & ~255ull);
  if (st->arena_off != end || O->nused > O->npcs) return;
  const long long used = O->nused > 0 ? O->nused : 0;
  st->arena_off = start + (((unsigned long long)used * 8ull + 255ull) & ~255ull);
  O->npcs = used;
}

void gb_launch_tile_bool(GbCtx& c, int op, const DLayer* A, const DLayer* B, DLayer* O, int g, int mode) {
  k_zero_counter<<<1, 1, 0, c.stream>>>(c.tile_counter);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c.prof) {
    if (c.prof_used + 2 > c.prof_ev.size()) {
      for (int i = 0; i < 64; ++i) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c.prof_ev.push_back(e);
      }
    }
    e0 = c.prof_ev[c.prof_used++];
    e1 = c.prof_ev[c.prof_used++];
    // inside a stream capture only an external record becomes a real event node
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c.stream, &cs);
    c.prof_flags = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0;
    cudaEventRecordWithFlags(e0, c.stream, c.prof_flags);
  }
  if (c.timing)
    k_tile<true><<<c.tile_blocks, TK_NT, c.tile_smem, c.stream>>>(op, A, B, O, g, mode | 4, c.tile_scratch,
                                                                c.tile_scr_bytes, c.tile_counter, c.st);
  else
    k_tile<false><<<c.tile_blocks, TK_NT, c.tile_smem, c.stream>>>(op, A, B, O, g, mode, c.tile_scratch,
                                                                 c.tile_scr_bytes, c.tile_counter, c.st);
  if (c.prof) cudaEventRecordWithFlags(e1, c.stream, c.prof_flags);
  c.launches += 2;
  if (mode == 0) {
    k_pool_trim<<<1, 1, 0, c.stream>>>(O, c.st);
    ++c.launches;
  }
}

// ===================================================================== no-allocation entry point
// gb_bool_tile_noalloc: the scanline Boolean for callers that cannot allocate
// device memory -- code running where cudaMalloc is not permitted on the
// request path (a serving loop that has reserved its whole device budget up
// front, a host that must not take the allocator's implicit device-wide
// synchronisation, or a Fortran/C caller that only owns the buffers it
// passes).  It computes the canonical strips of pred(A, B) for boxes that all
// lie inside one 65536-dbu tile, entirely in memory reserved statically in
// this library: every GPU that loads libgbool.so holds this storage until the
// process exits.
//
// Limits: nA + nB <= GB_NA_MAX_IN boxes (nA alone for MERGE, which ignores
// B), at most GB_NA_MAX_OUT result strips, and the CTA scratch of
// GB_NA_SCRATCH bytes.  Beyond any of them the call returns GB_ERR_CAPACITY;
// a result with more strips than the caller's out_cap does too.  On every
// status other than GB_OK, *d_count (and *d_area when given) is -1.
//
// All calls share the static storage (each call re-initialises what must
// start at zero and keeps the last call's contents otherwise), so calls whose
// work overlaps on the GPU -- on different streams, or from different host
// threads -- race and must be serialised by the caller.  Every call waits for
// its stream to finish before it returns.
//
// Set-up: the first call on a device resolves the device addresses of the
// static storage with cudaGetSymbolAddress (with that device current) and
// sets the kernel's shared-memory attribute; later calls on that device reuse
// them.
#define GB_NA_MAX_IN 16384
#define GB_NA_MAX_OUT 65536
#define GB_NA_SCRATCH (8u << 20)
#define GB_NA_MAX_DEV 64

// What the host reads back after a call, in one copy: the status and the
// result's strip count (also when it exceeds the caller's buffer).
struct NoAllocResult {
  DStatus st;       // status; its arena is empty (no spill space)
  long long nout;   // strips of the result
};

struct NoAllocState {
  NoAllocResult res;
  DLayer L[3];                              // A, B, result
  long long ctr[64];                        // work counters of the tile kernel
  int4 win[3];
  long long tbase[3][2];
  long long tstart[3][2];
  int tcount[3][2];
  long long cell_count[3];
  long long cell_area[3];
  int4 cbox[3];
  unsigned long long pcs_in[GB_NA_MAX_IN];  // packed pieces of A then B
  unsigned long long pcs_out[GB_NA_MAX_OUT];
};

static __device__ __align__(256) NoAllocState g_na_state;
static __device__ __align__(256) char g_na_scratch[GB_NA_SCRATCH];

static NoAllocState* g_na_state_ptr[GB_NA_MAX_DEV];
static char* g_na_scratch_ptr[GB_NA_MAX_DEV];
static std::mutex g_na_mu;

// Re-initialise the shared state and pack the inputs (one block).  Every box
// must lie inside the tile of the first box; otherwise the status says so.
// MERGE reads A only.
__global__ void k_na_prep(NoAllocState* S, int op, const int4* A, int nA, const int4* B, int nB, int g) {
  __shared__ int bad;
  __shared__ int tx0, ty0;
  if (op == GB_OP_MERGE) nB = 0;
  if (threadIdx.x == 0) {
    bad = 0;
    const int4 f = nA ? A[0] : (nB ? B[0] : make_int4(0, 0, 1, 1));
    tx0 = gb_floor_shift(f.x, g);
    ty0 = gb_floor_shift(f.y, g);
    memset(&S->res, 0, sizeof(S->res));  // empty arena: spills report GB_ERR_CAPACITY
    for (int i = 0; i < 64; ++i) S->ctr[i] = 0;
  }
  __syncthreads();
  const int n = nA + nB;
  const int ox = tx0 << g, oy = ty0 << g;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int4 b = i < nA ? A[i] : B[i - nA];
    const bool ok = b.x < b.z && b.y < b.w && gb_floor_shift(b.x, g) == tx0 &&
                    gb_floor_shift(b.z - 1, g) == tx0 && gb_floor_shift(b.y, g) == ty0 &&
                    gb_floor_shift(b.w - 1, g) == ty0;
    if (!ok) { atomicOr(&bad, 1); continue; }
    S->pcs_in[i] = gb_pack(b.x - ox, b.y - oy, b.z - ox, b.w - oy);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bad) gb_set_error(&S->res.st, GB_ERR_INVALID_BOX, 60, 0);
    for (int l = 0; l < 3; ++l) {
      DLayer& d = S->L[l];
      memset(&d, 0, sizeof(d));
      d.ncell = 1;
      d.g = g;
      d.binned = 1;
      S->win[l] = make_int4(tx0, ty0, 1, 1);
      S->tbase[l][0] = 0;
      S->tbase[l][1] = 1;
      S->cell_count[l] = 0;
      S->cell_area[l] = 0;
      S->cbox[l] = make_int4(ox, oy, ox + (1 << g), oy + (1 << g));
      d.win = &S->win[l];
      d.tbase = S->tbase[l];
      d.tstart = S->tstart[l];
      d.tcount = S->tcount[l];
      d.cell_count = &S->cell_count[l];
      d.cell_area = &S->cell_area[l];
      d.cbox = &S->cbox[l];
      d.ntiles = 1;
    }
    S->L[0].pcs = S->pcs_in;
    S->tstart[0][0] = 0;
    S->tcount[0][0] = nA;
    S->L[0].npcs = S->L[0].nused = S->L[0].ntot = nA;
    S->L[1].pcs = S->pcs_in;
    S->tstart[1][0] = nA;
    S->tcount[1][0] = nB;
    S->L[1].npcs = S->L[1].nused = S->L[1].ntot = nB;
    S->L[2].pcs = S->pcs_out;
    S->L[2].npcs = GB_NA_MAX_OUT;
    S->tstart[2][0] = 0;
    S->tcount[2][0] = 0;
    if (bad) S->L[2].ntiles = 0;  // nothing runs on invalid input
  }
}

// Unpack the result into the caller's buffer; *count = strips, or -1 when the
// call failed or the buffer is too small.  The strip count also goes to the
// state, for the host.
__global__ void k_na_export(NoAllocState* S, int4* out, long long cap, long long* count, long long* area) {
  const DLayer& O = S->L[2];
  const long long n = O.ntiles ? O.tcount[0] : 0;
  const bool ok = S->res.st.err == 0 && n <= cap;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *count = ok ? n : -1;
    if (area) *area = ok ? S->cell_area[2] : -1;
  }
  if (!ok) {
    if (threadIdx.x == 0 && blockIdx.x == 0) S->res.nout = n;
    return;
  }
  const int4 w = S->win[2];
  const int ox = w.x << O.g, oy = w.y << O.g;
  const unsigned long long* p = O.pcs + O.tstart[0];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int a, b, c, d;
    gb_unpack(p[i], a, b, c, d);
    out[i] = make_int4(ox + a, oy + b, ox + c, oy + d);
  }
  if (threadIdx.x == 0 && blockIdx.x == 0) S->res.nout = n;
}

// *d_count = -1 (and *d_area) for a call refused before its kernels run.
static int na_refuse(int code, long long* d_count, long long* d_area, cudaStream_t s) {
  if (d_count) cudaMemsetAsync(d_count, 0xff, sizeof(long long), s);
  if (d_area) cudaMemsetAsync(d_area, 0xff, sizeof(long long), s);
  if (d_count || d_area) cudaStreamSynchronize(s);
  return code;
}

extern "C" int gb_bool_tile_noalloc(int op, const int4* d_A, int nA, const int4* d_B, int nB, int4* d_out,
                                    long long out_cap, long long* d_count, long long* d_area, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (op == GB_OP_MERGE) nB = nB < 0 ? nB : 0;
  if (op < GB_OP_XOR || op > GB_OP_MERGE || nA < 0 || nB < 0 || out_cap < 0 || !d_out || !d_count ||
      (nA && !d_A) || (nB && !d_B))
    return na_refuse(GB_ERR_ARG, d_count, d_area, s);
  if ((long long)nA + nB > GB_NA_MAX_IN) {
    fprintf(stderr, "gb_bool_tile_noalloc: %lld input boxes exceed the static limit of %d\n",
            (long long)nA + nB, GB_NA_MAX_IN);
    return na_refuse(GB_ERR_CAPACITY, d_count, d_area, s);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GB_NA_MAX_DEV)
    return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
  NoAllocState* S;
  char* scr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_state_ptr[dev]) {
      void* a = nullptr;
      void* b = nullptr;
      if (cudaGetSymbolAddress(&a, g_na_state) != cudaSuccess ||
          cudaGetSymbolAddress(&b, g_na_scratch) != cudaSuccess) {
        fprintf(stderr, "gb_bool_tile_noalloc: cudaGetSymbolAddress failed on device %d\n", dev);
        return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
      }
      if (cudaFuncSetAttribute(k_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TileSmem)) !=
          cudaSuccess)
        return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
      g_na_state_ptr[dev] = (NoAllocState*)a;
      g_na_scratch_ptr[dev] = (char*)b;
    }
    S = g_na_state_ptr[dev];
    scr = g_na_scratch_ptr[dev];
  }
  // each launch reports its own error (no reliance on the thread's last-error state)
  const int g = 16;
  {
    void* args[] = {&S, &op, &d_A, &nA, &d_B, &nB, (void*)&g};
    if (cudaLaunchKernel((const void*)k_na_prep, dim3(1), dim3(256), args, 0, s) != cudaSuccess)
      return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
  }
  {
    DLayer* la = &S->L[0];
    DLayer* lb = &S->L[1];
    DLayer* lo = &S->L[2];
    int gg = g, mode = 0;
    unsigned long long scr_bytes = GB_NA_SCRATCH;
    long long* ctr = S->ctr;
    DStatus* st = &S->res.st;
    void* args[] = {&op, &la, &lb, &lo, &gg, &mode, &scr, &scr_bytes, &ctr, &st};
    if (cudaLaunchKernel((const void*)k_tile<false>, dim3(1), dim3(TK_NT), args, sizeof(TileSmem), s) != cudaSuccess)
      return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
  }
  {
    void* args[] = {&S, &d_out, &out_cap, &d_count, &d_area};
    if (cudaLaunchKernel((const void*)k_na_export, dim3(8), dim3(256), args, 0, s) != cudaSuccess)
      return na_refuse(GB_ERR_CUDA, d_count, d_area, s);
  }
  NoAllocResult hr;
  if (cudaMemcpyAsync(&hr, &S->res, sizeof(hr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GB_ERR_CUDA;
  if (hr.st.err == GB_ERR_CAPACITY)
    fprintf(stderr, "gb_bool_tile_noalloc: result exceeds the static limits (%d strips, %u scratch bytes)\n",
            GB_NA_MAX_OUT, GB_NA_SCRATCH);
  if (hr.st.err) return hr.st.err;
  if (hr.nout > out_cap) {
    fprintf(stderr, "gb_bool_tile_noalloc: %lld result strips exceed out_cap %lld\n", hr.nout, out_cap);
    return GB_ERR_CAPACITY;
  }
  return GB_OK;
}
