// gb_radix.cu -- hand-written LSD radix sort (onesweep form) for 64-bit keys
// with 32-bit payloads: Morton-ordered boxes (gpu_morton.cu:113-187),
// tracker events (event_sorter.cu:48-81) and canonical strip order.
//
//  1. One read of the keys builds the digit histograms of every pass
//     (one CTA per SM with shared-memory counters, merged with global
//     atomics; two adjacent narrow passes share a joint table, so a shared
//     atomic counts a key for both).
//  2. Each pass is one kernel: a CTA takes the next tile from an atomic
//     counter (so tiles start in order) and pulls the tile's keys and values
//     into shared memory with two bulk asynchronous copies completing on an
//     mbarrier.  Warps rank the keys stably (peers by shared lane masks, or
//     warp match and per-bit ballots for wide digits), the CTA
//     publishes its per-digit counts, and obtains the exclusive prefix of all
//     earlier tiles by a decoupled look-back over a status array.  Keys and
//     values are then permuted in place in shared memory by digit and
//     written out in runs.
// Digits are 1..10 bits wide; the passes split the significant key bits as
// evenly as possible (e.g. 52 bits in 6 passes: 9,9,9,9,8,8), so the pass
// count is a free choice.  An even pass count leaves the result in place;
// an odd one costs a final copy.
// Status words ([tile][digit]) carry an epoch tag, so the array is never
// cleared between passes.  Every wait is bounded: after the limit the kernel flags
// GB_ERR_TIMEOUT in the context status and finishes without hanging.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "gb_internal.h"
#include "gb_scan.cuh"

#define RS_MAXPASS 16
#define RS_HIST_SLOTS 8192
#define RS_SPIN_LIMIT (1 << 22)
#define RS_LBDEPTH 8  // predecessors a digit's thread polls per round trip
#define KID_RADIX 40
#define KID_RADIX_COPY 41

// status word: [63:48] epoch, [47:46] flag (1 aggregate, 2 inclusive prefix), [45:0] value
#define RS_FLAG_AGG 1ull
#define RS_FLAG_PRE 2ull

struct RsPlan {
  int np;
  int shift[RS_MAXPASS];
  int bits[RS_MAXPASS];
  int off[RS_MAXPASS];  // offset of the pass's counters in the histogram array
};

// ---------------------------------------------------------------- histogram
// Counters of adjacent passes whose digits together are at most
// RS_JOINT_BITS wide are kept as one joint table indexed by both digits (a
// 7-bit and a 7-bit digit: 16384 counters), so one shared atomic counts a key
// for two passes; each pass's counts are the table's row or column sums.
#define RS_JOINT_BITS 14
#define RS_HIST_WORDS (48 * 1024)  // shared counters of one histogram CTA (192 KB)
#define RS_HIST_KPT 4              // keys per thread per step

struct RsHistPlan {
  int ng;                // counter groups
  int words;             // shared counters in all groups
  int gshift[RS_MAXPASS];  // shift of the group's low digit
  int gbits[RS_MAXPASS];   // width of the group's (joint) index
  int goff[RS_MAXPASS];    // offset of the group's counters in shared memory
  int gp[RS_MAXPASS];      // first pass of the group
  int gn[RS_MAXPASS];      // passes in the group: 1 or 2
};

template <bool VEC>
__global__ void __launch_bounds__(1024, 1)
k_rs_hist(const unsigned long long* __restrict__ keys, long long n, RsPlan plan, RsHistPlan hp,
          unsigned* __restrict__ ghist) {
  extern __shared__ unsigned hj[];
  const int ng = hp.ng;
  for (int i = threadIdx.x; i < hp.words; i += blockDim.x) hj[i] = 0;
  __syncthreads();
  const long long nq = n / RS_HIST_KPT;
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += step) {
    unsigned long long k[RS_HIST_KPT];
    if (VEC) {
      const ulonglong2* q = reinterpret_cast<const ulonglong2*>(keys) + (RS_HIST_KPT / 2) * i;
#pragma unroll
      for (int j = 0; j < RS_HIST_KPT / 2; ++j) {
        const ulonglong2 a = q[j];
        k[2 * j] = a.x;
        k[2 * j + 1] = a.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < RS_HIST_KPT; ++j) k[j] = keys[RS_HIST_KPT * i + j];
    }
#pragma unroll
    for (int g = 0; g < RS_MAXPASS; ++g) {
      if (g >= ng) break;
      const int sh = hp.gshift[g];
      const unsigned m = (1u << hp.gbits[g]) - 1u;
      unsigned* t = hj + hp.goff[g];
#pragma unroll
      for (int j = 0; j < RS_HIST_KPT; ++j) atomicAdd(&t[(unsigned)(k[j] >> sh) & m], 1u);
    }
  }
  const long long r0 = nq * RS_HIST_KPT;
  if (blockIdx.x == 0 && threadIdx.x < n - r0) {
    const unsigned long long kk = keys[r0 + threadIdx.x];
    for (int g = 0; g < ng; ++g)
      atomicAdd(&hj[hp.goff[g] + ((unsigned)(kk >> hp.gshift[g]) & ((1u << hp.gbits[g]) - 1u))], 1u);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int g = 0; g < ng; ++g) {
    const unsigned* t = hj + hp.goff[g];
    const int p = hp.gp[g];
    if (hp.gn[g] == 1) {
      for (int d = threadIdx.x; d < (1 << hp.gbits[g]); d += blockDim.x) {
        const unsigned v = t[d];
        if (v) atomicAdd(&ghist[plan.off[p] + d], v);
      }
      continue;
    }
    // joint index = low digit | high digit << bl
    const int bl = plan.bits[p], rl = 1 << bl, rh = 1 << plan.bits[p + 1];
    for (int d = threadIdx.x; d < rl; d += blockDim.x) {  // low pass: column sums
      unsigned v = 0;
      for (int e = 0; e < rh; ++e) v += t[(e << bl) | d];
      if (v) atomicAdd(&ghist[plan.off[p] + d], v);
    }
    for (int e = threadIdx.x >> 5; e < rh; e += blockDim.x >> 5) {  // high pass: row sums, a warp per row
      unsigned v = 0;
      for (int d = lane; d < rl; d += 32) v += t[(e << bl) | d];
      v = __reduce_add_sync(0xffffffffu, v);
      if (lane == 0 && v) atomicAdd(&ghist[plan.off[p + 1] + e], v);
    }
  }
}

// one block of 1024 threads per pass: exclusive scan of the pass's digit counts
__global__ void __launch_bounds__(1024) k_rs_hist_scan(unsigned* ghist, RsPlan plan) {
  __shared__ long long tmp[33];
  const int p = blockIdx.x;
  const int radix = 1 << plan.bits[p];
  unsigned* g = ghist + plan.off[p];
  const long long v = threadIdx.x < radix ? g[threadIdx.x] : 0;
  long long tot;
  const long long ex = gb_block_excl(v, tmp, &tot);
  if (threadIdx.x < radix) g[threadIdx.x] = (unsigned)ex;
}

// ---------------------------------------------------------------- async copy helpers
__device__ __forceinline__ unsigned rs_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void rs_mbar_init(unsigned a) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void rs_mbar_expect(unsigned a, unsigned bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(a), "r"(bytes)
               : "memory");
}

// global -> shared bulk copy; both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void rs_bulk_load(unsigned dst, const void* src, unsigned bytes, unsigned mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

__device__ __forceinline__ bool rs_mbar_try(unsigned a, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for phase 0 of the mbarrier; false after `limit` polls
__device__ __forceinline__ bool rs_mbar_wait(unsigned a, int limit) {
  for (int i = 0; i < limit; ++i)
    if (rs_mbar_try(a, 0)) return true;
  return false;
}

// ---------------------------------------------------------------- one pass
// Radices up to RS_AO_RADIX find a key's peers through per-warp lane masks in
// shared memory (one word per digit); larger ones by warp match / ballots.
#define RS_AO_RADIX 128

// Shared memory of a pass with NT threads, tile T = NT * IT keys and radix R:
//   keys T*8 | vals T*4 | wh[NT/32][R] u16 | bstart[R] u32 | gpos[R] u32 | mbarrier, tile, scan scratch
//   | lane masks [NT/32][R] u32 when R <= RS_AO_RADIX
__host__ __device__ constexpr size_t rs_smem_bytes(int nt, int it, int radix) {
  return (size_t)nt * it * 12 + (size_t)(nt / 32) * radix * 2 + (size_t)radix * 8 + 16 + 33 * 8 +
         (radix <= RS_AO_RADIX ? (size_t)(nt / 32) * radix * 4 : 0);
}

// The digit [shift, shift + dbits) of a key, taken from its two 32-bit words
// with one funnel shift (the word choice is uniform over the pass).
struct RsDigit {
  bool hiw;
  int s;
  unsigned mask;
  __device__ RsDigit(int shift, unsigned m) : hiw(shift >= 32), s(shift & 31), mask(m) {}
  __device__ __forceinline__ unsigned operator()(unsigned long long k) const {
    const unsigned lo = (unsigned)k, hi = (unsigned)(k >> 32);
    return __funnelshift_r(hiw ? hi : lo, hiw ? 0u : hi, s) & mask;
  }
};

// The work on a tile resident in shared memory: rank, prefix, permutation,
// look-back and write-out.  FULL: the tile holds TILE keys (no bounds tests).
template <int NT, int IT, int MAXB, bool FULL>
__device__ __forceinline__ void rs_tile(unsigned long long* sk, unsigned* sv, unsigned short* wh, unsigned* bstart,
                                        unsigned* gpos, long long* tmp, unsigned* mbuf, const RsDigit& digit,
                                        int radix, int cnt,
                                        long long tile, long long ntile, const unsigned* __restrict__ gofs,
                                        unsigned long long* status, unsigned long long epoch, DStatus* st,
                                        int spin_limit, unsigned long long* __restrict__ kout,
                                        unsigned* __restrict__ vout) {
  constexpr int TILE = NT * IT;
  constexpr int NW = NT / 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  // ---- rank: warp w owns keys [w*32*IT, (w+1)*32*IT) in order.  Peers with
  // the same digit are found through shared lane masks (radix <= RS_AO_RADIX)
  // or by a warp match (every third item) and one ballot per digit bit (the
  // others), so the match unit and the integer pipe share the work; the lowest peer adds the group to the warp's counter (two 16-bit counters share a 32-bit
  // word; a count never exceeds 32*IT, so no carry crosses halves) and
  // broadcasts the old value.  Keys stay in registers; ranks are packed two
  // to a register.
  const unsigned lt = (1u << lane) - 1u;
  const int wbase = wid * 32 * IT;
  unsigned short* mywh = wh + wid * radix;
  unsigned* mywh32 = reinterpret_cast<unsigned*>(mywh);
  unsigned long long kk[IT];
  unsigned rd[(IT + 1) / 2];
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int idx = wbase + it * 32 + lane;
    const bool ok = FULL || idx < cnt;
    kk[it] = ok ? sk[idx] : 0ull;
    const unsigned d = digit(kk[it]);
    unsigned peers;
    if (radix <= RS_AO_RADIX) {
      // lane masks: each lane ORs its bit into its warp's word for its digit
      // and reads the word back (shared-memory pipe, no votes); the peers
      // then clear it for the next item
      unsigned* mm = mbuf + wid * radix;
      if (ok) atomicOr(&mm[d], 1u << lane);
      __syncwarp();
      peers = ok ? mm[d] : 0u;
      if (!FULL) {
        const unsigned vm = __ballot_sync(0xffffffffu, ok);
        if (!ok) peers = ~vm;
      }
      __syncwarp();
      if (ok) mm[d] = 0u;
      __syncwarp();
    } else if (it % 3 == 1) {
      // every third item: warp match (its own pipe), invalid lanes carry an out-of-range digit
      peers = __match_any_sync(0xffffffffu, ok ? d : 0xFFFFFFFFu);
    } else {
      // the others: one ballot per digit bit (integer pipe)
      peers = 0xffffffffu;
      if (!FULL) {
        const unsigned vm = __ballot_sync(0xffffffffu, ok);
        peers = ok ? vm : ~vm;
      }
#pragma unroll
      for (int b = 0; b < MAXB; ++b) {
        const unsigned bit = (d >> b) & 1u;
        const unsigned bb = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? bb : ~bb;
      }
    }
    const int leader = __ffs(peers) - 1;
    unsigned old = 0;
    if (ok && lane == leader) old = atomicAdd(&mywh32[d >> 1], (unsigned)__popc(peers) << ((d & 1u) * 16));
    old = __shfl_sync(0xffffffffu, old, leader);
    const unsigned r = ((old >> ((d & 1u) * 16)) & 0xFFFFu) + __popc(peers & lt);
    if (it & 1) rd[it >> 1] |= r << 16;
    else rd[it >> 1] = r;
  }
  __syncthreads();

  // ---- per digit: tile total (published as the tile's aggregate), the
  // tile's bucket start, and each warp's first slot of the digit, folded
  // into the warp counters (loops over a thread's digits run to the
  // compile-time bound 4 so the per-digit arrays stay in registers)
  const int dpt = radix > NT ? radix / NT : 1;  // digits per thread (1..4)
  const int d0 = tid * dpt;
  const bool own = d0 < radix;
  unsigned tots[4] = {0u, 0u, 0u, 0u};
  long long tsum = 0;
  const unsigned long long etag = (epoch & 0xFFFFull) << 48;
  if (own) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < dpt) {
        const int d = d0 + j;
        unsigned tot = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) tot += wh[w * radix + d];
        tots[j] = tot;
        tsum += tot;
        gpos[d] = tot;  // kept for the look-back, which replaces it
        const unsigned long long flag = tile == 0 ? RS_FLAG_PRE : RS_FLAG_AGG;
        *(volatile unsigned long long*)(status + (size_t)tile * radix + d) = etag | (flag << 46) | tot;
      }
    }
  }
  {
    long long tt;
    long long ex = gb_block_excl(tsum, tmp, &tt);
    if (own) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j < dpt) {
          const int d = d0 + j;
          bstart[d] = (unsigned)ex;
          unsigned run = (unsigned)ex;
#pragma unroll
          for (int w = 0; w < NW; ++w) {
            const unsigned c = wh[w * radix + d];
            wh[w * radix + d] = (unsigned short)run;
            run += c;
          }
          ex += tots[j];
        }
      }
    }
  }
  __syncthreads();

  // ---- permute in place: every read of the key array happened before the
  // last barrier, so keys go straight from registers to their slots; rd
  // becomes the slot pair.  Values: all reads, a barrier, then the writes.
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    if (FULL || wbase + it * 32 + lane < cnt) {
      const unsigned d = digit(kk[it]);
      const unsigned r = (it & 1) ? (rd[it >> 1] >> 16) : (rd[it >> 1] & 0xFFFFu);
      const unsigned p = mywh[d] + r;
      sk[p] = kk[it];
      rd[it >> 1] = (it & 1) ? ((rd[it >> 1] & 0xFFFFu) | (p << 16)) : ((rd[it >> 1] & 0xFFFF0000u) | p);
    }
  }
  {
    unsigned vv[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int idx = wbase + it * 32 + lane;
      if (FULL || idx < cnt) vv[it] = sv[idx];
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; ++it)
      if (FULL || wbase + it * 32 + lane < cnt) sv[(it & 1) ? (rd[it >> 1] >> 16) : (rd[it >> 1] & 0xFFFFu)] = vv[it];
  }

  // ---- decoupled look-back: the thread of digit d polls the status words of
  // RS_LBDEPTH / (digits per thread) predecessors at once (a warp reads whole
  // rows of the [tile][digit] array), sums aggregates up to the nearest
  // inclusive prefix, and polls again from the first word not yet published.
  if (own) {
    constexpr int DEPTH = RS_LBDEPTH;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < dpt) {
        const int d = d0 + j;
        unsigned excl = 0;
        if (tile > 0) {
          long long jp = tile - 1;  // next predecessor to read
          int spins = 0;
          const int depth = DEPTH / dpt;
          for (;;) {
            unsigned long long w[DEPTH];
#pragma unroll
            for (int i = 0; i < DEPTH; ++i)
              w[i] = (i < depth && jp - i >= 0) ? *(volatile unsigned long long*)(status + (size_t)(jp - i) * radix + d)
                                               : 0ull;
            int used = 0;
            bool fin = false;
#pragma unroll
            for (int i = 0; i < DEPTH; ++i) {
              if (fin || used < i || i >= depth || jp - i < 0) continue;
              const unsigned long long fl = (w[i] >> 46) & 3ull;
              if ((w[i] & 0xFFFF000000000000ull) != etag || fl == 0) continue;  // not published yet
              excl += (unsigned)w[i];  // values are below 2^32
              used = i + 1;
              if (fl == RS_FLAG_PRE) fin = true;
            }
            jp -= used;
            if (fin || jp < 0) break;
            if (used == 0 && ++spins > spin_limit) {
              gb_set_error(st, GB_ERR_TIMEOUT, KID_RADIX, tile);
              break;
            }
          }
          *(volatile unsigned long long*)(status + (size_t)tile * radix + d) =
              etag | (RS_FLAG_PRE << 46) | (unsigned long long)(excl + tots[j]);
        }
        gpos[d] = gofs[d] + excl - bstart[d];  // modulo 2^32: slot + gpos < n < 2^32
      }
    }
  }
  __syncthreads();
  // ---- write runs: consecutive threads write consecutive slots of a digit's run
  for (int i = tid; i < (FULL ? TILE : cnt); i += NT) {
    const unsigned long long k = sk[i];
    const unsigned gp = gpos[digit(k)] + (unsigned)i;
    kout[gp] = k;
    vout[gp] = sv[i];
  }
}

// NT threads, IT keys per thread; digits of at most MAXB bits; n < 2^32.
template <int NT, int IT, int MAXB>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : (IT <= 12 ? 4 : 3))
k_rs_pass(const unsigned long long* __restrict__ kin, const unsigned* __restrict__ vin,
          unsigned long long* __restrict__ kout, unsigned* __restrict__ vout, long long n, int shift, int dbits,
          const unsigned* __restrict__ gofs, unsigned long long* status, unsigned long long epoch,
          long long* counter, DStatus* st, int spin_limit, int bulk) {
  constexpr int TILE = NT * IT;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int radix = 1 << dbits;
  const RsDigit digit(shift, (unsigned)radix - 1u);
  unsigned long long* sk = reinterpret_cast<unsigned long long*>(smraw);
  unsigned* sv = reinterpret_cast<unsigned*>(sk + TILE);
  unsigned short* wh = reinterpret_cast<unsigned short*>(sv + TILE);  // [NW][radix]
  unsigned* bstart = reinterpret_cast<unsigned*>(wh + NW * radix);
  unsigned* gpos = bstart + radix;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(gpos + radix);
  long long* stile = reinterpret_cast<long long*>(mbar + 1);
  long long* tmp = stile + 1;  // [33]
  unsigned* mbuf = reinterpret_cast<unsigned*>(tmp + 33);  // [NW][radix] lane masks (radix <= RS_AO_RADIX)
  const int tid = threadIdx.x;
  const long long ntile = (n + TILE - 1) / TILE;
  const unsigned mb = rs_smem(mbar);

  if (tid == 0) {
    const long long t = (long long)atomicAdd((unsigned long long*)counter, 1ull);
    *stile = t;
    if (bulk && t < ntile) {
      const long long tb = t * TILE;
      const int cb = (int)min((long long)TILE, n - tb) & ~3;  // bulk part: whole 16-byte groups
      rs_mbar_init(mb);
      rs_mbar_expect(mb, (unsigned)cb * 12u);
      if (cb > 0) {
        rs_bulk_load(rs_smem(sk), kin + tb, (unsigned)cb * 8u, mb);
        rs_bulk_load(rs_smem(sv), vin + tb, (unsigned)cb * 4u, mb);
      }
    }
  }
  for (int i = tid; i < NW * radix / 2; i += NT) reinterpret_cast<unsigned*>(wh)[i] = 0u;
  if (radix <= RS_AO_RADIX)
    for (int i = tid; i < NW * radix; i += NT) mbuf[i] = 0u;
  __syncthreads();
  const long long tile = *stile;
  if (tile >= ntile) return;
  const long long tb = tile * TILE;
  const int cnt = (int)min((long long)TILE, n - tb);
  if (bulk) {
    for (int i = (cnt & ~3) + tid; i < cnt; i += NT) {
      sk[i] = kin[tb + i];
      sv[i] = vin[tb + i];
    }
    const bool ok = rs_mbar_wait(mb, spin_limit);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) gb_set_error(st, GB_ERR_TIMEOUT, KID_RADIX_COPY, tile);
      rs_mbar_wait(mb, spin_limit);  // let copies in flight land before the CTA exits
      return;
    }
  } else {
    for (int i = tid; i < cnt; i += NT) {
      sk[i] = kin[tb + i];
      sv[i] = vin[tb + i];
    }
    __syncthreads();
  }

  if (cnt == TILE)
    rs_tile<NT, IT, MAXB, true>(sk, sv, wh, bstart, gpos, tmp, mbuf, digit, radix, cnt, tile, ntile, gofs, status, epoch, st,
                            spin_limit, kout, vout);
  else
    rs_tile<NT, IT, MAXB, false>(sk, sv, wh, bstart, gpos, tmp, mbuf, digit, radix, cnt, tile, ntile, gofs, status, epoch, st,
                             spin_limit, kout, vout);
}

__global__ void k_rs_zero(unsigned* p, int n, long long* ctrs, int nc) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0;
  if (threadIdx.x < nc) ctrs[threadIdx.x] = 0;
}

// ---------------------------------------------------------------- host side
namespace {

struct RsState {
  unsigned* ghist = nullptr;
  unsigned long long* status = nullptr;
  size_t status_words = 0;
  long long* ctrs = nullptr;
  unsigned long long epoch = 0;
};

using PassFn = void (*)(const unsigned long long*, const unsigned*, unsigned long long*, unsigned*, long long,
                        int, int, const unsigned*, unsigned long long*, unsigned long long, long long*, DStatus*,
                        int, int);

struct RsKernel {
  int nt, it;
  PassFn fn[4];  // digits of at most 6, 7, 8, 10 bits
  int tile() const { return nt * it; }
};
const RsKernel kKernels[] = {
    {256, 12, {k_rs_pass<256, 12, 6>, k_rs_pass<256, 12, 7>, k_rs_pass<256, 12, 8>, k_rs_pass<256, 12, 10>}},
    {256, 16, {k_rs_pass<256, 16, 6>, k_rs_pass<256, 16, 7>, k_rs_pass<256, 16, 8>, k_rs_pass<256, 16, 10>}},
    {256, 20, {k_rs_pass<256, 20, 6>, k_rs_pass<256, 20, 7>, k_rs_pass<256, 20, 8>, k_rs_pass<256, 20, 10>}},
    {512, 12, {k_rs_pass<512, 12, 6>, k_rs_pass<512, 12, 7>, k_rs_pass<512, 12, 8>, k_rs_pass<512, 12, 10>}},
    {512, 16, {k_rs_pass<512, 16, 6>, k_rs_pass<512, 16, 7>, k_rs_pass<512, 16, 8>, k_rs_pass<512, 16, 10>}},
};

// the kernel whose tile holds `tile` keys
const RsKernel* kernel_for(int tile) {
  for (const RsKernel& k : kKernels)
    if (k.tile() == tile) return &k;
  return nullptr;
}

PassFn pass_fn(const RsKernel* K, int dbits) { return K->fn[dbits <= 6 ? 0 : dbits == 7 ? 1 : dbits == 8 ? 2 : 3]; }

RsState* state_of(GbCtx& c) {
  if (!c.rs) c.rs = new RsState();
  return static_cast<RsState*>(c.rs);
}

void make_plan(int bits, int passes, RsPlan& p) {
  p.np = passes;
  int sh = 0, off = 0;
  for (int i = 0; i < passes; ++i) {
    const int w = bits / passes + (i < bits % passes ? 1 : 0);
    p.shift[i] = sh;
    p.bits[i] = w;
    p.off[i] = off;
    sh += w;
    off += 1 << w;
  }
}

// Groups the passes' counters for k_rs_hist: each pass alone, then adjacent
// pairs joined left to right while the joint index stays within
// RS_JOINT_BITS and all counters fit in RS_HIST_WORDS.
void make_hist_plan(const RsPlan& p, RsHistPlan& h) {
  int words = 0;
  for (int i = 0; i < p.np; ++i) words += 1 << p.bits[i];
  h.ng = 0;
  int off = 0;
  for (int i = 0; i < p.np;) {
    const int g = h.ng++;
    h.gshift[g] = p.shift[i];
    h.gp[g] = i;
    const int jb = i + 1 < p.np ? p.bits[i] + p.bits[i + 1] : 99;
    const int extra = jb <= RS_JOINT_BITS ? (1 << jb) - (1 << p.bits[i]) - (1 << p.bits[i + 1]) : 0;
    if (jb <= RS_JOINT_BITS && words + extra <= RS_HIST_WORDS) {
      words += extra;
      h.gbits[g] = jb;
      h.gn[g] = 2;
      i += 2;
    } else {
      h.gbits[g] = p.bits[i];
      h.gn[g] = 1;
      i += 1;
    }
    h.goff[g] = off;
    off += 1 << h.gbits[g];
  }
  h.words = off;
}

// process-wide table of tuned configurations: (device, bits, log2 n) -> (passes, tile keys)
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tuned;

int log2_bucket(long long n) {
  int b = 0;
  while ((1ll << (b + 1)) <= n) ++b;
  return b;
}

}  // namespace

void gb_radix_free(GbCtx& c) {
  RsState* s = static_cast<RsState*>(c.rs);
  if (!s) return;
  cudaFree(s->ghist);
  cudaFree(s->status);
  cudaFree(s->ctrs);
  delete s;
  c.rs = nullptr;
}

// Default configuration for a sort of `bits` significant bits: the fewest
// passes with digits of at most 7 bits (radix <= RS_AO_RADIX ranks through
// shared lane masks), one more when that makes the count even (it moves as
// many bytes as the final copy it saves), tiles of 8192 keys.
// The plan gb_radix_sort_pairs takes for `bits` significant bits and n keys
// on `device`: the tuned one for that bit width and size class, else the
// default.
extern "C" int gb_radix_plan(int device, int bits, long long n, int* passes, int* tile) {
  if (!passes || !tile || bits < 1 || bits > 64 || n < 1) return GB_ERR_ARG;
  int tp = 0, ti = 0;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto f = g_tuned.find(std::make_tuple(device, bits, log2_bucket(n)));
    if (f != g_tuned.end()) {
      tp = f->second.first;
      ti = f->second.second;
    }
  }
  if (!tp) gb_radix_default(bits, &tp, &ti);
  *passes = std::min(tp, bits);
  *tile = ti;
  return GB_OK;
}

void gb_radix_default(int bits, int* passes, int* tile) {
  int p = (bits + 6) / 7;
  if ((p & 1) && p + 1 <= bits) ++p;
  *passes = std::max(1, p);
  *tile = 8192;
}

int gb_radix_sort_pairs(GbCtx& c, unsigned long long* keys, unsigned* vals, long long n, int bits,
                        unsigned long long* keys_tmp, unsigned* vals_tmp, int passes, int tile) {
  if (n <= 1) return 0;
  if (n >= (1ll << 32)) return -1;  // slots and values are 32-bit
  if (bits < 1) bits = 1;
  if (bits > 64) bits = 64;
  if (passes <= 0 || tile <= 0) {
    int tp = 0, ti = 0;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto f = g_tuned.find(std::make_tuple(c.device, bits, log2_bucket(n)));
      if (f != g_tuned.end()) {
        tp = f->second.first;
        ti = f->second.second;
      }
    }
    if (!tp) gb_radix_default(bits, &tp, &ti);
    if (passes <= 0) passes = tp;
    if (tile <= 0) tile = ti;
  }
  if (passes > bits) passes = bits;
  if (passes > RS_MAXPASS || (bits + passes - 1) / passes > 10) return -1;  // digits of 1..10 bits only
  const RsKernel* K = kernel_for(tile);
  if (!K) return -1;
  RsPlan plan;
  make_plan(bits, passes, plan);
  const int maxradix = 1 << plan.bits[0];
  const int TILE = K->tile();
  const long long ntile = (n + TILE - 1) / TILE;
  RsState* S = state_of(c);
  if (!S->ghist) {
    if (cudaMalloc(&S->ghist, RS_HIST_SLOTS * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&S->ctrs, RS_MAXPASS * sizeof(long long)) != cudaSuccess)
      return -2;
  }
  const size_t want = (size_t)(ntile + 1024) * maxradix;
  if (S->status_words < want) {
    if (S->status) cudaFree(S->status);
    S->status = nullptr;
    S->status_words = 0;
    if (cudaMalloc(&S->status, want * 8) != cudaSuccess) return -2;
    cudaMemsetAsync(S->status, 0, want * 8, c.stream);
    S->status_words = want;
  }
  // passes of different digit widths lay shared memory out differently (the
  // lane masks exist only for radix <= RS_AO_RADIX): size for the largest
  size_t smem = 0;
  for (int p = 0; p < passes; ++p) smem = std::max(smem, rs_smem_bytes(K->nt, K->it, 1 << plan.bits[p]));
  for (int i = 0; i < 4; ++i) {
    cudaFuncSetAttribute((const void*)K->fn[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute((const void*)K->fn[i], cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  }
  const bool al = !(((uintptr_t)keys | (uintptr_t)vals | (uintptr_t)keys_tmp | (uintptr_t)vals_tmp) & 15u);
  k_rs_zero<<<1, 1024, 0, c.stream>>>(S->ghist, RS_HIST_SLOTS, S->ctrs, RS_MAXPASS);
  RsHistPlan hplan;
  make_hist_plan(plan, hplan);
  {
    const size_t hsm = (size_t)hplan.words * sizeof(unsigned);
    const long long want_blocks = (n / RS_HIST_KPT + 1023) / 1024;
    const unsigned hb = (unsigned)std::max(1ll, std::min<long long>(c.nsm, want_blocks));
    const void* hf = !((uintptr_t)keys & 15u) ? (const void*)k_rs_hist<true> : (const void*)k_rs_hist<false>;
    cudaFuncSetAttribute(hf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
    if (!((uintptr_t)keys & 15u))
      k_rs_hist<true><<<hb, 1024, hsm, c.stream>>>(keys, n, plan, hplan, S->ghist);
    else
      k_rs_hist<false><<<hb, 1024, hsm, c.stream>>>(keys, n, plan, hplan, S->ghist);
  }
  k_rs_hist_scan<<<passes, 1024, 0, c.stream>>>(S->ghist, plan);
  c.launches += 3;
  unsigned long long* ka = keys;
  unsigned* va = vals;
  unsigned long long* kb = keys_tmp;
  unsigned* vb = vals_tmp;
  for (int p = 0; p < passes; ++p) {
    S->epoch = (S->epoch + 1) & 0xFFFFull;
    if (S->epoch == 0) {
      cudaMemsetAsync(S->status, 0, S->status_words * 8, c.stream);
      S->epoch = 1;
    }
    pass_fn(K, plan.bits[p])<<<(unsigned)ntile, K->nt, smem, c.stream>>>(ka, va, kb, vb, n, plan.shift[p],
                                                                              plan.bits[p],
                                                          S->ghist + plan.off[p], S->status, S->epoch,
                                                          S->ctrs + p, c.st, RS_SPIN_LIMIT, al ? 1 : 0);
    ++c.launches;
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    cudaMemcpyAsync(keys, ka, (size_t)n * 8, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream);
  }
  return passes;
}

// Time each candidate (passes, tile keys) on a copy of the caller's
// keys and remember the fastest for this device, bit width and size class
// (powers of two of n); later sorts in that class use it.
int gb_radix_tune(GbCtx& c, const unsigned long long* keys, const unsigned* vals, long long n, int bits,
                      int* best_passes, int* best_tile, float* best_ms) {
  if (n <= 1 || bits < 1 || bits > 64) return -1;
  unsigned long long *k = nullptr, *kt = nullptr;
  unsigned *v = nullptr, *vt = nullptr;
  if (cudaMalloc(&k, (size_t)n * 8) != cudaSuccess || cudaMalloc(&kt, (size_t)n * 8) != cudaSuccess ||
      cudaMalloc(&v, (size_t)n * 4) != cudaSuccess || cudaMalloc(&vt, (size_t)n * 4) != cudaSuccess) {
    cudaFree(k);
    cudaFree(kt);
    cudaFree(v);
    return -2;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int bp = 0, bi = 0;
  float bms = 1e30f;
  const int pmin = std::max(1, (bits + 9) / 10), pmax = std::min(bits, pmin + 3);
  for (int p = pmin; p <= pmax; ++p) {
    for (const RsKernel& K : kKernels) {
      float tot = 0.f;
      for (int rep = 0; rep < 3; ++rep) {
        cudaMemcpyAsync(k, keys, (size_t)n * 8, cudaMemcpyDeviceToDevice, c.stream);
        cudaMemcpyAsync(v, vals, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream);
        cudaEventRecord(e0, c.stream);
        const int r = gb_radix_sort_pairs(c, k, v, n, bits, kt, vt, p, K.tile());
        cudaEventRecord(e1, c.stream);
        cudaEventSynchronize(e1);
        if (r < 0) {
          tot = 1e30f;
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) tot += ms;  // the first run warms up
      }
      if (tot / 2 < bms) {
        bms = tot / 2;
        bp = p;
        bi = K.tile();
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(k);
  cudaFree(kt);
  cudaFree(v);
  cudaFree(vt);
  if (!bp) return -1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[std::make_tuple(c.device, bits, log2_bucket(n))] = {bp, bi};
  }
  if (best_passes) *best_passes = bp;
  if (best_tile) *best_tile = bi;
  if (best_ms) *best_ms = bms;
  return 0;
}

void gb_radix_forget_tuning() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned.clear();
}

// Diagnostics for the bounded look-back: one CTA is handed tile 1 of a
// two-tile pass, so it waits for a tile-0 status word that nothing ever
// publishes.  After spin_limit polls it must flag GB_ERR_TIMEOUT and finish.
__global__ void k_rs_set_counter(long long* c, long long v) { *c = v; }
int gb_radix_lookback_timeout_probe(GbCtx& c, int spin_limit) {
  constexpr int NT = 256, IT = 16, TILE = NT * IT;
  const long long n = 2 * TILE;
  unsigned long long *k = nullptr, *k2 = nullptr, *status = nullptr;
  unsigned *v = nullptr, *v2 = nullptr, *gofs = nullptr;
  long long* ctr = nullptr;
  cudaMalloc(&k, n * 8); cudaMalloc(&k2, n * 8); cudaMalloc(&v, n * 4); cudaMalloc(&v2, n * 4);
  cudaMalloc(&status, 2 * 256 * 8); cudaMalloc(&gofs, 256 * 4); cudaMalloc(&ctr, 8);
  cudaMemsetAsync(k, 0, n * 8, c.stream);
  cudaMemsetAsync(v, 0, n * 4, c.stream);
  cudaMemsetAsync(status, 0, 2 * 256 * 8, c.stream);
  cudaMemsetAsync(gofs, 0, 256 * 4, c.stream);
  k_rs_set_counter<<<1, 1, 0, c.stream>>>(ctr, 1);
  const size_t smem = rs_smem_bytes(NT, IT, 256);
  cudaFuncSetAttribute((const void*)k_rs_pass<NT, IT, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_rs_pass<NT, IT, 8><<<1, NT, smem, c.stream>>>(k, v, k2, v2, n, 0, 8, gofs, status, 7, ctr, c.st, spin_limit,
                                                   1);
  const cudaError_t e = cudaStreamSynchronize(c.stream);
  cudaFree(k); cudaFree(k2); cudaFree(v); cudaFree(v2); cudaFree(status); cudaFree(gofs); cudaFree(ctr);
  return e == cudaSuccess ? 0 : -1;
}
