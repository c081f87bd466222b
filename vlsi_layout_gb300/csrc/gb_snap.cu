// gb_snap.cu -- SNAP layer streams on the device: the box codec of
// box_codec.f90 (CompressBoxesUsingCodec :616-698, DecompressBoxesUsingCodec
// :446-525) over 65536-box chunks, the Snappy raw format that
// snappy_api.cpp:9-37 applies to each chunk's codec bytes, and the .snap file
// of serialization.f90:15-130 (SaveCompressedStreamToDisk /
// RestoreCompressedStreamFromDisk).
//
// Encoding, per chunk (one 1024-thread CTA):
//   * widths, then heights of the non-square boxes, go into an open-addressing
//     table (16384 slots in shared memory; a chunk with more than 8192
//     distinct values is redone with a 131072-slot table in global memory)
//     that keeps each value's first position; a bitmap of first positions
//     with prefix popcounts gives each value its 1-based order of first
//     appearance, the codec's dictionary index, stored per box;
//   * boxes are then taken in order, 1024 at a time: a box's record (infobyte,
//     zigzag varint anchor deltas, the width / height as a varint when new or
//     an int16 index when seen before) depends only on the previous box, the
//     previous non-square box (a block scan) and the two ranks, and lands at
//     the exclusive sum of the record sizes.  One launch sizes the chunks, a
//     second writes them.
// Snappy: each 65536-byte fragment of a chunk's codec bytes is compressed by
// one warp, 32 positions at a time: a position's candidate is the latest
// earlier position with the same 11-bit hash of its 4 bytes (warp match for
// the batch, a 2048-slot table across batches); the greedy parse jumps to
// the next verified candidate, extends the match 32 bytes per step and, when
// it is at least 8 bytes long, emits Snappy literal / copy elements.  Fragments are concatenated behind the
// chunk's length preamble.  Decoding takes one warp per chunk through the
// elements (all element forms of the format are accepted), with the last
// 32 KB of output in a shared-memory ring for the copies.
// Decoding the codec: one CTA per chunk finds the record boundaries (seven
// warps compute, per 4 KB window, the lengths of the next four records from
// every byte; one thread walks the chain four records per load, overlapped
// with the next window's computation), then one CTA per chunk parses the
// records 1024 at a time, rebuilds the anchors and dictionary indices with
// block scans and gathers widths and heights from per-chunk dictionaries.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gbool.h"
#include "gb_internal.h"

#define SN_CHUNK 65536  // boxes per chunk (box_codec.f90:227)
#define SN_FRAG 65536   // Snappy fragment (bytes)
#define SN_FCAP (SN_FRAG + SN_FRAG / 6 + 64)
#define SN_T 1024       // threads of the per-chunk CTAs
#define SN_REC_MAX 31   // longest record of a valid box (1 + 5 + 5 + 10 + 10)
#define SN_WPAD 64      // look-ahead behind the window
#define SN_MIN_MATCH 8  // shortest copy the compressor emits
#define SN_CODEC_VERSION 1
#define SN_LAYER_STATE_PNUM 4
#define KID_SNAP_ENC 60
#define KID_SNAP_BOUNDS 61
#define KID_SNAP_DEC 62
#define KID_SNAPPY_C 63
#define KID_SNAPPY_D 64

namespace {

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ unsigned sn_zigzag(int v) {  // box_codec.f90:334-349 (fits 32 bits)
  return v < 0 ? (unsigned)(-(long long)v * 2 - 1) : (unsigned)v * 2u;
}
__device__ __forceinline__ int sn_unzigzag(unsigned long long v) {  // box_codec.f90:351-356
  return (int)(unsigned)((v >> 1) ^ (0ull - (v & 1ull)));
}
__host__ __device__ __forceinline__ int sn_vlen(unsigned long long v) {
  int n = 1;
  while (v >= 128ull) {
    v >>= 7;
    ++n;
  }
  return n;
}
__device__ __forceinline__ unsigned char* sn_put_varint(unsigned char* o, unsigned long long v) {
  while (v >= 128ull) {
    *o++ = (unsigned char)(v | 128ull);
    v >>= 7;
  }
  *o++ = (unsigned char)v;
  return o;
}
// varint at p (at most 10 bytes); *k receives its length, 0 when malformed
__device__ __forceinline__ unsigned long long sn_get_varint(const unsigned char* p, int* k) {
  unsigned long long r = 0;
  for (int i = 0; i < 10; ++i) {
    const unsigned b = p[i];
    r |= (unsigned long long)(b & 127u) << (7 * i);
    if (!(b & 128u)) {
      *k = i + 1;
      return r;
    }
  }
  *k = 0;
  return 0;
}

// ---------------------------------------------------------------- block scans
struct SumS {
  unsigned a;
};
struct LastS {  // last valid value (has = 0: none)
  int has, val;
};
struct Sum4 {
  unsigned x, y, nw, nh;
};
struct Last2 {
  int w, h;  // 0 = none
};
__device__ __forceinline__ SumS op(SumS p, SumS q) { return {p.a + q.a}; }
__device__ __forceinline__ LastS op(LastS p, LastS q) { return q.has ? q : p; }
__device__ __forceinline__ Sum4 op(Sum4 p, Sum4 q) { return {p.x + q.x, p.y + q.y, p.nw + q.nw, p.nh + q.nh}; }
__device__ __forceinline__ Last2 op(Last2 p, Last2 q) { return {q.w ? q.w : p.w, q.h ? q.h : p.h}; }
__device__ __forceinline__ SumS shup(SumS v, int d) { return {__shfl_up_sync(0xffffffffu, v.a, d)}; }
__device__ __forceinline__ LastS shup(LastS v, int d) {
  return {__shfl_up_sync(0xffffffffu, v.has, d), __shfl_up_sync(0xffffffffu, v.val, d)};
}
__device__ __forceinline__ Sum4 shup(Sum4 v, int d) {
  return {__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
          __shfl_up_sync(0xffffffffu, v.nw, d), __shfl_up_sync(0xffffffffu, v.nh, d)};
}
__device__ __forceinline__ Last2 shup(Last2 v, int d) {
  return {__shfl_up_sync(0xffffffffu, v.w, d), __shfl_up_sync(0xffffffffu, v.h, d)};
}

// Exclusive block scan (all threads of the block call it); buf holds 32
// entries and must not be reused by the next call (callers alternate two).
// *tot receives the block total.
template <class T>
__device__ __forceinline__ T block_excl(T x, T ident, T* buf, T* tot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T inc = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T o = shup(inc, d);
    if (lane >= d) inc = op(o, inc);
  }
  if (lane == 31) buf[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    T v = lane < nw ? buf[lane] : ident;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T o = shup(v, d);
      if (lane >= d) v = op(o, v);
    }
    if (lane < nw) buf[lane] = v;
  }
  __syncthreads();
  T ex = shup(inc, 1);
  if (lane == 0) ex = ident;
  *tot = buf[nw - 1];
  return wid ? op(buf[wid - 1], ex) : ex;
}

// ---------------------------------------------------------------- encoder: dictionary ranks
// Open-addressing table of one chunk: slot = (first position << 32) | value,
// empty = all ones (positions are below 65536, so an occupied slot never has
// an all-ones high word).  Inserting an existing value lowers its position
// with atomicMin on the whole word, which keeps the value.
#define SN_EMPTY 0xffffffffffffffffull
#define SN_STAB_SLOTS 16384  // shared table: at most 8192 distinct values
#define SN_GTAB_SLOTS 131072 // global table (a chunk has at most 65536 values)

__device__ __forceinline__ unsigned sn_slot(int v, unsigned mask) { return ((unsigned)v * 0x9E3779B1u >> 15) & mask; }

// inserts (v, j); false when the table holds `limit` values already
__device__ __forceinline__ bool tab_insert(unsigned long long* tab, unsigned mask, int v, unsigned j,
                                           unsigned* ndist, unsigned limit) {
  const unsigned long long mine = ((unsigned long long)j << 32) | (unsigned)v;
  unsigned s = sn_slot(v, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    unsigned long long cur = *(volatile unsigned long long*)&tab[s];
    if (cur == SN_EMPTY) {
      if (*(volatile unsigned*)ndist >= limit) return false;
      cur = atomicCAS(&tab[s], SN_EMPTY, mine);
      if (cur == SN_EMPTY) {
        atomicAdd(ndist, 1u);
        return true;
      }
    }
    if ((unsigned)cur == (unsigned)v) {
      if ((unsigned)(cur >> 32) > j) atomicMin(&tab[s], mine);
      return true;
    }
    s = (s + 1u) & mask;
  }
  return false;
}

// first position of v (the value must be in the table)
__device__ __forceinline__ unsigned tab_first(const unsigned long long* tab, unsigned mask, int v) {
  unsigned s = sn_slot(v, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const unsigned long long cur = *(const volatile unsigned long long*)&tab[s];
    if (cur == SN_EMPTY) break;
    if ((unsigned)cur == (unsigned)v) return (unsigned)(cur >> 32);
    s = (s + 1u) & mask;
  }
  return 0xffffffffu;
}

// 1-based order of first appearance of the value first seen at position p
__device__ __forceinline__ unsigned sn_rank(const unsigned* bits, const unsigned* pre, unsigned p) {
  return pre[p >> 5] + __popc(bits[p >> 5] & ((1u << (p & 31)) - 1u)) + 1u;
}

// Dictionary ranks of one chunk per CTA: ranks[b] (widths) and ranks[n + b]
// (heights of non-square boxes) = order of first appearance | first << 31.
// The width table is built and read, then the height table in the same
// storage.  GT: 131072-slot tables in global memory for the chunks in list
// (one table per CTA), else 16384-slot shared tables (chunk = block index);
// a chunk with more values than a shared table holds goes to ovf_list.
template <bool GT>
__global__ void __launch_bounds__(SN_T, 1)
k_enc_rank(const int4* __restrict__ boxes, long long n, const int* __restrict__ list, int nlist,
           unsigned long long* gtab, unsigned* __restrict__ ranks, int* ovf_list, int* ovf_count, DStatus* st) {
  extern __shared__ __align__(16) unsigned char sm[];
  constexpr unsigned SLOTS = GT ? SN_GTAB_SLOTS : SN_STAB_SLOTS;
  constexpr unsigned MASK = SLOTS - 1u;
  constexpr unsigned LIMIT = GT ? SLOTS : SLOTS / 2;
  unsigned char* q = sm;
  unsigned long long* tab;
  if (GT) {
    tab = gtab + (size_t)blockIdx.x * SLOTS;
  } else {
    tab = (unsigned long long*)q;
    q += SLOTS * 8;
  }
  unsigned* bits = (unsigned*)q;  // [2048] first-position bitmap
  unsigned* pre = bits + 2048;    // [2048] exclusive popcounts
  int* wsum = (int*)(pre + 2048); // [32]
  unsigned* flags = (unsigned*)(wsum + 32);  // distinct values, overflow
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const long long nchunks = (n + SN_CHUNK - 1) / SN_CHUNK;
  const long long nitems = GT ? nlist : nchunks;
  for (long long li = blockIdx.x; li < nitems; li += gridDim.x) {
    const long long c = GT ? list[li] : li;
    const long long b0 = c * SN_CHUNK;
    const int nb = (int)min((long long)SN_CHUNK, n - b0);
    bool ovf = false;
    for (int which = 0; which < 2 && !ovf; ++which) {
      for (unsigned i = t; i < SLOTS; i += SN_T) tab[i] = SN_EMPTY;
      for (int i = t; i < 2048; i += SN_T) bits[i] = 0;
      if (t < 2) flags[t] = 0;
      __syncthreads();
      for (int j = t; j < nb; j += SN_T) {
        const int4 b = boxes[b0 + j];
        const int w = (int)((unsigned)b.z - (unsigned)b.x), h = (int)((unsigned)b.w - (unsigned)b.y);
        if (which && w == h) continue;
        if (!tab_insert(tab, MASK, which ? h : w, (unsigned)j, &flags[0], LIMIT)) {
          flags[1] = 1;
          break;
        }
      }
      __syncthreads();
      ovf = *(volatile unsigned*)&flags[1] != 0;
      if (ovf) break;  // uniform
      for (unsigned i = t; i < SLOTS; i += SN_T) {
        const unsigned long long cur = *(volatile unsigned long long*)&tab[i];
        if (cur != SN_EMPTY) {
          const unsigned p = (unsigned)(cur >> 32);
          atomicOr(&bits[p >> 5], 1u << (p & 31));
        }
      }
      __syncthreads();
      {  // exclusive popcount prefix, two words per thread
        const int pc = __popc(bits[2 * t]) + __popc(bits[2 * t + 1]);
        int inc = pc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int o = __shfl_up_sync(0xffffffffu, inc, d);
          if (lane >= d) inc += o;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
          int v = wsum[lane];
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += o;
          }
          wsum[lane] = v;
        }
        __syncthreads();
        const int ex = inc - pc + (wid ? wsum[wid - 1] : 0);
        pre[2 * t] = (unsigned)ex;
        pre[2 * t + 1] = (unsigned)ex + __popc(bits[2 * t]);
      }
      __syncthreads();
      unsigned* out = ranks + (which ? n : 0) + b0;
      for (int j = t; j < nb; j += SN_T) {
        const int4 b = boxes[b0 + j];
        const int w = (int)((unsigned)b.z - (unsigned)b.x), h = (int)((unsigned)b.w - (unsigned)b.y);
        if (which && w == h) continue;
        const unsigned p = tab_first(tab, MASK, which ? h : w);
        if (p >= SN_CHUNK) {
          gb_set_error(st, GB_ERR_INTERNAL, KID_SNAP_ENC, b0 + j);
          continue;
        }
        out[j] = sn_rank(bits, pre, p) | ((p == (unsigned)j) ? 0x80000000u : 0u);
      }
      __syncthreads();
    }
    if (ovf && t == 0) {
      if (GT)
        gb_set_error(st, GB_ERR_INTERNAL, KID_SNAP_ENC, c);
      else
        ovf_list[atomicAdd(ovf_count, 1)] = (int)c;
    }
    __syncthreads();
  }
}

// Codec records of one chunk per CTA from the ranks: WRITE emits the bytes
// at raw + raw_off[c], else raw_size[c] receives the chunk's byte count.
template <bool WRITE>
__global__ void __launch_bounds__(SN_T, 1)
k_enc_emit(const int4* __restrict__ boxes, long long n, const unsigned* __restrict__ ranks,
           long long* raw_size, const long long* __restrict__ raw_off, unsigned char* __restrict__ raw, DStatus* st) {
  __shared__ SumS bufS[2][32];
  __shared__ LastS bufL[2][32];
  const long long c = blockIdx.x;
  const int t = threadIdx.x;
  const long long b0 = c * SN_CHUNK;
  const int nb = (int)min((long long)SN_CHUNK, n - b0);
  unsigned long long cbytes = 0;  // bytes of the records so far
  LastS chl{0, 0};                // last non-square box's height so far
  unsigned char* out = WRITE ? raw + raw_off[c] : nullptr;
  for (int k = 0; k * SN_T < nb; ++k) {
    const int j = k * SN_T + t;
    const bool valid = j < nb;
    int4 b = make_int4(0, 0, 0, 0), pb = make_int4(0, 0, 0, 0);
    if (valid) {
      b = boxes[b0 + j];
      if (j) pb = boxes[b0 + j - 1];
    }
    const int w = (int)((unsigned)b.z - (unsigned)b.x), h = (int)((unsigned)b.w - (unsigned)b.y);
    const bool sq = w == h;
    LastS tl;
    LastS ph = block_excl(LastS{valid && !sq, h}, LastS{0, 0}, bufL[k & 1], &tl);
    ph = op(chl, ph);
    unsigned info = 0, size = 0, wr = 0, hr = 0;
    int dx = 0, dy = 0;
    if (valid) {
      const int pw = j ? (int)((unsigned)pb.z - (unsigned)pb.x) : 0;
      dx = (int)((unsigned)b.x - (unsigned)pb.x);  // the anchor cursor starts at 0 and follows x1
      dy = (int)((unsigned)b.y - (unsigned)pb.y);
      if (sq) info |= 16;
      if (dx) info |= 32;
      if (dy) info |= 64;
      const unsigned rw = ranks[b0 + j];
      wr = rw & 0x7fffffffu;
      if (j == 0 || w != pw) info |= (rw >> 31) ? 3u : 1u;
      if (!sq) {
        const unsigned rh = ranks[n + b0 + j];
        hr = rh & 0x7fffffffu;
        if (!ph.has || ph.val != h) info |= (rh >> 31) ? 12u : 4u;
      }
      size = 1;
      if (info & 32) size += sn_vlen(sn_zigzag(dx));
      if (info & 64) size += sn_vlen(sn_zigzag(dy));
      if (info & 1) size += (info & 2) ? sn_vlen((unsigned long long)(long long)w) : 2;
      if (info & 4) size += (info & 8) ? sn_vlen((unsigned long long)(long long)h) : 2;
    }
    SumS ts;
    const SumS ex = block_excl(SumS{size}, SumS{0}, bufS[k & 1], &ts);
    if (WRITE && valid) {
      unsigned char* o = out + cbytes + ex.a;
      *o++ = (unsigned char)info;
      if (info & 32) o = sn_put_varint(o, sn_zigzag(dx));
      if (info & 64) o = sn_put_varint(o, sn_zigzag(dy));
      if (info & 1) {
        if (info & 2) {
          o = sn_put_varint(o, (unsigned long long)(long long)w);
        } else {  // int16 index, little-endian (wraps above 32767 as the reference's int16 does)
          *o++ = (unsigned char)wr;
          *o++ = (unsigned char)(wr >> 8);
        }
      }
      if (info & 4) {
        if (info & 8) {
          o = sn_put_varint(o, (unsigned long long)(long long)h);
        } else {
          *o++ = (unsigned char)hr;
          *o++ = (unsigned char)(hr >> 8);
        }
      }
    }
    cbytes += ts.a;
    chl = op(chl, tl);
  }
  if (t == 0) {
    if (!WRITE)
      raw_size[c] = (long long)cbytes;
    else if ((long long)cbytes != raw_off[c + 1] - raw_off[c])
      gb_set_error(st, GB_ERR_INTERNAL, KID_SNAP_ENC, c);
  }
}

// ---------------------------------------------------------------- codec decoder
// One 256-thread CTA per chunk: rec[c * SN_CHUNK + r] = offset of record r in
// the chunk.  The chunk is taken in 4 KB windows.  For a window, warps 1..7
// load its bytes (and the look-ahead), mark the varint continuation bits
// with ballots, compute at every byte the length a record starting there
// would have (each varint's length is one find-first-zero in the continuation
// bits) and then, per byte, the lengths of the four records of the chain
// starting there (one word).  Meanwhile lane 0 of warp 0 walks the previous
// window's chain four records per shared-memory load.
#define SN_BT 256
#define SN_BWIN 4096
#define SN_BPAD 256  // lengths are needed up to three records (3 * 41 bytes) past the window
#define SN_BBUF (SN_BWIN + SN_BPAD + 64)
__device__ __forceinline__ int sn_vl(const unsigned* cont, int q) {  // varint length at q (0: longer than 10)
  const unsigned long long w = ((unsigned long long)cont[(q >> 5) + 1] << 32) | cont[q >> 5];
  const int k = __ffsll(~(w >> (q & 31)));  // first byte without the continuation bit, 1-based
  return k <= 10 ? k : 0;
}

// Branch-free: every field's varint length is looked up and selected by the
// infobyte's bits, so the lanes of a warp (at different bytes) do not diverge.
__device__ __forceinline__ int sn_rec_len_bits(const unsigned char* buf, const unsigned* cont, int b) {
  const unsigned info = buf[b];
  int l = 1;
  bool bad = false;
  int k = sn_vl(cont, b + l);
  bad |= (info & 32) && !k;
  l += (info & 32) ? k : 0;
  k = sn_vl(cont, b + l);
  bad |= (info & 64) && !k;
  l += (info & 64) ? k : 0;
  k = sn_vl(cont, b + l);
  bad |= (info & 3) == 3 && !k;
  l += (info & 1) ? ((info & 2) ? k : 2) : 0;
  k = sn_vl(cont, b + l);
  const bool hf = (info & 20) == 4;
  bad |= hf && (info & 8) && !k;
  l += hf ? ((info & 8) ? k : 2) : 0;
  return bad ? 0 : l;
}

__global__ void __launch_bounds__(SN_BT)
k_codec_bounds(const unsigned char* __restrict__ raw, const long long* __restrict__ raw_off,
               const long long* __restrict__ raw_len, long long n, long long nchunks, unsigned* __restrict__ rec,
               DStatus* st) {
  __shared__ unsigned char buf[SN_BBUF];
  __shared__ unsigned cont[SN_BBUF / 32 + 2];
  __shared__ unsigned char lenb[SN_BWIN + SN_BPAD];
  __shared__ unsigned quad[2][SN_BWIN];
  __shared__ int s_pos, s_r, s_bad, s_skip;  // s_pos: offset into the next window
  const int t = threadIdx.x, wid = t >> 5;
  const long long c = blockIdx.x;
  if (t == 0) {
    s_skip = *(volatile int*)&st->err;  // the Snappy layer was malformed: one read for the whole CTA
    s_pos = 0;
    s_r = 0;
    s_bad = 0;
  }
  __syncthreads();
  if (s_skip) return;
  const int nb = (int)min((long long)SN_CHUNK, n - c * SN_CHUNK);
  const long long L = raw_len[c];
  const unsigned char* base = raw + raw_off[c];
  unsigned* out = rec + c * SN_CHUNK;
  auto sync = [&](int bar, int nt) {
    if (bar)
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nt) : "memory");
    else
      __syncthreads();
  };
  // quads of window w into quad[w & 1]; run by threads [t0, t0 + nt) (whole warps), barrier id bar
  auto build = [&](long long w, int t0, int nt, int bar) {
    const long long ws = w * SN_BWIN;
    const int u = t - t0;
#pragma unroll 8
    for (int b = u; b < SN_BBUF; b += nt) buf[b] = ws + b < L ? base[ws + b] : 0;  // independent loads in flight
    sync(bar, nt);
    for (int b = u; b < SN_BBUF; b += nt) {
      const unsigned m = __ballot_sync(0xffffffffu, buf[b] & 128u);
      if ((b & 31) == 0) cont[b >> 5] = m;
    }
    if (u < 2) cont[SN_BBUF / 32 + u] = 0xffffffffu;  // past the buffer: a varint there is too long
    sync(bar, nt);
    for (int b = u; b < SN_BWIN + SN_BPAD; b += nt) lenb[b] = (unsigned char)sn_rec_len_bits(buf, cont, b);
    sync(bar, nt);
    unsigned* qd = quad[w & 1];
    for (int b = u; b < SN_BWIN; b += nt) {
      const unsigned l0 = lenb[b];
      const unsigned l1 = l0 ? lenb[b + l0] : 0u;
      const unsigned l2 = l1 ? lenb[b + l0 + l1] : 0u;
      const unsigned l3 = l2 ? lenb[b + l0 + l1 + l2] : 0u;
      qd[b] = l0 | (l1 << 8) | (l2 << 16) | (l3 << 24);
    }
  };
  const long long nwin = (L + SN_BWIN - 1) / SN_BWIN;
  if (nwin > 0) build(0, 0, SN_BT, 0);
  __syncthreads();
  for (long long w = 0;; ++w) {
    // every thread reads the walk's state before the barrier; lane 0 of warp 0 changes it only after
    const int done = (s_r >= nb || s_bad) ? 1 : (w >= nwin ? 2 : 0);
    __syncthreads();
    if (done) {
      if (done == 2 && t == 0) s_bad = 1;  // the stream ends before the chunk's last record
      break;
    }
    if (t == 0) {
      const unsigned ws = (unsigned)(w * SN_BWIN);
      const unsigned* qd = quad[w & 1];
      const int lim = (int)min((long long)SN_BWIN, L - (long long)ws);  // starts inside window and stream
      int pos = s_pos, r = s_r, bad = 0;
      while (r < nb && pos < SN_BWIN) {
        const unsigned q = qd[pos];
        const int l0 = q & 255u, l1 = (q >> 8) & 255u, l2 = (q >> 16) & 255u, l3 = q >> 24;
        const int p1 = pos + l0, p2 = p1 + l1, p3 = p2 + l2;
        if (l3 && p3 < lim && r + 4 <= nb) {  // four whole records (l3 != 0 implies l0..l2 != 0)
          out[r] = ws + pos;
          out[r + 1] = ws + p1;
          out[r + 2] = ws + p2;
          out[r + 3] = ws + p3;
          r += 4;
          pos = p3 + l3;
          continue;
        }
        if (pos >= lim || !l0) {  // the stream ends early, or a malformed record
          bad = 1;
          break;
        }
        out[r++] = ws + pos;
        pos = p1;
      }
      if (!bad && r >= nb && (long long)ws + pos > L) bad = 1;  // the last record runs past the stream
      s_pos = pos - SN_BWIN;
      s_r = r;
      s_bad = bad;
    } else if (wid > 0 && w + 1 < nwin) {
      build(w + 1, 32, SN_BT - 32, 1);
    }
    __syncthreads();
  }
  if (t == 0 && s_bad) gb_set_error(st, GB_ERR_CORRUPT, KID_SNAP_BOUNDS, c);
}

// One CTA per chunk: records -> boxes.  dict: per chunk 2 * SN_CHUNK ints.
__global__ void __launch_bounds__(SN_T, 1)
k_codec_decode(const unsigned char* __restrict__ raw, const long long* __restrict__ raw_off,
               const unsigned* __restrict__ rec, long long n, int* dict, int4* __restrict__ out, DStatus* st) {
  __shared__ Sum4 bufA[2][32];
  __shared__ Last2 bufB[2][32];
  __shared__ int s_skip;
  const long long c = blockIdx.x;
  const int t = threadIdx.x;
  if (t == 0) s_skip = *(volatile int*)&st->err;  // the boundaries (or the Snappy layer) were malformed
  __syncthreads();
  if (s_skip) return;
  const long long b0 = c * SN_CHUNK;
  const int nb = (int)min((long long)SN_CHUNK, n - b0);
  const unsigned char* base = raw + raw_off[c];
  int* dw = dict + c * 2 * SN_CHUNK;
  int* dh = dw + SN_CHUNK;
  Sum4 cA{0, 0, 0, 0};
  Last2 cB{0, 0};
  for (int k = 0; k * SN_T < nb; ++k) {
    const int j = k * SN_T + t;
    const bool valid = j < nb;
    unsigned info = 0;
    int dx = 0, dy = 0, wv = 0, hv = 0, wsel = 0, hsel = 0, bad = 0;
    if (valid) {
      const unsigned char* p = base + rec[b0 + j];
      info = p[0];
      int i = 1, kk;
      if (info & 32) {
        dx = sn_unzigzag(sn_get_varint(p + i, &kk));
        i += kk;
      }
      if (info & 64) {
        dy = sn_unzigzag(sn_get_varint(p + i, &kk));
        i += kk;
      }
      if (info & 1) {
        if (info & 2) {
          wv = (int)(unsigned)sn_get_varint(p + i, &kk);
          i += kk;
          wsel = 1;
        } else {
          wv = (short)(unsigned short)(p[i] | (p[i + 1] << 8));
          i += 2;
          wsel = 2;
        }
      }
      if (!(info & 16) && (info & 4)) {
        if (info & 8) {
          hv = (int)(unsigned)sn_get_varint(p + i, &kk);
          i += kk;
          hsel = 1;
        } else {
          hv = (short)(unsigned short)(p[i] | (p[i + 1] << 8));
          i += 2;
          hsel = 2;
        }
      }
    }
    Sum4 tA;
    Sum4 ea = block_excl(Sum4{(unsigned)dx, (unsigned)dy, wsel == 1 ? 1u : 0u, hsel == 1 ? 1u : 0u},
                         Sum4{0, 0, 0, 0}, bufA[k & 1], &tA);
    ea = op(cA, ea);
    int wself = 0, hself = 0;
    if (wsel == 1) {
      wself = (int)ea.nw + 1;
      dw[wself - 1] = wv;
    } else if (wsel == 2) {
      if (wv < 1 || wv > (int)ea.nw) bad = 1;
      wself = bad ? 0 : wv;
    }
    if (hsel == 1) {
      hself = (int)ea.nh + 1;
      dh[hself - 1] = hv;
    } else if (hsel == 2) {
      if (hv < 1 || hv > (int)ea.nh) bad = 1;
      hself = bad ? 0 : hv;
    }
    Last2 tB;
    Last2 eb = block_excl(Last2{wself, hself}, Last2{0, 0}, bufB[k & 1], &tB);
    eb = op(cB, eb);
    if (valid) {
      const int cw = wself ? wself : eb.w;
      const int x = (int)(ea.x + (unsigned)dx), y = (int)(ea.y + (unsigned)dy);
      int w = 0, h = 0;
      if (cw < 1)
        bad = 1;
      else
        w = dw[cw - 1];
      if (info & 16) {
        h = w;
      } else {
        const int ch = hself ? hself : eb.h;
        if (ch < 1)
          bad = 1;
        else
          h = dh[ch - 1];
      }
      if (bad) gb_set_error(st, GB_ERR_CORRUPT, KID_SNAP_DEC, b0 + j);
      out[b0 + j] = make_int4(x, y, (int)((unsigned)x + (unsigned)w), (int)((unsigned)y + (unsigned)h));
    }
    cA = op(cA, tA);
    cB = op(cB, tB);
  }
}

// ---------------------------------------------------------------- Snappy
__device__ __forceinline__ unsigned sn_ld32(const unsigned char* p) {
  return (unsigned)p[0] | ((unsigned)p[1] << 8) | ((unsigned)p[2] << 16) | ((unsigned)p[3] << 24);
}

// Writes one Snappy copy element of 4..64 bytes (lane 0 only); returns its size.
__device__ __forceinline__ int sn_copy_piece(unsigned char* o, unsigned off, int len, bool write) {
  if (len <= 11 && off < 2048u) {
    if (write) {
      o[0] = (unsigned char)(1u | ((unsigned)(len - 4) << 2) | ((off >> 8) << 5));
      o[1] = (unsigned char)off;
    }
    return 2;
  }
  if (write) {
    o[0] = (unsigned char)(2u | ((unsigned)(len - 1) << 2));
    o[1] = (unsigned char)off;
    o[2] = (unsigned char)(off >> 8);
  }
  return 3;
}

// One warp per fragment (8 per CTA).  fsrc / flen: the fragment's bytes in
// raw; the compressed elements go to fout + f * SN_FCAP, their count to flout.
__global__ void __launch_bounds__(256)
k_snappy_compress(const unsigned char* __restrict__ raw, const long long* __restrict__ fsrc,
                  const int* __restrict__ flen, long long nfrag, unsigned char* __restrict__ fout,
                  int* __restrict__ flout, DStatus* st) {
  extern __shared__ unsigned short table[];  // [8][2048]: latest position + 1 (positions with 4 bytes left are < 65533)
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long f = (long long)blockIdx.x * 8 + wid;
  if (f >= nfrag) return;
  unsigned short* tab = table + wid * 2048;
  for (int i = lane; i < 2048; i += 32) tab[i] = 0;
  __syncwarp();
  const unsigned char* src = raw + fsrc[f];
  const int fl = flen[f];
  unsigned char* out = fout + f * SN_FCAP;
  int o = 0, p = 0, lit = 0;
  for (int bb = 0; bb + 4 <= fl; bb += 32) {
    const int q = bb + lane;
    const bool has = q + 4 <= fl;
    const unsigned v = has ? sn_ld32(src + q) : 0u;
    const unsigned h = (v * 0x9E3779B1u) >> 21;
    const unsigned peers = __match_any_sync(0xffffffffu, has ? h : 0x10000u + lane);
    const unsigned lower = peers & ((1u << lane) - 1u);
    unsigned cand = 0;  // 1-based
    if (has) cand = lower ? (unsigned)(bb + 31 - __clz(lower)) + 1u : tab[h];
    __syncwarp();
    if (has && (peers >> lane) == 1u) tab[h] = (unsigned short)(q + 1);
    __syncwarp();
    // a candidate counts when its first 8 bytes match (shorter copies are not emitted)
    const bool has8 = q + SN_MIN_MATCH <= fl;
    const bool ok = has8 && cand && sn_ld32(src + cand - 1) == v && sn_ld32(src + cand + 3) == sn_ld32(src + q + 4);
    const unsigned okm = __ballot_sync(0xffffffffu, ok);
    while (p < bb + 32 && p + 4 <= fl) {
      const unsigned m = okm & (0xffffffffu << (p - bb));
      if (!m) {
        p = bb + 32;
        break;
      }
      const int ln = __ffs(m) - 1;
      p = bb + ln;
      const int qs = (int)__shfl_sync(0xffffffffu, cand, ln) - 1;
      int L = SN_MIN_MATCH;
      for (;;) {
        const int a = p + L + lane;
        const bool eq = a < fl && src[qs + L + lane] == src[a];
        const unsigned ne = __ballot_sync(0xffffffffu, !eq);
        if (ne) {
          L += __ffs(ne) - 1;
          break;
        }
        L += 32;
      }
      // pending literal
      if (p > lit) {
        const int len = p - lit;
        const unsigned mm = (unsigned)len - 1u;
        const int nb = mm < 60u ? 0 : mm < 256u ? 1 : 2;
        if (o + 1 + nb + len + 3 * ((L + 59) / 60) > SN_FCAP) {
          if (lane == 0) gb_set_error(st, GB_ERR_INTERNAL, KID_SNAPPY_C, f);
          if (lane == 0) flout[f] = 0;
          return;
        }
        if (lane == 0) {
          out[o] = (unsigned char)(nb ? (59 + nb) << 2 : mm << 2);
          for (int i = 0; i < nb; ++i) out[o + 1 + i] = (unsigned char)(mm >> (8 * i));
        }
#pragma unroll 4
        for (int i = lane; i < len; i += 32) out[o + 1 + nb + i] = src[lit + i];
        o += 1 + nb + len;
      }
      {
        const unsigned off = (unsigned)(p - qs);
        int rem = L;
        while (rem >= 68) {
          o += sn_copy_piece(out + o, off, 64, lane == 0);
          rem -= 64;
        }
        if (rem > 64) {
          o += sn_copy_piece(out + o, off, 60, lane == 0);
          rem -= 60;
        }
        o += sn_copy_piece(out + o, off, rem, lane == 0);
      }
      p += L;
      lit = p;
    }
  }
  if (fl > lit) {
    const int len = fl - lit;
    const unsigned mm = (unsigned)len - 1u;
    const int nb = mm < 60u ? 0 : mm < 256u ? 1 : 2;
    if (o + 1 + nb + len > SN_FCAP) {
      if (lane == 0) gb_set_error(st, GB_ERR_INTERNAL, KID_SNAPPY_C, f);
      if (lane == 0) flout[f] = 0;
      return;
    }
    if (lane == 0) {
      out[o] = (unsigned char)(nb ? (59 + nb) << 2 : mm << 2);
      for (int i = 0; i < nb; ++i) out[o + 1 + i] = (unsigned char)(mm >> (8 * i));
    }
#pragma unroll 4
    for (int i = lane; i < len; i += 32) out[o + 1 + nb + i] = src[lit + i];
    o += 1 + nb + len;
  }
  if (lane == 0) flout[f] = o;
}

// Chunk preambles and fragment copies into the final stream.  One CTA per
// fragment; fdst[f] is the fragment's destination, pre_at / pre_val the
// chunks' preamble positions and values.
__global__ void k_snappy_gather(const unsigned char* __restrict__ fout, const int* __restrict__ flout,
                                const long long* __restrict__ fdst, long long nfrag,
                                const long long* __restrict__ pre_at, const long long* __restrict__ pre_val,
                                long long nchunks, unsigned char* __restrict__ dst) {
  const long long f = blockIdx.x;
  if (f < nfrag) {
    const unsigned char* s = fout + f * SN_FCAP;
    unsigned char* d = dst + fdst[f];
    for (int i = threadIdx.x; i < flout[f]; i += blockDim.x) d[i] = s[i];
  }
  if (blockIdx.x == 0)
    for (long long c = threadIdx.x; c < nchunks; c += blockDim.x) sn_put_varint(dst + pre_at[c], (unsigned long long)pre_val[c]);
}

// One single-warp CTA per chunk: Snappy raw stream -> codec bytes.  The
// element tags are read from a 4 KB staging copy of the input, literals are
// copied with four loads in flight per lane, and copies whose source lies in
// the last 32 KB of output are read from a shared-memory ring of it (older
// sources from global memory).
#define SN_RING 32768
#define SN_STAGE 4096
__global__ void __launch_bounds__(32)
k_snappy_decompress(const unsigned char* __restrict__ in_all, const long long* __restrict__ in_off,
                    const long long* __restrict__ in_len, unsigned char* out_all, const long long* __restrict__ out_off,
                    const long long* __restrict__ out_len, long long nchunks, DStatus* st) {
  extern __shared__ __align__(16) unsigned char dsm[];
  unsigned char* ring = dsm;           // output byte x at ring[x % SN_RING] for the last SN_RING bytes
  unsigned char* stg = dsm + SN_RING;  // input bytes [sb, sb + SN_STAGE)
  const int lane = threadIdx.x;
  const long long c = blockIdx.x;
  if (c >= nchunks) return;
  const unsigned char* in = in_all + in_off[c];
  const long long len = in_len[c];
  unsigned char* out = out_all + out_off[c];
  const long long want = out_len[c];
  long long sb = -(long long)SN_STAGE - 8;
  auto stage = [&](long long p) {  // bytes p .. p + 7 staged
    if (p < sb || p + 8 > sb + SN_STAGE) {
      sb = p;
      __syncwarp();
#pragma unroll 16
      for (int i = lane; i < SN_STAGE; i += 32) stg[i] = sb + i < len ? in[sb + i] : 0;  // 16 loads in flight
      __syncwarp();
    }
  };
  int bad = 0;
  long long p = 0, o = 0;
  stage(0);
  {
    unsigned long long v = 0;
    int k = 0;
    for (int i = 0; i < 5 && i < len; ++i) {
      const unsigned b = stg[i];
      v |= (unsigned long long)(b & 127u) << (7 * i);
      if (!(b & 128u)) {
        k = i + 1;
        break;
      }
    }
    if (!k || (long long)v != want) bad = 1;
    p = k;
  }
  while (!bad && p < len) {
    stage(p);
    const unsigned tag = stg[p - sb];
    const unsigned char* tb = stg + (p - sb) + 1;  // up to 4 bytes after the tag
    ++p;
    const unsigned tt = tag & 3u;
    if (tt == 0) {
      long long m = tag >> 2;
      if (m >= 60) {
        const int nb = (int)m - 59;
        if (p + nb > len) {
          bad = 1;
          break;
        }
        m = 0;
        for (int i = 0; i < nb; ++i) m |= (long long)tb[i] << (8 * i);
        p += nb;
      }
      const long long L = m + 1;
      if (p + L > len || o + L > want) {
        bad = 1;
        break;
      }
      for (long long i0 = 0; i0 < L; i0 += 128) {
        unsigned char v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const long long i = i0 + u * 32 + lane;
          v[u] = i < L ? in[p + i] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const long long i = i0 + u * 32 + lane;
          if (i < L) {
            out[o + i] = v[u];
            ring[(o + i) & (SN_RING - 1)] = v[u];
          }
        }
      }
      p += L;
      o += L;
    } else {
      long long L, off;
      if (tt == 1) {
        if (p + 1 > len) {
          bad = 1;
          break;
        }
        L = 4 + ((tag >> 2) & 7u);
        off = ((long long)(tag >> 5) << 8) | tb[0];
        p += 1;
      } else if (tt == 2) {
        if (p + 2 > len) {
          bad = 1;
          break;
        }
        L = 1 + (tag >> 2);
        off = (long long)tb[0] | ((long long)tb[1] << 8);
        p += 2;
      } else {
        if (p + 4 > len) {
          bad = 1;
          break;
        }
        L = 1 + (tag >> 2);
        off = (long long)tb[0] | ((long long)tb[1] << 8) | ((long long)tb[2] << 16) | ((long long)tb[3] << 24);
        p += 4;
      }
      if (off == 0 || off > o || o + L > want) {
        bad = 1;
        break;
      }
      // byte o + i repeats the period [o - off, o): every source precedes this element
      if (off + L <= SN_RING) {
        for (long long i = lane; i < L; i += 32) {
          const unsigned char v = ring[(o - off + (i < off ? i : i % off)) & (SN_RING - 1)];
          out[o + i] = v;
          ring[(o + i) & (SN_RING - 1)] = v;
        }
      } else {
        for (long long i = lane; i < L; i += 32) {
          const unsigned char v = out[o - off + (i < off ? i : i % off)];
          out[o + i] = v;
          ring[(o + i) & (SN_RING - 1)] = v;
        }
      }
      o += L;
    }
    __syncwarp();
  }
  if (lane == 0 && (bad || o != want)) gb_set_error(st, GB_ERR_CORRUPT, KID_SNAPPY_D, c);
}

// ---------------------------------------------------------------- host side
struct DevMem {  // stream-ordered scratch, freed on scope exit
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit DevMem(cudaStream_t st) : s(st) {}
  ~DevMem() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
  template <class T>
  T* get(size_t count) {
    void* p = nullptr;
    if (cudaMallocAsync(&p, std::max<size_t>(count * sizeof(T), 16), s) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (T*)p;
  }
};

size_t rank_smem(bool gt) { return (gt ? 0 : (size_t)SN_STAB_SLOTS * 8) + 2 * 2048 * 4 + 32 * 4 + 16; }

long long nchunks_of(long long n) { return (n + SN_CHUNK - 1) / SN_CHUNK; }

// Encodes n device boxes: chunk table (num_boxes, raw_byte_size,
// compressed_size) into meta, the chunks' data concatenated into d_out.
int snap_encode(gb_context* ctx, const int4* d_boxes, long long n, int method, unsigned char* d_out, long long cap,
                long long* meta, long long* total) {
  GbCtx& c = ctx->c;
  const long long nch = nchunks_of(n);
  *total = 0;
  if (nch == 0) return GB_OK;
  DevMem M(c.stream);
  long long* d_rsize = M.get<long long>(nch);
  long long* d_roff = M.get<long long>(nch + 1);
  int* d_ovf = M.get<int>(nch + 1);  // count, then the chunks that need global tables
  unsigned* d_rank = M.get<unsigned>((size_t)2 * n);
  if (!d_rsize || !d_roff || !d_ovf || !d_rank) return gbi::set_err(ctx, GB_ERR_OOM, "snap encode scratch");
  cudaMemsetAsync(d_ovf, 0, (nch + 1) * sizeof(int), c.stream);
  const size_t sm_s = rank_smem(false), sm_g = rank_smem(true);
  cudaFuncSetAttribute((const void*)k_enc_rank<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_s);
  k_enc_rank<false><<<(unsigned)nch, SN_T, sm_s, c.stream>>>(d_boxes, n, nullptr, 0, nullptr, d_rank, d_ovf + 1, d_ovf,
                                                             c.st);
  ++c.launches;
  int novf = 0;
  cudaMemcpyAsync(&novf, d_ovf, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
  if (cudaStreamSynchronize(c.stream) != cudaSuccess) return gbi::set_err(ctx, GB_ERR_CUDA, "snap encode (ranks)");
  if (novf) {
    const int gblocks = std::min(novf, std::max(1, c.nsm));
    unsigned long long* gtab = M.get<unsigned long long>((size_t)gblocks * SN_GTAB_SLOTS);
    if (!gtab) return gbi::set_err(ctx, GB_ERR_OOM, "snap encode tables");
    k_enc_rank<true><<<gblocks, SN_T, sm_g, c.stream>>>(d_boxes, n, d_ovf + 1, novf, gtab, d_rank, nullptr, nullptr,
                                                        c.st);
    ++c.launches;
  }
  k_enc_emit<false><<<(unsigned)nch, SN_T, 0, c.stream>>>(d_boxes, n, d_rank, d_rsize, nullptr, nullptr, c.st);
  ++c.launches;
  std::vector<long long> rsize(nch), roff(nch + 1, 0);
  cudaMemcpyAsync(rsize.data(), d_rsize, nch * 8, cudaMemcpyDeviceToHost, c.stream);
  if (cudaStreamSynchronize(c.stream) != cudaSuccess) return gbi::set_err(ctx, GB_ERR_CUDA, "snap encode (size)");
  {
    int e = gb_sync(ctx, nullptr);
    if (e) return e;
  }
  for (long long i = 0; i < nch; ++i) roff[i + 1] = roff[i] + rsize[i];
  const long long rtot = roff[nch];
  unsigned char* d_raw = method == 0 ? nullptr : M.get<unsigned char>((size_t)rtot + 16);
  if (method == 0 && rtot > cap) return gbi::set_err(ctx, GB_ERR_CAPACITY, "snap output buffer too small");
  if (method != 0 && !d_raw) return gbi::set_err(ctx, GB_ERR_OOM, "snap raw buffer");
  unsigned char* rawbuf = method == 0 ? d_out : d_raw;
  cudaMemcpyAsync(d_roff, roff.data(), (nch + 1) * 8, cudaMemcpyHostToDevice, c.stream);
  k_enc_emit<true><<<(unsigned)nch, SN_T, 0, c.stream>>>(d_boxes, n, d_rank, nullptr, d_roff, rawbuf, c.st);
  ++c.launches;
  if (method == 0) {
    for (long long i = 0; i < nch; ++i) {
      meta[3 * i] = std::min((long long)SN_CHUNK, n - i * SN_CHUNK);
      meta[3 * i + 1] = rsize[i];
      meta[3 * i + 2] = rsize[i];
    }
    *total = rtot;
    return gb_sync(ctx, nullptr);
  }
  // Snappy: fragments of each chunk's codec bytes
  std::vector<long long> fsrc, fchunk;
  std::vector<int> flen;
  for (long long i = 0; i < nch; ++i)
    for (long long f0 = 0; f0 < rsize[i]; f0 += SN_FRAG) {
      fsrc.push_back(roff[i] + f0);
      flen.push_back((int)std::min((long long)SN_FRAG, rsize[i] - f0));
      fchunk.push_back(i);
    }
  const long long nfrag = (long long)fsrc.size();
  long long* d_fsrc = M.get<long long>(nfrag + 1);
  int* d_flen = M.get<int>(nfrag + 1);
  int* d_flout = M.get<int>(nfrag + 1);
  long long* d_fdst = M.get<long long>(nfrag + 1);
  long long* d_pre = M.get<long long>(2 * nch);
  unsigned char* d_fout = M.get<unsigned char>((size_t)std::max(nfrag, 1ll) * SN_FCAP);
  if (!d_fsrc || !d_flen || !d_flout || !d_fdst || !d_pre || !d_fout) return gbi::set_err(ctx, GB_ERR_OOM, "snappy scratch");
  if (nfrag) {
    cudaMemcpyAsync(d_fsrc, fsrc.data(), nfrag * 8, cudaMemcpyHostToDevice, c.stream);
    cudaMemcpyAsync(d_flen, flen.data(), nfrag * 4, cudaMemcpyHostToDevice, c.stream);
    cudaFuncSetAttribute((const void*)k_snappy_compress, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 * 2048 * 2);
    k_snappy_compress<<<(unsigned)((nfrag + 7) / 8), 256, 8 * 2048 * 2, c.stream>>>(d_raw, d_fsrc, d_flen, nfrag, d_fout,
                                                                                    d_flout, c.st);
    ++c.launches;
  }
  std::vector<int> flout(nfrag);
  if (nfrag) cudaMemcpyAsync(flout.data(), d_flout, nfrag * 4, cudaMemcpyDeviceToHost, c.stream);
  {
    int e = gb_sync(ctx, nullptr);
    if (e) return e;
  }
  std::vector<long long> fdst(nfrag), pre(2 * nch);
  long long at = 0, fi = 0;
  for (long long i = 0; i < nch; ++i) {
    pre[i] = at;
    pre[nch + i] = rsize[i];
    const long long start = at;
    at += sn_vlen((unsigned long long)rsize[i]);
    for (; fi < nfrag && fchunk[fi] == i; ++fi) {
      fdst[fi] = at;
      at += flout[fi];
    }
    meta[3 * i] = std::min((long long)SN_CHUNK, n - i * SN_CHUNK);
    meta[3 * i + 1] = rsize[i];
    meta[3 * i + 2] = at - start;
  }
  if (at > cap) return gbi::set_err(ctx, GB_ERR_CAPACITY, "snap output buffer too small");
  if (nfrag) cudaMemcpyAsync(d_fdst, fdst.data(), nfrag * 8, cudaMemcpyHostToDevice, c.stream);
  cudaMemcpyAsync(d_pre, pre.data(), 2 * nch * 8, cudaMemcpyHostToDevice, c.stream);
  k_snappy_gather<<<(unsigned)std::max(nfrag, 1ll), 256, 0, c.stream>>>(d_fout, d_flout, d_fdst, nfrag, d_pre,
                                                                       d_pre + nch, nch, d_out);
  ++c.launches;
  *total = at;
  return gb_sync(ctx, nullptr);
}

// Decodes the concatenated chunk data (device) described by meta.
int snap_decode(gb_context* ctx, const unsigned char* d_data, const long long* meta, long long nch, int method,
                int4* d_boxes) {
  GbCtx& c = ctx->c;
  if (nch == 0) return GB_OK;
  long long n = 0;
  std::vector<long long> roff(nch + 1, 0), coff(nch + 1, 0), rlen(nch), clen(nch);
  for (long long i = 0; i < nch; ++i) {
    if (meta[3 * i] < 0 || meta[3 * i] > SN_CHUNK || (i + 1 < nch && meta[3 * i] != SN_CHUNK) || meta[3 * i + 1] < 0 ||
        meta[3 * i + 2] < 0)
      return gbi::set_err(ctx, GB_ERR_CORRUPT, "snap chunk table");
    n += meta[3 * i];
    rlen[i] = meta[3 * i + 1];
    clen[i] = meta[3 * i + 2];
    roff[i + 1] = roff[i] + rlen[i];
    coff[i + 1] = coff[i] + clen[i];
  }
  if (method == 0)
    for (long long i = 0; i < nch; ++i)
      if (rlen[i] != clen[i]) return gbi::set_err(ctx, GB_ERR_CORRUPT, "snap chunk sizes");
  DevMem M(c.stream);
  long long* d_tab = M.get<long long>(4 * (nch + 1));
  unsigned* d_rec = M.get<unsigned>((size_t)nch * SN_CHUNK);
  int* d_dict = M.get<int>((size_t)nch * 2 * SN_CHUNK);
  unsigned char* d_raw = method == 0 ? nullptr : M.get<unsigned char>((size_t)roff[nch] + 16);
  if (!d_tab || !d_rec || !d_dict || (method != 0 && !d_raw)) return gbi::set_err(ctx, GB_ERR_OOM, "snap decode scratch");
  std::vector<long long> tab(4 * (nch + 1));
  std::copy(roff.begin(), roff.end(), tab.begin());
  std::copy(coff.begin(), coff.end(), tab.begin() + (nch + 1));
  std::copy(rlen.begin(), rlen.end(), tab.begin() + 2 * (nch + 1));
  std::copy(clen.begin(), clen.end(), tab.begin() + 3 * (nch + 1));
  cudaMemcpyAsync(d_tab, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, c.stream);
  const long long* d_roff = d_tab;
  const long long* d_coff = d_tab + (nch + 1);
  const long long* d_rlen = d_tab + 2 * (nch + 1);
  const long long* d_clen = d_tab + 3 * (nch + 1);
  const unsigned char* raw = d_data;
  if (method != 0) {
    cudaFuncSetAttribute((const void*)k_snappy_decompress, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         SN_RING + SN_STAGE);
    k_snappy_decompress<<<(unsigned)nch, 32, SN_RING + SN_STAGE, c.stream>>>(d_data, d_coff, d_clen, d_raw, d_roff,
                                                                             d_rlen, nch, c.st);
    ++c.launches;
    raw = d_raw;
  }
  k_codec_bounds<<<(unsigned)nch, SN_BT, 0, c.stream>>>(raw, d_roff, d_rlen, n, nch, d_rec, c.st);
  k_codec_decode<<<(unsigned)nch, SN_T, 0, c.stream>>>(raw, d_roff, d_rec, n, d_dict, d_boxes, c.st);
  c.launches += 2;
  return gb_sync(ctx, nullptr);
}

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }

}  // namespace

extern "C" int gb_snap_max_bytes(long long n, long long* bytes) {
  if (n < 0 || !bytes) return GB_ERR_ARG;
  const long long nch = nchunks_of(n);
  const long long raw = n * SN_REC_MAX;
  *bytes = raw + raw / 6 + nch * 64 + (raw / SN_FRAG + nch) * 64 + 64;
  return GB_OK;
}

extern "C" int gb_compress_boxes_to_stream(gb_context* ctx, const c_box* d_boxes, long long n, int method,
                                           unsigned char* d_out, long long cap, long long* chunk_meta, long long* total) {
  if (!ctx || n < 0 || !total || (n > 0 && (!d_boxes || !d_out || !chunk_meta))) return GB_ERR_ARG;
  if (method != 0 && method != 1) return gbi::set_err(ctx, GB_ERR_ARG, "compression method: 0 (codec only) or 1 (Snappy)");
  if (n > 0xffffffffll || ((uintptr_t)d_boxes & 15u)) return GB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return snap_encode(ctx, (const int4*)d_boxes, n, method, d_out, cap, chunk_meta, total);
}

extern "C" int gb_decompress_stream_to_boxes(gb_context* ctx, const unsigned char* d_data, const long long* chunk_meta,
                                             long long num_chunks, int method, c_box* d_boxes) {
  if (!ctx || num_chunks < 0 || (num_chunks > 0 && (!d_data || !chunk_meta || !d_boxes))) return GB_ERR_ARG;
  if (method != 0 && method != 1) return gbi::set_err(ctx, GB_ERR_ARG, "compression method: 0 (codec only) or 1 (Snappy)");
  if ((uintptr_t)d_boxes & 15u) return GB_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return snap_decode(ctx, d_data, chunk_meta, num_chunks, method, (int4*)d_boxes);
}

extern "C" int gb_save_layer_to_snap(gb_context* ctx, const char* path, const c_box* d_boxes, long long n, int method,
                                     int layer_properties, const long long* pnum) {
  if (!ctx || !path || n < 0 || (n > 0 && !d_boxes)) return GB_ERR_ARG;
  long long cap = 0;
  gb_snap_max_bytes(n, &cap);
  const long long nch = nchunks_of(n);
  std::vector<long long> meta(3 * std::max(nch, 1ll));
  unsigned char* d_out = nullptr;
  if (n > 0 && cudaMalloc(&d_out, (size_t)cap) != cudaSuccess) return gbi::set_err(ctx, GB_ERR_OOM, "snap output buffer");
  long long total = 0;
  int e = n > 0 ? gb_compress_boxes_to_stream(ctx, d_boxes, n, method, d_out, cap, meta.data(), &total) : GB_OK;
  if (e == GB_OK && (method != 0 && method != 1)) e = gbi::set_err(ctx, GB_ERR_ARG, "compression method");
  std::vector<unsigned char> data((size_t)total);
  if (e == GB_OK && total > 0 &&
      cudaMemcpyAsync(data.data(), d_out, (size_t)total, cudaMemcpyDeviceToHost, ctx->c.stream) != cudaSuccess)
    e = GB_ERR_CUDA;
  if (e == GB_OK && cudaStreamSynchronize(ctx->c.stream) != cudaSuccess) e = GB_ERR_CUDA;
  if (d_out) cudaFree(d_out);
  if (e) return e;
  FILE* f = fopen(path, "wb");
  if (!f) return gbi::set_err(ctx, GB_ERR_ARG, "cannot open the .snap file for writing");
  // serialization.f90:27-48: version, properties, totals, [PNUM table], chunks, offset table, its position.
  // As SaveLayerToSnap (diskdesign_impl.f90:63-67) the R-tree bit is not saved; the PNUM bit says
  // whether the table follows, which is what RestoreCompressedStreamFromDisk reads.
  layer_properties &= ~8;
  layer_properties = pnum ? (layer_properties | SN_LAYER_STATE_PNUM) : (layer_properties & ~SN_LAYER_STATE_PNUM);
  const int ver = SN_CODEC_VERSION;
  bool ok = write_all(f, &ver, 4) && write_all(f, &layer_properties, 4) && write_all(f, &n, 8) &&
            write_all(f, &nch, 8) && write_all(f, &method, 4);
  long long pos = 28;
  if (ok && pnum) {
    ok = write_all(f, pnum, (size_t)n * 8);
    pos += n * 8;
  }
  std::vector<long long> offs(nch);
  long long dpos = 0;
  for (long long i = 0; ok && i < nch; ++i) {
    offs[i] = pos + 1;  // 1-based stream positions
    ok = write_all(f, &meta[3 * i], 24) && write_all(f, data.data() + dpos, (size_t)meta[3 * i + 2]);
    dpos += meta[3 * i + 2];
    pos += 24 + meta[3 * i + 2];
  }
  const long long table = pos + 1;
  ok = ok && write_all(f, offs.data(), (size_t)nch * 8) && write_all(f, &table, 8);
  ok = (fclose(f) == 0) && ok;
  return ok ? GB_OK : gbi::set_err(ctx, GB_ERR_ARG, "write to the .snap file failed");
}

namespace {
struct SnapFile {
  int ver = 0, props = 0, method = 0;
  long long total = 0, nch = 0;
  long long pnum_at = -1;
  std::vector<long long> meta;
  std::vector<unsigned char> data;
};

int read_snap(const char* path, SnapFile& S, bool with_data, std::string* why) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    *why = "cannot open the .snap file";
    return GB_ERR_ARG;
  }
  fseek(f, 0, SEEK_END);
  const long long size = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (size == 0) {  // serialization.f90:98-103: an empty file is an empty layer
    fclose(f);
    return GB_OK;
  }
  auto rd = [&](void* p, size_t k) { return k == 0 || fread(p, 1, k, f) == k; };
  bool ok = rd(&S.ver, 4) && rd(&S.props, 4) && rd(&S.total, 8) && rd(&S.nch, 8) && rd(&S.method, 4);
  if (!ok || S.total < 0 || S.nch < 0 || S.nch != nchunks_of(S.total) || S.total > 0xffffffffll) {
    fclose(f);
    *why = "malformed .snap header";
    return GB_ERR_CORRUPT;
  }
  long long pos = 28;
  if (S.props & SN_LAYER_STATE_PNUM) {
    S.pnum_at = pos;
    pos += 8 * S.total;
    fseek(f, pos, SEEK_SET);
  }
  S.meta.resize(3 * S.nch);
  long long dbytes = 0;
  std::vector<long long> at(S.nch);
  for (long long i = 0; ok && i < S.nch; ++i) {
    ok = rd(&S.meta[3 * i], 24) && S.meta[3 * i + 2] >= 0 && pos + 24 + S.meta[3 * i + 2] <= size;
    at[i] = pos + 24;
    pos += 24 + S.meta[3 * i + 2];
    dbytes += S.meta[3 * i + 2];
    if (ok) fseek(f, pos, SEEK_SET);
  }
  if (ok && with_data) {
    S.data.resize((size_t)dbytes);
    long long d = 0;
    for (long long i = 0; ok && i < S.nch; ++i) {
      fseek(f, at[i], SEEK_SET);
      ok = rd(S.data.data() + d, (size_t)S.meta[3 * i + 2]);
      d += S.meta[3 * i + 2];
    }
  }
  fclose(f);
  if (!ok) {
    *why = "truncated .snap file";
    return GB_ERR_CORRUPT;
  }
  return GB_OK;
}
}  // namespace

extern "C" int gb_snap_file_info(const char* path, long long* total_boxes, long long* num_chunks, int* method,
                                 int* layer_properties) {
  if (!path) return GB_ERR_ARG;
  SnapFile S;
  std::string why;
  const int e = read_snap(path, S, false, &why);
  if (e) return e;
  if (total_boxes) *total_boxes = S.total;
  if (num_chunks) *num_chunks = S.nch;
  if (method) *method = S.method;
  if (layer_properties) *layer_properties = S.props;
  return GB_OK;
}

extern "C" int gb_restore_snap_to_layer(gb_context* ctx, const char* path, c_box* d_boxes, long long cap, long long* n,
                                        long long* pnum) {
  if (!ctx || !path || !n) return GB_ERR_ARG;
  SnapFile S;
  std::string why;
  int e = read_snap(path, S, true, &why);
  if (e) return gbi::set_err(ctx, e, why.c_str());
  *n = S.total;
  if (S.total > cap || (S.total > 0 && !d_boxes)) return gbi::set_err(ctx, GB_ERR_CAPACITY, "box buffer too small");
  if (S.method != 0 && S.method != 1)
    return gbi::set_err(ctx, GB_ERR_ARG, "compression method of the file is not Snappy (ZLIB/ZSTD are not supported)");
  if (pnum && S.pnum_at >= 0) {
    FILE* f = fopen(path, "rb");
    const bool ok = f && fseek(f, S.pnum_at, SEEK_SET) == 0 && fread(pnum, 8, (size_t)S.total, f) == (size_t)S.total;
    if (f) fclose(f);
    if (!ok) return gbi::set_err(ctx, GB_ERR_CORRUPT, "truncated PNUM table");
  }
  if (S.total == 0) return GB_OK;
  unsigned char* d_data = nullptr;
  if (cudaMalloc(&d_data, std::max<size_t>(S.data.size(), 16)) != cudaSuccess)
    return gbi::set_err(ctx, GB_ERR_OOM, "snap data buffer");
  cudaMemcpyAsync(d_data, S.data.data(), S.data.size(), cudaMemcpyHostToDevice, ctx->c.stream);
  e = gb_decompress_stream_to_boxes(ctx, d_data, S.meta.data(), S.nch, S.method, d_boxes);
  cudaStreamSynchronize(ctx->c.stream);
  cudaFree(d_data);
  return e;
}
