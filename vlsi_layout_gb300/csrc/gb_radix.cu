// gb_radix.cu -- hand-written LSD radix sort (onesweep form) for 64-bit keys
// with 32-bit payloads: Morton-ordered boxes (gpu_morton.cu:113-187),
// tracker events (event_sorter.cu:48-81) and canonical strip order.
//
//  1. One read of the keys builds the digit histograms of every pass
//     (per-CTA shared-memory counters, merged with global atomics).
//  2. Each pass is one kernel: a CTA takes the next tile from an atomic
//     counter (so tiles start in order), ranks its keys stably with warp
//     match/ballot ranking, publishes its per-digit counts, and obtains the
//     exclusive prefix of all earlier tiles by a decoupled look-back over a
//     status array.  Keys are staged in shared memory by digit and written
//     out in runs.
// Status words carry an epoch tag, so the array is never cleared between
// passes.  Every look-back wait is bounded: after the limit the kernel flags
// GB_ERR_TIMEOUT in the context status and finishes without hanging.
#include "gb_internal.h"
#include "gb_scan.cuh"

#define RS_THREADS 256
#define RS_WARPS (RS_THREADS / 32)
#define RS_IT 16
#define RS_TILE (RS_THREADS * RS_IT)
#define RS_RADIX 256
#define RS_MAXPASS 8
#define RS_SPIN_LIMIT (1 << 22)
#define KID_RADIX 40

// status word: [63:48] epoch, [47:46] flag (1 aggregate, 2 inclusive prefix), [45:0] value
#define RS_FLAG_AGG 1ull
#define RS_FLAG_PRE 2ull

__global__ void __launch_bounds__(RS_THREADS)
k_rs_hist(const unsigned long long* __restrict__ keys, long long n, int passes, int dbits,
          unsigned* __restrict__ ghist) {
  __shared__ unsigned h[RS_MAXPASS][RS_RADIX];
  for (int i = threadIdx.x; i < RS_MAXPASS * RS_RADIX; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  const unsigned mask = (1u << dbits) - 1u;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (p * dbits)) & mask], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * RS_RADIX; i += blockDim.x) {
    const unsigned v = (&h[0][0])[i];
    if (v) atomicAdd(&ghist[i], v);
  }
}

__global__ void k_rs_hist_scan(unsigned* ghist, int passes, int radix) {
  // one block of RS_RADIX threads per pass
  __shared__ long long tmp[33];
  const int p = blockIdx.x;
  const long long v = threadIdx.x < radix ? ghist[p * RS_RADIX + threadIdx.x] : 0;
  long long tot;
  const long long ex = gb_block_excl(v, tmp, &tot);
  if (threadIdx.x < radix) ghist[p * RS_RADIX + threadIdx.x] = (unsigned)ex;
}

struct RsSmem {
  unsigned long long k[RS_TILE];
  unsigned v[RS_TILE];
  unsigned short wh[RS_WARPS][RS_RADIX];  // per-warp digit counts
  unsigned bstart[RS_RADIX];              // tile-local bucket start
  unsigned long long gpos[RS_RADIX];      // global start of this tile's run of digit d
  long long tile;
};

__global__ void __launch_bounds__(RS_THREADS)
k_rs_pass(const unsigned long long* __restrict__ kin, const unsigned* __restrict__ vin,
          unsigned long long* __restrict__ kout, unsigned* __restrict__ vout, long long n, int shift,
          int dbits, const unsigned* __restrict__ gofs, unsigned long long* status,
          unsigned long long epoch, long long* counter, DStatus* st, int spin_limit) {
  extern __shared__ __align__(16) unsigned char smraw[];
  RsSmem& s = *reinterpret_cast<RsSmem*>(smraw);
  const int lane = gb_lane(), wid = gb_warp();
  const int radix = 1 << dbits;
  const unsigned mask = (unsigned)radix - 1u;
  const long long ntile = (n + RS_TILE - 1) / RS_TILE;
  if (threadIdx.x == 0) s.tile = (long long)atomicAdd((unsigned long long*)counter, 1ull);
  for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += blockDim.x) (&s.wh[0][0])[i] = 0;
  __syncthreads();
  const long long tile = s.tile;
  if (tile >= ntile) return;
  const long long tbase = tile * RS_TILE;
  // ---- load (warp-striped: warp w owns a contiguous range) and rank
  unsigned long long key[RS_IT];
  unsigned val[RS_IT];
  unsigned short rnk[RS_IT];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < RS_IT; ++it) {
    const long long pos = tbase + (long long)wid * 32 * RS_IT + it * 32 + lane;
    const bool ok = pos < n;
    key[it] = ok ? kin[pos] : ~0ull;
    val[it] = ok ? vin[pos] : 0u;
    const unsigned d = ok ? (unsigned)((key[it] >> shift) & mask) : 0xFFFFu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned before = s.wh[wid][ok ? d : 0];
    __syncwarp();
    rnk[it] = (unsigned short)(before + __popc(peers & lt));
    if (ok && (peers & lt) == 0) s.wh[wid][d] = (unsigned short)(before + __popc(peers));
    __syncwarp();
  }
  __syncthreads();
  // ---- per-digit prefix over warps, tile totals, bucket starts
  unsigned tot = 0;
  if (threadIdx.x < radix) {
    const int d = threadIdx.x;
    for (int w = 0; w < RS_WARPS; ++w) {
      const unsigned c = s.wh[w][d];
      s.wh[w][d] = (unsigned short)tot;
      tot += c;
    }
  }
  {
    __shared__ long long tmp[33];
    long long tt;
    const long long ex = gb_block_excl((long long)(threadIdx.x < radix ? tot : 0), tmp, &tt);
    if (threadIdx.x < radix) s.bstart[threadIdx.x] = (unsigned)ex;
  }
  // ---- decoupled look-back (one thread per digit)
  if (threadIdx.x < radix) {
    const int d = threadIdx.x;
    unsigned long long* my = status + (size_t)tile * RS_RADIX + d;
    const unsigned long long etag = (epoch & 0xFFFFull) << 48;
    unsigned long long excl = 0;
    if (tile == 0) {
      *(volatile unsigned long long*)my = etag | (RS_FLAG_PRE << 46) | (unsigned long long)tot;
    } else {
      *(volatile unsigned long long*)my = etag | (RS_FLAG_AGG << 46) | (unsigned long long)tot;
      long long j = tile - 1;
      int spins = 0;
      while (j >= 0) {
        const unsigned long long w = *(volatile unsigned long long*)(status + (size_t)j * RS_RADIX + d);
        const unsigned long long flag = (w >> 46) & 3ull;
        if ((w & 0xFFFF000000000000ull) != etag || flag == 0) {
          if (++spins > spin_limit) {
            gb_set_error(st, GB_ERR_TIMEOUT, KID_RADIX, j);
            break;
          }
          continue;
        }
        excl += w & ((1ull << 46) - 1);
        if (flag == RS_FLAG_PRE) break;
        --j;
      }
      __threadfence();
      *(volatile unsigned long long*)my = etag | (RS_FLAG_PRE << 46) | (excl + tot);
    }
    s.gpos[d] = (unsigned long long)gofs[d] + excl;
  }
  __syncthreads();
  // ---- stage in shared memory by digit
#pragma unroll
  for (int it = 0; it < RS_IT; ++it) {
    const long long pos = tbase + (long long)wid * 32 * RS_IT + it * 32 + lane;
    if (pos < n) {
      const unsigned d = (unsigned)((key[it] >> shift) & mask);
      const unsigned lp = s.bstart[d] + s.wh[wid][d] + rnk[it];
      s.k[lp] = key[it];
      s.v[lp] = val[it];
    }
  }
  __syncthreads();
  // ---- write runs
  const int cnt = (int)min((long long)RS_TILE, n - tbase);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    const unsigned long long k = s.k[i];
    const unsigned d = (unsigned)((k >> shift) & mask);
    const unsigned long long gp = s.gpos[d] + (unsigned long long)(i - (int)s.bstart[d]);
    kout[gp] = k;
    vout[gp] = s.v[i];
  }
}

__global__ void k_rs_zero(unsigned* p, int n, long long* ctrs, int nc) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0;
  if (threadIdx.x < nc) ctrs[threadIdx.x] = 0;
}

struct RsState {
  unsigned* ghist = nullptr;
  unsigned long long* status = nullptr;
  long long status_tiles = 0;
  long long* ctrs = nullptr;
  unsigned long long epoch = 0;
  bool attr = false;
};
static RsState g_rs;

int gb_radix_sort_pairs(GbCtx& c, unsigned long long* keys, unsigned* vals, long long n, int bits,
                        unsigned long long* keys_tmp, unsigned* vals_tmp, int digit_bits) {
  if (n <= 1) return 0;
  if (digit_bits < 1 || digit_bits > 8) digit_bits = 8;
  int passes = (bits + digit_bits - 1) / digit_bits;
  if (passes < 1) passes = 1;
  if (passes > RS_MAXPASS) return -1;
  const long long ntile = (n + RS_TILE - 1) / RS_TILE;
  if (!g_rs.ghist) {
    cudaMalloc(&g_rs.ghist, RS_MAXPASS * RS_RADIX * sizeof(unsigned));
    cudaMalloc(&g_rs.ctrs, RS_MAXPASS * sizeof(long long));
  }
  if (g_rs.status_tiles < ntile) {
    if (g_rs.status) cudaFree(g_rs.status);
    const long long want = ntile + 1024;
    if (cudaMalloc(&g_rs.status, (size_t)want * RS_RADIX * 8) != cudaSuccess) return -2;
    cudaMemsetAsync(g_rs.status, 0, (size_t)want * RS_RADIX * 8, c.stream);
    g_rs.status_tiles = want;
  }
  if (!g_rs.attr) {
    cudaFuncSetAttribute(k_rs_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RsSmem));
    g_rs.attr = true;
  }
  k_rs_zero<<<1, 1024, 0, c.stream>>>(g_rs.ghist, RS_MAXPASS * RS_RADIX, g_rs.ctrs, RS_MAXPASS);
  k_rs_hist<<<c.nsm * 4, RS_THREADS, 0, c.stream>>>(keys, n, passes, digit_bits, g_rs.ghist);
  k_rs_hist_scan<<<passes, RS_RADIX, 0, c.stream>>>(g_rs.ghist, passes, 1 << digit_bits);
  unsigned long long* ka = keys;
  unsigned* va = vals;
  unsigned long long* kb = keys_tmp;
  unsigned* vb = vals_tmp;
  for (int p = 0; p < passes; ++p) {
    g_rs.epoch = (g_rs.epoch + 1) & 0xFFFFull;
    if (g_rs.epoch == 0) {
      cudaMemsetAsync(g_rs.status, 0, (size_t)g_rs.status_tiles * RS_RADIX * 8, c.stream);
      g_rs.epoch = 1;
    }
    k_rs_pass<<<(unsigned)ntile, RS_THREADS, sizeof(RsSmem), c.stream>>>(
        ka, va, kb, vb, n, p * digit_bits, digit_bits, g_rs.ghist + p * RS_RADIX, g_rs.status,
        g_rs.epoch, g_rs.ctrs + p, c.st, RS_SPIN_LIMIT);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    cudaMemcpyAsync(keys, ka, (size_t)n * 8, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream);
  }
  return passes;
}

// Diagnostics for the bounded look-back: one CTA is handed tile 1 of a
// two-tile pass, so it waits for a tile-0 status word that nothing ever
// publishes.  After spin_limit polls it must flag GB_ERR_TIMEOUT and finish.
__global__ void k_rs_set_counter(long long* c, long long v) { *c = v; }
int gb_radix_lookback_timeout_probe(GbCtx& c, int spin_limit) {
  const long long n = 2 * RS_TILE;
  unsigned long long *k = nullptr, *k2 = nullptr, *status = nullptr;
  unsigned *v = nullptr, *v2 = nullptr, *gofs = nullptr;
  long long* ctr = nullptr;
  cudaMalloc(&k, n * 8); cudaMalloc(&k2, n * 8); cudaMalloc(&v, n * 4); cudaMalloc(&v2, n * 4);
  cudaMalloc(&status, 2 * RS_RADIX * 8); cudaMalloc(&gofs, RS_RADIX * 4); cudaMalloc(&ctr, 8);
  cudaMemsetAsync(k, 0, n * 8, c.stream);
  cudaMemsetAsync(v, 0, n * 4, c.stream);
  cudaMemsetAsync(status, 0, 2 * RS_RADIX * 8, c.stream);
  cudaMemsetAsync(gofs, 0, RS_RADIX * 4, c.stream);
  k_rs_set_counter<<<1, 1, 0, c.stream>>>(ctr, 1);
  cudaFuncSetAttribute(k_rs_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RsSmem));
  k_rs_pass<<<1, RS_THREADS, sizeof(RsSmem), c.stream>>>(k, v, k2, v2, n, 0, 8, gofs, status, 7, ctr, c.st,
                                                        spin_limit);
  const cudaError_t e = cudaStreamSynchronize(c.stream);
  cudaFree(k); cudaFree(k2); cudaFree(v); cudaFree(v2); cudaFree(status); cudaFree(gofs); cudaFree(ctr);
  return e == cudaSuccess ? 0 : -1;
}
