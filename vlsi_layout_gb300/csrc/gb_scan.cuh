// gb_scan.cuh -- warp / block scan helpers used by the engine's kernels.
#pragma once
#include <cstdint>

__device__ __forceinline__ int gb_lane() { return threadIdx.x & 31; }
__device__ __forceinline__ int gb_warp() { return threadIdx.x >> 5; }

template <typename T>
__device__ __forceinline__ T gb_warp_incl(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, v, o);
    if (gb_lane() >= o) v += y;
  }
  return v;
}

// Exclusive warp scan; *total gets the warp sum.
template <typename T>
__device__ __forceinline__ T gb_warp_excl(T v, T* total) {
  T inc = gb_warp_incl(v);
  *total = __shfl_sync(0xffffffffu, inc, 31);
  return inc - v;
}

template <typename T>
__device__ __forceinline__ T gb_warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide exclusive scan (blockDim.x multiple of 32, <= 1024).  `tmp` must
// hold 33 elements of T in shared memory.  All threads must call it.
template <typename T>
__device__ __forceinline__ T gb_block_excl(T v, T* tmp, T* total) {
  const int lane = gb_lane(), wid = gb_warp(), nw = blockDim.x >> 5;
  T wt;
  T ex = gb_warp_excl(v, &wt);
  __syncthreads();
  if (lane == 0) tmp[wid] = wt;
  __syncthreads();
  if (wid == 0) {
    T x = lane < nw ? tmp[lane] : T(0);
    T t2;
    T e2 = gb_warp_excl(x, &t2);
    if (lane < nw) tmp[lane] = e2;
    if (lane == 0) tmp[32] = t2;
  }
  __syncthreads();
  T r = ex + tmp[wid];
  *total = tmp[32];
  __syncthreads();
  return r;
}

template <typename T>
__device__ __forceinline__ T gb_block_sum(T v, T* tmp) {
  T tot;
  gb_block_excl(v, tmp, &tot);
  return tot;
}
