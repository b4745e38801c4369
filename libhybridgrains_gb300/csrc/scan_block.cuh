// Warp- and block-level exclusive scans of int32 shared by the device-wide
// scan and the batched re-sort.
#pragma once

namespace hg {

__device__ __forceinline__ int warp_incl_scan(int x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// Exclusive scan of one value per thread across a block of NT threads;
// returns the exclusive prefix and writes the block total to *total.
template <int NT> __device__ __forceinline__ int block_excl_scan(int x, int *total) {
  __shared__ int s_warp[NT / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_incl_scan(x);
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < NT / 32 ? s_warp[lane] : 0;
    w = warp_incl_scan(w);
    if (lane < NT / 32) s_warp[lane] = w;
  }
  __syncthreads();
  const int warp_off = wid > 0 ? s_warp[wid - 1] : 0;
  *total = s_warp[NT / 32 - 1];
  __syncthreads();
  return warp_off + inc - x;
}

} // namespace hg
