// Exclusive scan of int64 values on the device: out[i] = sum of in[< i] and
// out[n] = the total. Three launches: per-tile scans (2048 values per
// 256-thread block), one block scanning the tile sums, and the tile offsets
// added back. Included by each translation unit that scans (internal linkage).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "covgpu.h"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER_THREAD = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;  // elements per scan block

inline unsigned scan_blocks_for(int64_t n, int per_block) {
  const int64_t b = (n + per_block - 1) / per_block;
  return (unsigned)(b < 1 ? 1 : b);
}

// exclusive scan of int64 values: out[i] = sum of in[< i], out[n] = total
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const int64_t* in, int64_t* out, int64_t* tile_sums,
                                                            int64_t n) {
  __shared__ int64_t s_warp[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER_THREAD;
  int64_t v[SCAN_PER_THREAD];
  int64_t sum = 0;
#pragma unroll
  for (int j = 0; j < SCAN_PER_THREAD; ++j) {
    v[j] = base + j < n ? in[base + j] : 0;
    sum += v[j];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  int64_t woff = 0;
  for (int k = 0; k < warp; ++k) woff += s_warp[k];
  int64_t run = woff + incl - sum;
#pragma unroll
  for (int j = 0; j < SCAN_PER_THREAD; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == SCAN_THREADS - 1) tile_sums[blockIdx.x] = woff + incl;
}

// one block: exclusive scan of the tile sums in place, total into *total
__global__ void __launch_bounds__(1024) k_scan_sums(int64_t* tile_sums, int64_t n_tiles, int64_t* total) {
  __shared__ int64_t s_warp[32];
  __shared__ int64_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t b0 = 0; b0 < n_tiles; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    const int64_t x = i < n_tiles ? tile_sums[i] : 0;
    int64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int64_t woff = 0;
    for (int k = 0; k < warp; ++k) woff += s_warp[k];
    const int64_t carry = s_carry;
    if (i < n_tiles) tile_sums[i] = carry + woff + incl - x;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = carry + woff + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

__global__ void k_scan_add(int64_t* out, const int64_t* tile_sums, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_sums[i / SCAN_TILE];
}

// out[0..n] = exclusive scan of in[0..n) with out[n] the total; scratch: tile sums
int scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* scratch, cudaStream_t s) {
  const unsigned tiles = scan_blocks_for(n, SCAN_TILE);
  k_scan_tiles<<<tiles, SCAN_THREADS, 0, s>>>(in, out, scratch, n);
  k_scan_sums<<<1, 1024, 0, s>>>(scratch, (int64_t)tiles, out + n);
  k_scan_add<<<scan_blocks_for(n, 256), 256, 0, s>>>(out, scratch, n);
  return cudaGetLastError() == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
}


}  // namespace
