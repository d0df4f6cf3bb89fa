// Launch helpers and tuning constants shared by the covgpu translation units
// (covgpu.cu: the day kernels and the state entry points; covgpu_reference.cu:
// the reference's standalone kernels; covgpu_testing.cu: testing and tracing).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "covgpu.h"

namespace covgpu {

constexpr int AGENT_THREADS = 256;     // one agent per thread; agent blocks hold <= 256 agents
constexpr int EDGE_THREADS = 256;
constexpr int EDGE_VEC = 4;            // edges per 128-bit load
constexpr int EDGE_ROUND = EDGE_THREADS * EDGE_VEC;  // edges one block reads per round
constexpr int64_t EDGE_TILE_MAX = 8192;  // edge tiles: 1024, 2048, 4096 or 8192 edges (covgpu_state.edge_tile)

inline int launch_status() {
  return cudaGetLastError() == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
}
inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline int grid_for(int64_t n, int threads, int max_blocks = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

// Blocks of one wave of `kernel` with `threads` threads: its resident blocks per
// SM on the current device times the SM count (for the passes that walk
// agent-block ranges; any grid gives the same results), and the grid of such a
// pass over a state's agent blocks.
template <class K>
inline int64_t wave_blocks(K kernel, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return (int64_t)1 << 30;  // no wave bound: one block per agent block
  }
  return (int64_t)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
}
inline unsigned wave_grid(const covgpu_state* st, int64_t wave) {
  const int64_t nb = st->n_agent_blocks;
  return (unsigned)(nb < wave ? (nb > 0 ? nb : 1) : wave);
}

// the checks every state entry point makes before launching (covgpu.cu)
int check_state(const covgpu_state* st);
// the testing, tracing and post passes of day t (covgpu_testing.cu)
int launch_test_trace(const covgpu_state* st, int t, cudaStream_t s);

}  // namespace covgpu
