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

// the checks every state entry point makes before launching (covgpu.cu)
int check_state(const covgpu_state* st);
// the testing, tracing and post passes of day t (covgpu_testing.cu)
int launch_test_trace(const covgpu_state* st, int t, cudaStream_t s);

}  // namespace covgpu
