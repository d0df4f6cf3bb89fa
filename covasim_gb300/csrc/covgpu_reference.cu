// covgpu_reference: the reference's three numba functions (covasim/utils.py:38-128)
// as standalone GPU drop-ins -- compute_viral_load, compute_trans_sus and
// compute_infections (ordered output, bit-exact), with the allocation-free
// variant of compute_infections.
#include <cuda.h>
#include <cuda_runtime.h>
#include <atomic>
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_ff.cuh"
#include "covgpu_launch.cuh"

using namespace covgpu;

namespace {

constexpr int INF_TILE = 2048;         // edges per block of the ordered compute_infections
constexpr int INF_THREADS = 256;
constexpr int INF_PER_THREAD = INF_TILE / INF_THREADS;

// ============================================================ standalone kernels

__global__ void k_viral_load(int t, const float* __restrict__ ts, const float* __restrict__ tr,
                             const float* __restrict__ td, int64_t n, float frac_time, float load_ratio,
                             float high_cap, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = viral_load_one(t, ts[i], tr[i], td[i], frac_time, load_ratio, high_cap);
}

// utils.py:82-90: rel_trans*inf*f_quar*f_asymp*f_iso*beta_layer*viral_load and
// rel_sus*sus*f_quar*(1-immunity), float32 left to right (a factor of 1.0 is exact).
__global__ void k_trans_sus(const float* __restrict__ rt, const float* __restrict__ rs,
                            const uint8_t* __restrict__ inf, const uint8_t* __restrict__ sus, float beta_layer,
                            const float* __restrict__ vl, const uint8_t* __restrict__ symp,
                            const uint8_t* __restrict__ iso, const uint8_t* __restrict__ quar, float asymp_factor,
                            float iso_factor, float quar_factor, const float* __restrict__ imm, int64_t n,
                            float* __restrict__ ort, float* __restrict__ ors) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool q = quar[i];
    float a = __fmul_rn(rt[i], inf[i] ? 1.0f : 0.0f);
    a = __fmul_rn(a, q ? quar_factor : 1.0f);
    a = __fmul_rn(a, symp[i] ? 1.0f : asymp_factor);
    a = __fmul_rn(a, iso[i] ? iso_factor : 1.0f);
    a = __fmul_rn(a, beta_layer);
    a = __fmul_rn(a, vl[i]);
    float b = __fmul_rn(rs[i], sus[i] ? 1.0f : 0.0f);
    b = __fmul_rn(b, q ? quar_factor : 1.0f);
    b = __fmul_rn(b, __fsub_rn(1.0f, imm[i]));
    ort[i] = a;
    ors[i] = b;
  }
}

// utils.py:113-124 for one (direction, edge): in inf_inds (source trans != 0),
// drawn (beta != 0) and u < p in float64.
struct InfArgs {
  float beta; const int32_t* p1; const int32_t* p2; const float* lb; int64_t E;
  const float* rt; const float* rs; int64_t n_agents; const double* uni; uint32_t k0, k1; int day, variant, layer;
  int32_t* status;
};
__device__ __forceinline__ bool inf_hit(const InfArgs& a, int dir, int64_t e, int32_t& src, int32_t& tgt) {
  src = dir ? a.p2[e] : a.p1[e];
  tgt = dir ? a.p1[e] : a.p2[e];
  if ((uint32_t)src >= (uint64_t)a.n_agents || (uint32_t)tgt >= (uint64_t)a.n_agents) {  // bad index: skip
    if (a.status) atomicOr(a.status, COVGPU_BADARG);
    return false;
  }
  const float st = a.rt[src];
  if (st == 0.0f) return false;
  const float p = __fmul_rn(__fmul_rn(__fmul_rn(a.beta, a.lb[e]), st), a.rs[tgt]);
  if (p == 0.0f) return false;
  double u;
  if (a.uni) {
    u = a.uni[(int64_t)dir * a.E + e];
  } else {
    const uint4 w = philox(make_uint4((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)a.day,
                                      TAG_EDGE | ((uint32_t)a.variant << 8) | (uint32_t)a.layer), a.k0, a.k1);
    return dir ? bern52(w.z, w.w, p) : bern52(w.x, w.y, p);
  }
  return u < (double)p;
}

__global__ void __launch_bounds__(INF_THREADS) k_infections_count(InfArgs a, int64_t ntiles, int32_t* counts) {
  const int dir = blockIdx.y;
  const int64_t tile = blockIdx.x;
  const int64_t e0 = tile * INF_TILE + (int64_t)threadIdx.x * INF_PER_THREAD;
  int c = 0;
  for (int j = 0; j < INF_PER_THREAD; ++j) {
    const int64_t e = e0 + j;
    int32_t s, g;
    if (e < a.E && inf_hit(a, dir, e, s, g)) ++c;
  }
  __shared__ int s_sum;
  if (threadIdx.x == 0) s_sum = 0;
  __syncthreads();
  c = __reduce_add_sync(0xffffffffu, (unsigned)c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_sum, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[(int64_t)dir * ntiles + tile] = s_sum;
}

// single-block exclusive scan of m counts into int64 offsets; total into *total
__global__ void __launch_bounds__(1024) k_scan(const int32_t* counts, int64_t m, int64_t* offs, int64_t* total,
                                               int64_t capacity, int32_t* status) {
  __shared__ int64_t s_part[1024];
  const int64_t per = (m + blockDim.x - 1) / blockDim.x;
  const int64_t b = threadIdx.x * per, e = min(b + per, m);
  int64_t sum = 0;
  for (int64_t i = b; i < e; ++i) sum += counts[i];
  s_part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {  // Hillis-Steele inclusive scan
    const int64_t v = threadIdx.x >= (unsigned)off ? s_part[threadIdx.x - off] : 0;
    __syncthreads();
    s_part[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t run = s_part[threadIdx.x] - sum;
  for (int64_t i = b; i < e; ++i) { offs[i] = run; run += counts[i]; }
  if (threadIdx.x == blockDim.x - 1) {
    *total = s_part[threadIdx.x];
    if (s_part[threadIdx.x] > capacity && status) atomicOr(status, COVGPU_OVERFLOW);
  }
}

// ordered write: block-level exclusive scan of per-thread hit counts keeps edge order
__global__ void __launch_bounds__(INF_THREADS) k_infections_write(InfArgs a, int64_t ntiles, const int64_t* offs,
                                                                  int32_t* out_src, int32_t* out_tgt, int64_t cap) {
  const int dir = blockIdx.y;
  const int64_t tile = blockIdx.x;
  const int64_t e0 = tile * INF_TILE + (int64_t)threadIdx.x * INF_PER_THREAD;
  uint32_t hits = 0;
  int32_t hs[INF_PER_THREAD], ht[INF_PER_THREAD];
#pragma unroll
  for (int j = 0; j < INF_PER_THREAD; ++j) {
    const int64_t e = e0 + j;
    int32_t s = 0, g = 0;
    if (e < a.E && inf_hit(a, dir, e, s, g)) hits |= 1u << j;
    hs[j] = s;
    ht[j] = g;
  }
  const int c = __popc(hits);
  // block exclusive scan of c (warp shuffle scan + warp totals in shared memory)
  __shared__ int s_warp[INF_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < INF_THREADS / 32 ? s_warp[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += v;
    }
    if (lane < INF_THREADS / 32) s_warp[lane] = wi - w;
  }
  __syncthreads();
  int64_t pos = offs[(int64_t)dir * ntiles + tile] + s_warp[warp] + (incl - c);
#pragma unroll
  for (int j = 0; j < INF_PER_THREAD; ++j) {
    if (hits & (1u << j)) {
      if (pos < cap) { out_src[pos] = hs[j]; out_tgt[pos] = ht[j]; }
      ++pos;
    }
  }
}

}  // namespace

extern "C" {

int covgpu_viral_load(int32_t t, const float* date_inf, const float* date_rec, const float* date_dead, int64_t n,
                      float frac_time, float load_ratio, float high_cap, float* out_load, void* stream) {
  if (n < 0 || (n > 0 && (!date_inf || !date_rec || !date_dead || !out_load))) return COVGPU_BADARG;
  if (n == 0) return COVGPU_OK;
  k_viral_load<<<grid_for(n, 256), 256, 0, S(stream)>>>(t, date_inf, date_rec, date_dead, n, frac_time, load_ratio,
                                                         high_cap, out_load);
  return launch_status();
}

int covgpu_trans_sus(const float* rel_trans, const float* rel_sus, const uint8_t* inf, const uint8_t* sus,
                     float beta_layer, const float* viral_load, const uint8_t* symp, const uint8_t* iso,
                     const uint8_t* quar, float asymp_factor, float iso_factor, float quar_factor,
                     const float* immunity_factors, int64_t n, float* out_rel_trans, float* out_rel_sus,
                     void* stream) {
  if (n < 0) return COVGPU_BADARG;
  if (n == 0) return COVGPU_OK;
  if (!rel_trans || !rel_sus || !inf || !sus || !viral_load || !symp || !iso || !quar || !immunity_factors ||
      !out_rel_trans || !out_rel_sus)
    return COVGPU_BADARG;
  k_trans_sus<<<grid_for(n, 256), 256, 0, S(stream)>>>(rel_trans, rel_sus, inf, sus, beta_layer, viral_load, symp, iso,
                                                        quar, asymp_factor, iso_factor, quar_factor, immunity_factors,
                                                        n, out_rel_trans, out_rel_sus);
  return launch_status();
}

int64_t covgpu_infections_scratch_bytes(int64_t n_edges) {
  if (n_edges < 0) return -1;
  const int64_t ntiles = (n_edges + INF_TILE - 1) / INF_TILE;
  const int64_t m = 2 * (ntiles > 0 ? ntiles : 1);
  return m * (int64_t)sizeof(int64_t) + m * (int64_t)sizeof(int32_t) + 256;
}

int covgpu_infections(float beta, const int32_t* p1, const int32_t* p2, const float* layer_betas, int64_t n_edges,
                      const float* rel_trans, const float* rel_sus, int64_t n_agents, const double* uniforms,
                      uint64_t seed, int32_t day,
                      int32_t variant, int32_t layer, int32_t* out_src, int32_t* out_tgt, int64_t capacity,
                      int64_t* out_count, int32_t* status, void* scratch, int64_t scratch_bytes, void* stream) {
  if (n_edges < 0 || capacity < 0 || n_agents < 0 || !out_count) return COVGPU_BADARG;
  if (variant < 0 || variant >= COVGPU_MAX_VARIANTS || layer < 0 || layer >= COVGPU_MAX_LAYERS) return COVGPU_BADARG;
  if (scratch_bytes < covgpu_infections_scratch_bytes(n_edges) || !scratch) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  if (n_edges == 0) {
    return cudaMemsetAsync(out_count, 0, sizeof(int64_t), s) == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
  }
  if (!p1 || !p2 || !layer_betas || !rel_trans || !rel_sus || (capacity > 0 && (!out_src || !out_tgt)))
    return COVGPU_BADARG;
  const int64_t ntiles = (n_edges + INF_TILE - 1) / INF_TILE;
  if (ntiles > 0x7FFFFFFF) return COVGPU_BADARG;
  const int64_t m = 2 * ntiles;
  int64_t* offs = reinterpret_cast<int64_t*>(scratch);
  int32_t* counts = reinterpret_cast<int32_t*>(offs + m);
  InfArgs a;
  a.beta = beta; a.p1 = p1; a.p2 = p2; a.lb = layer_betas; a.E = n_edges; a.rt = rel_trans; a.rs = rel_sus;
  a.n_agents = n_agents; a.status = status; a.uni = uniforms; a.k0 = (uint32_t)seed; a.k1 = (uint32_t)(seed >> 32); a.day = day; a.variant = variant;
  a.layer = layer;
  dim3 grid((unsigned)ntiles, 2);
  k_infections_count<<<grid, INF_THREADS, 0, s>>>(a, ntiles, counts);
  k_scan<<<1, 1024, 0, s>>>(counts, m, offs, out_count, capacity, status);
  k_infections_write<<<grid, INF_THREADS, 0, s>>>(a, ntiles, offs, out_src, out_tgt, capacity);
  return launch_status();
}

// ---- compute_infections without allocation: scratch in a file-scope device array
//
// For callers that may not allocate device memory at all (see the declaration in
// covgpu.h). The tile counts and offsets that covgpu_infections keeps in caller
// scratch live here instead; every call rewrites all of the part it reads, so
// nothing needs clearing between calls, and calls whose kernels overlap on the
// GPU race on it.
constexpr int64_t NOALLOC_MAX_EDGES = COVGPU_NOALLOC_MAX_EDGES;
constexpr int64_t NOALLOC_TILES = (NOALLOC_MAX_EDGES + INF_TILE - 1) / INF_TILE;
constexpr int64_t NOALLOC_SCRATCH = 2 * NOALLOC_TILES * (int64_t)(sizeof(int64_t) + sizeof(int32_t));
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH];
constexpr int NOALLOC_MAX_DEVICES = 64;
// The device address of g_noalloc_scratch per device, with the context it was
// looked up in: a device reset or a new primary context (the module loaded
// again, possibly elsewhere) makes the next call look it up again. Atomic, so
// that host threads calling at the same time do not race on the cache.
struct NoallocSlot {
  std::atomic<void*> ptr{nullptr};
  std::atomic<void*> ctx{nullptr};
};
static NoallocSlot g_noalloc[NOALLOC_MAX_DEVICES];

// The current CUDA context, through the driver's cuCtxGetCurrent resolved by
// the runtime (no link against the driver library); null when unavailable.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
static CUcontext current_context() {
  static std::atomic<CtxGetCurrentFn> fn{nullptr};
  CtxGetCurrentFn f = fn.load(std::memory_order_acquire);
  if (!f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return nullptr;
    f = reinterpret_cast<CtxGetCurrentFn>(p);
    fn.store(f, std::memory_order_release);
  }
  CUcontext c = nullptr;
  return f(&c) == CUDA_SUCCESS ? c : nullptr;
}

// The array's host-side name is not a device address: look the address up once
// per device (and context), with that device current.
static int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return COVGPU_CUDA_ERROR;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return COVGPU_BADARG;
  NoallocSlot& slot = g_noalloc[dev];
  void* ctx = reinterpret_cast<void*>(current_context());
  void* p = slot.ptr.load(std::memory_order_acquire);
  if (!p || !ctx || slot.ctx.load(std::memory_order_acquire) != ctx) {
    p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return COVGPU_CUDA_ERROR;
    slot.ctx.store(reinterpret_cast<void*>(current_context()), std::memory_order_release);
    slot.ptr.store(p, std::memory_order_release);
  }
  *out = p;
  return COVGPU_OK;
}

int covgpu_infections_noalloc(float beta, const int32_t* p1, const int32_t* p2, const float* layer_betas,
                              int64_t n_edges, const float* rel_trans, const float* rel_sus, int64_t n_agents,
                              const double* uniforms, uint64_t seed, int32_t day, int32_t variant, int32_t layer,
                              int32_t* out_src, int32_t* out_tgt, int64_t capacity, int64_t* out_count,
                              int32_t* status, void* stream) {
  if (n_edges < 0 || n_edges > NOALLOC_MAX_EDGES) return COVGPU_BADARG;
  if (capacity < 0 || n_agents < 0 || !out_count) return COVGPU_BADARG;
  if (variant < 0 || variant >= COVGPU_MAX_VARIANTS || layer < 0 || layer >= COVGPU_MAX_LAYERS) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  if (n_edges == 0) {
    return cudaMemsetAsync(out_count, 0, sizeof(int64_t), s) == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
  }
  if (!p1 || !p2 || !layer_betas || !rel_trans || !rel_sus || (capacity > 0 && (!out_src || !out_tgt)))
    return COVGPU_BADARG;
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != COVGPU_OK) return rc;
  const int64_t ntiles = (n_edges + INF_TILE - 1) / INF_TILE;
  const int64_t m = 2 * ntiles;
  int64_t* offs = reinterpret_cast<int64_t*>(scratch);
  int32_t* counts = reinterpret_cast<int32_t*>(offs + m);
  InfArgs a;
  a.beta = beta; a.p1 = p1; a.p2 = p2; a.lb = layer_betas; a.E = n_edges; a.rt = rel_trans; a.rs = rel_sus;
  a.n_agents = n_agents; a.status = status; a.uni = uniforms; a.k0 = (uint32_t)seed; a.k1 = (uint32_t)(seed >> 32);
  a.day = day; a.variant = variant; a.layer = layer;
  dim3 grid((unsigned)ntiles, 2);
  k_infections_count<<<grid, INF_THREADS, 0, s>>>(a, ntiles, counts);
  k_scan<<<1, 1024, 0, s>>>(counts, m, offs, out_count, capacity, status);
  k_infections_write<<<grid, INF_THREADS, 0, s>>>(a, ntiles, offs, out_src, out_tgt, capacity);
  return launch_status();
}

}  // extern "C"
