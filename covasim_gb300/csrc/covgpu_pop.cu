// covgpu_pop: synthetic populations built on the device (sm_103a).
//
// The same distributions as Covasim 3.1.7's generators (covasim/population.py):
// ages by bin weight then uniform within the bin (population.py:196-204),
// random layers with round(Poisson(n)/2) (or negative-binomial) partners per
// member drawn uniformly among the members (population.py:241-284), household
// clusters of Poisson(h) consecutive agents with every pair inside a cluster
// once (population.py:287-329), and the prognoses with negative-binomial
// rel_trans (people.py:139-161). The reference loops over agents in Python;
// here each agent, member or cluster is one thread and the variable-length
// outputs are placed by exclusive scans. Draws are Philox-4x32-10 keyed by
// (seed, purpose, layer, index), so a population depends only on its seed.
//
// Every rejection loop is bounded; a loop that runs out sets an error bit in
// the caller's status word and returns a valid value.
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_scan.cuh"

using namespace covgpu;

namespace {

constexpr uint32_t TAG_POP = 0x06000000u;  // | purpose << 16 | layer
enum { POP_AGE = 1, POP_COUNT = 2, POP_PARTNER = 3, POP_CLUSTER = 4, POP_TRANS = 5 };
constexpr int POP_THREADS = 256;
constexpr int MAX_TRIES = 1000;                           // bound of every rejection loop

inline int status_of_launch() { return cudaGetLastError() == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR; }
inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline unsigned blocks_for(int64_t n, int per_block) {
  int64_t b = (n + per_block - 1) / per_block;
  return (unsigned)(b < 1 ? 1 : b);
}

// A stream of uniform doubles in (0, 1) for one index: Philox blocks
// (index_lo, index_hi, block, tag), two 52-bit uniforms per block.
struct UStream {
  uint32_t k0, k1, lo, hi, tag, block;
  uint4 w;
  int left;
  __device__ UStream(uint64_t seed, uint32_t tag_, int64_t index)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), lo((uint32_t)index), hi((uint32_t)((uint64_t)index >> 32)),
        tag(tag_), block(0), left(0) {}
  __device__ double next() {
    if (left == 0) {
      w = philox(make_uint4(lo, hi, block++, tag), k0, k1);
      left = 2;
      return u01_52(w.x, w.y);
    }
    left = 0;
    return u01_52(w.z, w.w);
  }
  __device__ uint64_t next64() {  // 64 random bits (for uniform_index)
    const uint4 v = philox(make_uint4(lo, hi, block++, tag), k0, k1);
    return ((uint64_t)v.x << 32) | v.y;
  }
};

__device__ double std_normal(UStream& r) {  // Box-Muller, one of the pair
  const double u1 = r.next(), u2 = r.next();
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// Poisson(lam): inversion below 10, else the transformed rejection with squeeze
// of Hörmann (1993, "The transformed rejection method for generating Poisson
// random variables", algorithm PTRS).
__device__ int64_t poisson(UStream& r, double lam, int* status) {
  if (!(lam > 0.0)) return 0;
  if (lam < 10.0) {
    const double u = r.next();
    double p = exp(-lam), s = p;
    int64_t k = 0;
    while (u > s && k < 4 * MAX_TRIES) {
      ++k;
      p *= lam / (double)k;
      s += p;
    }
    return k;
  }
  const double slam = sqrt(lam), loglam = log(lam);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < MAX_TRIES; ++it) {
    const double U = r.next() - 0.5, V = r.next();
    const double us = 0.5 - fabs(U);
    const double kd = floor((2.0 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return (int64_t)kd;
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + kd * loglam - lgamma(kd + 1.0)) return (int64_t)kd;
  }
  atomicOr(status, COVGPU_TIMEOUT);
  return (int64_t)floor(lam + 0.5);
}

// Gamma(shape, 1): Marsaglia and Tsang (2000); shape < 1 by Gamma(shape + 1) * U^(1/shape).
__device__ double gamma1(UStream& r, double shape, int* status) {
  if (!(shape > 0.0)) return 0.0;
  double boost = 1.0;
  if (shape < 1.0) {
    boost = pow(r.next(), 1.0 / shape);
    shape += 1.0;
  }
  const double d = shape - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (int it = 0; it < MAX_TRIES; ++it) {
    const double x = std_normal(r);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    const double u = r.next();
    if (log(u) < 0.5 * x * x + d - d * v + d * log(v)) return d * v * boost;
  }
  atomicOr(status, COVGPU_TIMEOUT);
  return shape * boost;
}

// numpy's negative_binomial(n, p): Poisson(Gamma(n, (1 - p) / p))
__device__ int64_t neg_binomial(UStream& r, double n, double p, int* status) {
  return poisson(r, gamma1(r, n, status) * (1.0 - p) / p, status);
}

// ------------------------------------------------------------------ scans (covgpu_scan.cuh)
// ------------------------------------------------------------------ kernels
__global__ void k_pop_ages(int64_t n, const double* lo, const double* width, const double* cdf, int n_bins,
                           uint64_t seed, float* age, int32_t* sex) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  UStream r(seed, TAG_POP | (POP_AGE << 16), i);
  const double u = r.next() * cdf[n_bins - 1];
  int b = 0;
  while (b < n_bins - 1 && u > cdf[b]) ++b;
  age[i] = (float)(lo[b] + width[b] * r.next());
  if (sex) sex[i] = r.next() < 0.5 ? 1 : 0;
}

// members of an age range: flags for the scan, then the scatter
__global__ void k_pop_age_flags(int64_t n, const float* age, float lo, float hi, int64_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = (age[i] >= lo && age[i] < hi) ? 1 : 0;
}
__global__ void k_pop_scatter_members(int64_t n, const int64_t* flags, const int64_t* pos, int32_t* members) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flags[i]) members[pos[i]] = (int32_t)i;
}

// partners per member: round(X / 2) half to even, X ~ Poisson(mean) or NB
__global__ void k_pop_counts(int64_t n_members, double mean, double dispersion, uint64_t seed, int layer,
                             int64_t* counts, int* status) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_members) return;
  UStream r(seed, TAG_POP | (POP_COUNT << 16) | (uint32_t)layer, m);
  int64_t x;
  if (dispersion > 0.0) x = neg_binomial(r, dispersion, dispersion / (mean + dispersion), status);
  else x = poisson(r, mean, status);
  const int64_t h = x >> 1;
  counts[m] = h + ((x & 1) && (h & 1) ? 1 : 0);  // np.round(x / 2): halves to even
}

__global__ void k_pop_fill_random(int64_t n_members, const int32_t* members, const int64_t* offsets, uint64_t seed,
                                  int layer, int32_t* p1, int32_t* p2) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_members) return;
  const int32_t self = members ? members[m] : (int32_t)m;
  for (int64_t j = offsets[m]; j < offsets[m + 1]; ++j) {
    UStream r(seed, TAG_POP | (POP_PARTNER << 16) | (uint32_t)layer, j);
    const uint64_t x = r.next64();
    const int64_t k = uniform_index((uint32_t)(x >> 32), (uint32_t)x, (uint64_t)n_members);
    p1[j] = self;
    p2[j] = members ? members[k] : (int32_t)k;
  }
}

__global__ void k_pop_cluster_sizes(int64_t n_clusters, double mean, uint64_t seed, int layer, int64_t* sizes,
                                    int* status) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_clusters) return;
  UStream r(seed, TAG_POP | (POP_CLUSTER << 16) | (uint32_t)layer, k);
  sizes[k] = poisson(r, mean, status);
}

// pairs (i, j > i) in agent i's cluster (clusters truncated at n)
__global__ void k_pop_cluster_targets(int64_t n, int64_t n_clusters, const int64_t* starts, int64_t* counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t lo = 0, hi = n_clusters;  // last cluster with start <= i
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (starts[mid] <= i) lo = mid; else hi = mid;
  }
  int64_t end = starts[lo + 1];
  if (end > n) end = n;
  counts[i] = end - i - 1 > 0 ? end - i - 1 : 0;
}

__global__ void k_pop_fill_cluster(int64_t n, const int64_t* offsets, int32_t* p1, int32_t* p2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = offsets[i], c = offsets[i + 1] - o;
  for (int64_t j = 0; j < c; ++j) {
    p1[o + j] = (int32_t)i;
    p2[o + j] = (int32_t)(i + 1 + j);
  }
}

// people.py:139-161: per-agent prognoses from the age bin; rel_trans = trans_OR * draw
__global__ void k_pop_prognoses(int64_t n, const float* age, const double* cutoffs, int n_bins, const double* tables,
                                int trans_dist, double par1, double par2, double step, uint64_t seed, float* symp,
                                float* severe, float* crit, float* death, float* rel_sus, float* rel_trans,
                                int* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = (double)age[i];
  int b = 0;  // np.digitize(age, cutoffs) - 1
  while (b + 1 < n_bins && cutoffs[b + 1] <= a) ++b;
  symp[i] = (float)tables[0 * n_bins + b];
  severe[i] = (float)tables[1 * n_bins + b];
  crit[i] = (float)tables[2 * n_bins + b];
  death[i] = (float)tables[3 * n_bins + b];
  rel_sus[i] = (float)tables[4 * n_bins + b];
  UStream r(seed, TAG_POP | (POP_TRANS << 16), i);
  double draw;
  if (trans_dist == 0) {  // neg_binomial(mean par1, dispersion par2) in units of step
    const double p = par2 / (par1 / step + par2);
    draw = (double)neg_binomial(r, par2, p, status) * step;
  } else {  // lognormal with mean par1 and sd par2
    const double mu = log(par1 * par1 / sqrt(par2 * par2 + par1 * par1));
    const double sg = sqrt(log(par2 * par2 / (par1 * par1) + 1.0));
    draw = exp(mu + sg * std_normal(r));
  }
  rel_trans[i] = (float)(tables[5 * n_bins + b] * draw);
}

}  // namespace

extern "C" {

int64_t covgpu_pop_scan_scratch(int64_t n) { return (int64_t)blocks_for(n, SCAN_TILE); }

int covgpu_pop_ages(int64_t n, const double* bin_lo, const double* bin_width, const double* bin_cdf, int32_t n_bins,
                    uint64_t seed, float* age, int32_t* sex, void* stream) {
  if (n < 0 || n_bins < 1 || (n > 0 && (!bin_lo || !bin_width || !bin_cdf || !age))) return COVGPU_BADARG;
  if (n == 0) return COVGPU_OK;
  k_pop_ages<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, S(stream)>>>(n, bin_lo, bin_width, bin_cdf, n_bins, seed,
                                                                         age, sex);
  return status_of_launch();
}

int covgpu_pop_members(int64_t n, const float* age, float age_lo, float age_hi, int64_t* flags, int64_t* pos,
                       int64_t* scratch, int32_t* members, void* stream) {
  if (n < 1 || !age || !flags || !pos || !scratch || !members) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  k_pop_age_flags<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, s>>>(n, age, age_lo, age_hi, flags);
  int rc = scan_i64(flags, pos, n, scratch, s);
  if (rc) return rc;
  k_pop_scatter_members<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, s>>>(n, flags, pos, members);
  return status_of_launch();
}

int covgpu_pop_random_counts(int64_t n_members, double mean, double dispersion, uint64_t seed, int32_t layer,
                             int64_t* counts, int64_t* offsets, int64_t* scratch, int32_t* status, void* stream) {
  if (n_members < 1 || !counts || !offsets || !scratch || !status || !(mean >= 0.0)) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  k_pop_counts<<<blocks_for(n_members, POP_THREADS), POP_THREADS, 0, s>>>(n_members, mean, dispersion, seed, layer,
                                                                           counts, status);
  return scan_i64(counts, offsets, n_members, scratch, s);
}

int covgpu_pop_random_fill(int64_t n_members, const int32_t* members, const int64_t* offsets, uint64_t seed,
                           int32_t layer, int32_t* p1, int32_t* p2, void* stream) {
  if (n_members < 1 || !offsets || !p1 || !p2) return COVGPU_BADARG;
  k_pop_fill_random<<<blocks_for(n_members, POP_THREADS), POP_THREADS, 0, S(stream)>>>(n_members, members, offsets,
                                                                                       seed, layer, p1, p2);
  return status_of_launch();
}

int covgpu_pop_cluster_sizes(int64_t n_clusters, double mean, uint64_t seed, int32_t layer, int64_t* sizes,
                             int64_t* starts, int64_t* scratch, int32_t* status, void* stream) {
  if (n_clusters < 1 || !sizes || !starts || !scratch || !status || !(mean >= 0.0)) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  k_pop_cluster_sizes<<<blocks_for(n_clusters, POP_THREADS), POP_THREADS, 0, s>>>(n_clusters, mean, seed, layer,
                                                                                   sizes, status);
  return scan_i64(sizes, starts, n_clusters, scratch, s);
}

int covgpu_pop_cluster_counts(int64_t n, int64_t n_clusters, const int64_t* starts, int64_t* counts,
                              int64_t* offsets, int64_t* scratch, void* stream) {
  if (n < 1 || n_clusters < 1 || !starts || !counts || !offsets || !scratch) return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  k_pop_cluster_targets<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, s>>>(n, n_clusters, starts, counts);
  return scan_i64(counts, offsets, n, scratch, s);
}

int covgpu_pop_cluster_fill(int64_t n, const int64_t* offsets, int32_t* p1, int32_t* p2, void* stream) {
  if (n < 1 || !offsets || !p1 || !p2) return COVGPU_BADARG;
  k_pop_fill_cluster<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, S(stream)>>>(n, offsets, p1, p2);
  return status_of_launch();
}

int covgpu_pop_prognoses(int64_t n, const float* age, const double* cutoffs, int32_t n_bins, const double* tables,
                         int32_t trans_dist, double par1, double par2, double step, uint64_t seed, float* symp,
                         float* severe, float* crit, float* death, float* rel_sus, float* rel_trans, int32_t* status,
                         void* stream) {
  if (n < 0 || n_bins < 1 || (trans_dist != 0 && trans_dist != 1)) return COVGPU_BADARG;
  if (n == 0) return COVGPU_OK;
  if (!age || !cutoffs || !tables || !symp || !severe || !crit || !death || !rel_sus || !rel_trans || !status)
    return COVGPU_BADARG;
  if (trans_dist == 0 && !(par1 > 0.0 && par2 > 0.0 && step > 0.0)) return COVGPU_BADARG;
  k_pop_prognoses<<<blocks_for(n, POP_THREADS), POP_THREADS, 0, S(stream)>>>(
      n, age, cutoffs, n_bins, tables, trans_dist, par1, par2, step, seed, symp, severe, crit, death, rel_sus,
      rel_trans, status);
  return status_of_launch();
}

}  // extern "C"
