// Device-side building blocks of the covgpu library (sm_103a).
//
// All float32 arithmetic that the reference performs in float32 is written as
// explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, ...) in the
// reference's left-to-right order, and the library is compiled with
// -fmad=false, so no product is contracted into an FMA: results are the
// reference's bit for bit.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "covgpu.h"

namespace covgpu {

// ---------------------------------------------------------------- state bits
// defaults.py:59-76 in order
constexpr uint32_t B_SUS = 1u << 0, B_NAIVE = 1u << 1, B_EXP = 1u << 2, B_INF = 1u << 3,
                   B_SYMP = 1u << 4, B_SEV = 1u << 5, B_CRIT = 1u << 6, B_TESTED = 1u << 7,
                   B_DIAG = 1u << 8, B_REC = 1u << 9, B_KDEAD = 1u << 10, B_DEAD = 1u << 11,
                   B_KCONT = 1u << 12, B_QUAR = 1u << 13, B_ISO = 1u << 14, B_VACC = 1u << 15;
constexpr int EXPV_SHIFT = 16, INFV_SHIFT = 24;
constexpr uint32_t BYVAR_MASK = 0xFFFF0000u;
constexpr uint32_t NOV = COVGPU_NO_VARIANT;

// per-sim-day integer result slots: flows (defaults.py:167-183) ...
enum { R_INFECTIONS = 0, R_REINFECTIONS, R_INFECTIOUS, R_SYMPTOMATIC, R_SEVERE, R_CRITICAL,
       R_RECOVERIES, R_DEATHS, R_TESTS, R_DIAGNOSES, R_KNOWN_DEATHS, R_QUARANTINED, R_ISOLATED,
       R_DOSES, R_VACCINATED,
       // ... then the stocks (defaults.py:145-159)
       R_N_FIRST = 15 };
constexpr int N_STOCKS = 13;
__device__ __constant__ uint32_t STOCK_BITS[N_STOCKS] = {
    B_SUS, B_EXP, B_INF, B_SYMP, B_SEV, B_CRIT, B_REC, B_DEAD, B_DIAG, B_KDEAD, B_QUAR, B_ISO, B_VACC};
// per-sim-day-variant slots
enum { RV_INFECTIONS = 0, RV_SYMPTOMATIC, RV_SEVERE, RV_INFECTIOUS, RV_N_EXPOSED, RV_N_INFECTIOUS };

// Day t is held back for a host step (a due rescaling): its day kernels return
// at once. The flag is written by an earlier kernel of the same sequence.
__device__ __forceinline__ bool held(const covgpu_state& st, int t) { return st.hold && *st.hold <= t; }

// ---------------------------------------------------------------- Philox-4x32-10
// Salmon et al., SC'11. Round constants and Weyl increments of that paper.
constexpr uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
constexpr uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;
constexpr uint32_t TAG_EDGE = 0x01000000u, TAG_INFECT = 0x03000000u;
constexpr uint32_t TAG_TEST = 0x04000000u, TAG_TRACE = 0x05000000u;

__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += PH_W0; k1 += PH_W1; }
    const uint32_t hi0 = __umulhi(PH_M0, c.x), lo0 = PH_M0 * c.x;
    const uint32_t hi1 = __umulhi(PH_M1, c.z), lo1 = PH_M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
  }
  return c;
}

// exact double in (0,1): (k + 0.5) * 2^-52 with k the top 26 bits of a and of b
__device__ __forceinline__ double u01_52(uint32_t a, uint32_t b) {
  const uint64_t k = ((uint64_t)(a >> 6) << 26) | (uint64_t)(b >> 6);
  return __dmul_rn(__dadd_rn((double)k, 0.5), 2.220446049250313080847263336181640625e-16);
}
// exact double in (0,1): (a + 0.5) * 2^-32
__device__ __forceinline__ double u01_32(uint32_t a) {
  return __dmul_rn(__dadd_rn((double)a, 0.5), 2.3283064365386962890625e-10);
}
// 2^32 mod n: the rejection threshold of an unbiased bounded draw (Lemire 2019,
// "Fast random integer generation in an interval"), the high half of x * n
// redrawn while its low half is below it
__host__ __device__ __forceinline__ uint32_t bounded_thr(uint32_t n) { return (uint32_t)(-n) % n; }

// ---------------------------------------------------------------- redrawn layers, per agent
// A layer redrawn every day (base.py:1849-1876, Layer.update with frac = 1) has E
// edges whose endpoints p1, p2 are i.i.d. uniform over the sim's n agents. The
// edges of agent a as p1 and as p2 are two lists: list d of a has k_d(a) ~
// Binomial(E, 1/n) entries, each partner uniform over the n agents. Transmission
// only ever needs the edges of the day's sources (an edge without a source
// endpoint infects nobody) and tracing only those of the traced agents, so the
// library draws the lists of those agents alone, keyed by (agent, day, layer):
//   counts   Philox (a, 0, day, TAG_DYN | layer): words x:y -> k_0, z:w -> k_1
//            (a 64-bit uniform U, k = the first k with U < cdf[k]);
//   partners Philox (a, 1 + d * 256 + (j >> 2), day, TAG_DYN | layer), word j & 3
//            -> partner j of list d (unbiased bounded draw; redraw r of entry j:
//            Philox (a, d << 10 | j, day, TAG_DYN_RETRY | r << 8 | layer), word x).
// An edge between two sources sits in both of their lists as independent draws;
// it carries no transmission either way (a source is never a target).
// Entry j of list d of agent a is the edge with identity dyn_edge_id(a, j): a
// bijection of a << 10 | j on 40 bits (a < 2^30, j < 2^10), so identities are
// distinct and their order, which decides the first infector among one layer's
// transmissions to the same target, is scrambled as the reference's i.i.d. edge
// order is.
constexpr uint32_t TAG_DYN = 0x08000000u, TAG_DYN_RETRY = 0x09000000u, TAG_DYN_HIT = 0x0A000000u;
constexpr int DYN_MAX_LIST = 1 << 10;  // entries of one list (the count table has at most this many)
constexpr uint64_t MASK40 = (1ull << 40) - 1;

__host__ __device__ __forceinline__ uint64_t dyn_edge_id(uint32_t a, uint32_t j, uint32_t day, uint32_t layer) {
  uint64_t x = (((uint64_t)a << 10) | j) ^ ((((uint64_t)day << 8) | layer) * 0x9E3779B97Full & MASK40);
  x = (x * 0xD6E8FEB86659Dull) & MASK40;  // odd multipliers: bijections modulo 2^40
  x ^= x >> 21;
  x = (x * 0xA0761D6478BDull) & MASK40;
  x ^= x >> 19;
  return x;
}

// the two list lengths of agent a: U = x:y (list 0), z:w (list 1); the first k with U < cdf[k]
// (cdf[kn - 1] = 2^64 - 1, so k < kn)
__device__ __forceinline__ int dyn_sample_k(const uint64_t* __restrict__ cdf, int kn, uint64_t u) {
  int lo = 0, hi = kn - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (u < __ldg(reinterpret_cast<const unsigned long long*>(cdf) + mid)) hi = mid; else lo = mid + 1;
  }
  return lo;
}
__device__ __forceinline__ void dyn_counts(const uint64_t* cdf, int kn, uint32_t a, uint32_t day, uint32_t layer,
                                           uint32_t k0, uint32_t k1, int& n0, int& n1) {
  const uint4 w = philox(make_uint4(a, 0u, day, TAG_DYN | layer), k0, k1);
  n0 = dyn_sample_k(cdf, kn, ((uint64_t)w.x << 32) | w.y);
  n1 = dyn_sample_k(cdf, kn, ((uint64_t)w.z << 32) | w.w);
}
// partner j of list d, given the word of its Philox block
__device__ __forceinline__ uint32_t dyn_partner(uint32_t x, uint32_t n, uint32_t thr, uint32_t a, int d, int j,
                                               uint32_t day, uint32_t layer, uint32_t k0, uint32_t k1) {
  uint64_t m = (uint64_t)x * n;
  for (uint32_t r = 0; (uint32_t)m < thr && r < 16; ++r) {
    const uint4 w = philox(make_uint4(a, ((uint32_t)d << 10) | (uint32_t)j, day, TAG_DYN_RETRY | (r << 8) | layer), k0, k1);
    m = (uint64_t)w.x * n;
  }
  return (uint32_t)(m >> 32);
}
__device__ __forceinline__ uint4 dyn_partner_block(uint32_t a, int d, int j, uint32_t day, uint32_t layer, uint32_t k0,
                                                   uint32_t k1) {
  return philox(make_uint4(a, 1u + ((uint32_t)d << 8) + ((uint32_t)j >> 2), day, TAG_DYN | layer), k0, k1);
}
__device__ __forceinline__ uint32_t word_of(const uint4& w, int k) {
  return k == 0 ? w.x : (k == 1 ? w.y : (k == 2 ? w.z : w.w));
}

// Thinning of a source's list entries. Every entry of source s's lists in a
// layer transmits with p(s, g) = beta * rel_trans'(s) * rel_sus'(g) <= pmax(s) =
// beta * rel_trans'(s) * rse_max (rse_max bounds rel_sus' over the sim's agents).
// An entry is first a potential transmission with probability 2^-m, the power
// of two just above pmax (m = thin_shift(pmax)), decided by the top m bits of
// one 32-bit word of Philox (a, d * 256 + j / 4, day, TAG_DYN_HIT | layer); only
// then is its partner drawn, and it transmits when u < p * 2^m (u the edge's
// Bernoulli uniform, p * 2^m exact in float32). So P(transmission) = p, with one
// 32-bit word per entry instead of a partner, a gather and a Bernoulli draw.
__device__ __forceinline__ int thin_shift(float pmax) {
  if (pmax >= 1.0f) return 0;
  const int ex = (int)((__float_as_uint(pmax) >> 23) & 0xffu);  // pmax in [2^(ex-127), 2^(ex-126))
  return ex == 0 ? 32 : min(32, 126 - ex);
}
__device__ __forceinline__ bool thin_potential(uint32_t w, int m) {
  return m == 0 || (w >> (32 - m)) == 0u;
}
__device__ __forceinline__ uint4 dyn_hit_block(uint32_t a, int d, int j, uint32_t day, uint32_t layer, uint32_t k0,
                                               uint32_t k1) {
  return philox(make_uint4(a, ((uint32_t)d << 8) + ((uint32_t)j >> 2), day, TAG_DYN_HIT | layer), k0, k1);
}

// 32 x 32 bit-matrix transpose across a warp (row j = lane j's x): bit j of lane
// k's result is bit k of lane j's x, so lane k holds the ballot of bit k and its
// popcount counts the lanes with bit k set. Five exchange stages, each swapping
// the off-diagonal blocks of half the previous size. All 32 lanes call it.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int s = 16 >> k;
    const uint32_t m = k == 0 ? 0x0000FFFFu : k == 1 ? 0x00FF00FFu : k == 2 ? 0x0F0F0F0Fu
                     : k == 3 ? 0x33333333u : 0x55555555u;  // the bits b with (b & s) == 0
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, s);
    x = (lane & s) ? ((x & ~m) | ((y >> s) & m)) : ((x & m) | ((y & m) << s));
  }
  return x;
}

// The set bits of one agent block's bitmap words, handed to the lanes 32 at a
// time: lanes 0..nw-1 hold the words (nw warp-uniform, <= 32), warp_bits_scan
// forms their exclusive prefix counts, and warp_bits_nth gives the lane whose
// word holds the idx-th set bit (idx < total) and the bit's position in it.
// All 32 lanes call both.
struct WarpBits {
  uint32_t word;
  int pre, total;
};
__device__ __forceinline__ WarpBits warp_bits_scan(uint32_t word) {
  const int lane = threadIdx.x & 31;
  const int cnt = __popc(word);
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int x = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += x;
  }
  WarpBits r;
  r.word = word;
  r.pre = inc - cnt;
  r.total = __shfl_sync(0xffffffffu, inc, 31);
  return r;
}
__device__ __forceinline__ int warp_bits_nth(const WarpBits& wb, int nw, int idx, int& bit) {
  int src = 0;
  for (int k = 1; k < nw; ++k)
    if (__shfl_sync(0xffffffffu, wb.pre, k) <= idx) src = k;
  const uint32_t wd = __shfl_sync(0xffffffffu, wb.word, src);
  const int pk = __shfl_sync(0xffffffffu, wb.pre, src);
  const int r = idx - pk;
  bit = (r >= 0 && r < __popc(wd)) ? (int)__fns(wd, 0u, r + 1) : 0;
  return src;
}

// floor(x * n / 2^64) for x = a:b
__device__ __forceinline__ int64_t uniform_index(uint32_t a, uint32_t b, uint64_t n) {
  const uint64_t x = ((uint64_t)a << 32) | b;
  return (int64_t)__umul64hi(x, n);
}
// ---------------------------------------------------------------- small helpers
// Read-only global loads with an L1 policy (the data is not written while the
// kernel runs). COVGPU_L1_HINTS selects them: bit 0 keeps the source bitmap in
// L1 (evict_last), bit 1 streams the edge lists past L1 (no_allocate). L2
// policy is the default: the edge lists stay L2-resident from day to day.
// Streaming the edge lists past L1 shortened a 1M-agent, 180-day run by 7%
// (the agent and infect passes gained most); sending the candidates' agent
// gathers past L1 as well lengthened it (sources recur across edges).
#ifndef COVGPU_L1_HINTS
#define COVGPU_L1_HINTS 3
#endif
__device__ __forceinline__ int4 ld_stream_v4(const int32_t* p) {
#if COVGPU_L1_HINTS & 2
  int4 v;
  asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  return v;
#else
  return __ldg(reinterpret_cast<const int4*>(p));
#endif
}
__device__ __forceinline__ uint32_t ld_keep_u32(const uint32_t* p) {
#if COVGPU_L1_HINTS & 1
  uint32_t v;
  asm("ld.global.nc.L1::evict_last.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
#else
  return __ldg(p);
#endif
}

__device__ __forceinline__ float f32nan() { return __int_as_float(0x7fc00000); }
__device__ __forceinline__ bool defined(float x) { return !isnan(x); }
__device__ __forceinline__ float* date_row(const covgpu_state& st, int d) { return st.dates + (int64_t)d * st.n; }
// words of each role bitmap (source bitmap first, then target bitmap)
__device__ __forceinline__ int64_t roles_words(const covgpu_state& st) { return (st.n + 31) >> 5; }
__device__ __forceinline__ float* dur_row(const covgpu_state& st, int d) { return st.durs + (int64_t)d * st.n; }

// utils.py:39-79 for one agent, float32 as numba types it (the int32 t and the
// float32 arrays meet in a float32 ufunc loop).
__device__ __forceinline__ float viral_load_one(int t, float ts, float tr, float td, float frac_time,
                                                float load_ratio, float high_cap) {
  const float stop = isnan(td) ? tr : td;
  const float total = __fsub_rn(stop, ts);
  const float trans_day = __fmul_rn(frac_time, total);
  const float trans_point = (trans_day > high_cap) ? __fdiv_rn(high_cap, total) : frac_time;
  const bool early = __fdiv_rn(__fsub_rn((float)t, ts), total) < trans_point;
  const float den = __fadd_rn(1.0f, __fmul_rn(frac_time, __fsub_rn(load_ratio, 1.0f)));
  return __fdiv_rn(early ? load_ratio : 1.0f, den);
}


// ---------------------------------------------------------------- block reduction helpers
__device__ __forceinline__ long long warp_sum_ll(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}
// warp sum of the non-negative fixed-point values: two 32-bit reductions of the
// 20-bit low and 27-bit high parts when every lane's x < 2^47 (their sums over 32
// lanes cannot overflow), else the 64-bit shuffle sum
__device__ __forceinline__ long long warp_sum_fx(long long x) {
  if (__any_sync(0xffffffffu, (unsigned long long)x >= (1ull << 47))) return warp_sum_ll(x);
  const unsigned lo = __reduce_add_sync(0xffffffffu, (unsigned)(x & 0xFFFFF));
  const unsigned hi = __reduce_add_sync(0xffffffffu, (unsigned)(x >> 20));
  return ((long long)hi << 20) + (long long)lo;
}

}  // namespace covgpu
