// covgpu_testing: test_prob, contact_tracing and update_states_post on the device
// (covasim/interventions.py:858-1145, covasim/people.py:189-196,315-366,589-640),
// and the agent index of stored layers that tracing walks.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_ff.cuh"
#include "covgpu_scan.cuh"
#include "covgpu_launch.cuh"

using namespace covgpu;

namespace {

// ============================================================ testing and tracing
//
// Day t with a test_prob / contact_tracing sim, after the agent pass and any
// importations (sim.py:596-600): k_test_pass draws who tests and marks the
// agents to trace, k_trace_scan marks their contacts layer by layer, and
// k_post_pass notifies the contacts and runs update_states_post.

__device__ __forceinline__ bool day_active(int t, int start, int end) { return t >= start && t <= end; }

// interventions.py:682-710: is agent i a quarantined tester on day t?
__device__ __forceinline__ bool quar_tester(const covgpu_state& st, const covgpu_testing& T, int64_t i, int t,
                                            uint32_t f) {
  const int qp = T.quar_policy;
  if (!qp) return false;
  bool q = false;
  if (qp & (COVGPU_QP_START | COVGPU_QP_OFFSETS)) {
    const float dq = date_row(st, COVGPU_DATE_QUARANTINED)[i];
    if ((qp & COVGPU_QP_START) && dq == (float)(t - 1)) q = true;
    if ((qp & COVGPU_QP_OFFSETS) && defined(dq)) {
      const float back = (float)(t - 1) - dq;  // exact: both are small integers when it matters
      if (back >= 0.0f && back < 32.0f && back == floorf(back) && ((T.quar_offsets >> (int)back) & 1u)) q = true;
    }
  }
  if ((qp & COVGPU_QP_END) && date_row(st, COVGPU_DATE_END_QUARANTINE)[i] == (float)(t + 1)) q = true;
  if ((qp & COVGPU_QP_DAILY) && (f & B_QUAR)) q = true;
  return q;
}

// whole days since symptom onset, as test_prob forms them: the float32 difference
// t - date_symptomatic truncated to int32 (cvd.default_int)
__device__ __forceinline__ int symp_days(const covgpu_state& st, int64_t i, int t) {
  return (int)__fsub_rn((float)t, date_row(st, COVGPU_DATE_SYMPTOMATIC)[i]);
}

// ceil(p * 2^53) (the host's prob_threshold): the Bernoulli threshold of a float64 p
__device__ __forceinline__ uint64_t prob_thr(double p) {
  if (!(p > 0.0)) return 0ull;
  if (p >= 1.0) return (1ull << 53) + 1ull;
  return __double2ull_ru(__dmul_rn(p, 9007199254740992.0));
}

// test_prob's symptomatic probability under a swab delay (interventions.py:930-938):
// pdf(days) * adjusted symp_prob * (symptomatic agents / those with the same days),
// in float64 with the reference's operations and order
__device__ __forceinline__ uint64_t swab_threshold(const covgpu_state& st, const covgpu_testing& T, int64_t i, int t) {
  const int d = symp_days(st, i, t);
  if (d < 0 || d >= T.swab_len) return 0ull;
  const double inv = __ddiv_rn((double)T.swab_bins[d], (double)T.swab_bins[T.swab_len]);
  const double cnt = __ddiv_rn(1.0, inv);
  const double x = __dmul_rn((double)d, T.symp_prob);
  const double adj = 1.0 > x ? __ddiv_rn(T.symp_prob, __dsub_rn(1.0, x)) : 1.0;
  return prob_thr(__dmul_rn(__dmul_rn(T.swab_pdf[d], adj), cnt));
}

// test_prob.apply (interventions.py:921-981) + People.test (people.py:589-617),
// then the trace bits of contact_tracing.select_cases (interventions.py:1066-1072)
// One agent block of the test pass (thread k on agent begin + k); the tested are
// counted into the thread's accumulator
__device__ __forceinline__ void test_block(const covgpu_state& st, int t, const covgpu_agent_block& blk,
                                           unsigned& tested_acc) {
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const covgpu_testing& T = sp.testing;
  const bool test_on = day_active(t, T.test_start, T.test_end);
  const bool trace_on = day_active(t, T.trace_start, T.trace_end);
  if (!test_on && !trace_on) return;  // uniform over the agent block (one sim per agent block)
  const int64_t i = blk.begin + threadIdx.x;
  const bool valid = i < blk.end;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t tested = 0, trace = 0;
  if (valid) {
    uint32_t f = st.flags[i];
    float* d_diag = date_row(st, COVGPU_DATE_DIAGNOSED) + i;
    float dd = *d_diag;  // loaded with the flags; kept current below
    if (test_on) {
      uint64_t thr = 0;
      if (!(f & B_DIAG)) {  // the diagnosed do not test
        const bool symp = f & B_SYMP;
        const int64_t loc = i - sp.agent_off;
        // an influenza-like illness without COVID symptoms: the symptomatic probability,
        // never the quarantine ones (interventions.py:966-969)
        if (!symp && T.ili_mark && T.ili_mark[loc] == t)
          thr = T.thr_symp;
        else if (quar_tester(st, T, i, t, f))
          thr = symp ? T.thr_symp_quar : T.thr_asymp_quar;
        else
          thr = !symp ? T.thr_asymp : (T.swab_pdf ? swab_threshold(st, T, i, t) : T.thr_symp);
        if (T.sub_thr) {  // subtargets (interventions.py:970-972)
          const uint64_t sv = T.sub_thr[loc];
          if (sv != COVGPU_NO_SUBTARGET) thr = sv;
        }
      }
      if (thr) {
        const uint32_t local = (uint32_t)(i - sp.agent_off);
        const uint4 w = philox(make_uint4(local, 0u, (uint32_t)t, TAG_TEST), sp.key0, sp.key1);
        if (bern52_thr(w.x, w.y, thr)) {
          tested = 1;
          st.flags[i] = f | B_TESTED;
          date_row(st, COVGPU_DATE_TESTED)[i] = (float)t;
          if ((f & B_INF) && bern52_thr(w.z, w.w, T.thr_sensitivity) && isnan(dd)) {
            const uint4 w1 = philox(make_uint4(local, 1u, (uint32_t)t, TAG_TEST), sp.key0, sp.key1);
            if (bern52_thr(w1.x, w1.y, T.thr_not_lost)) {
              dd = (float)(t + T.test_delay);
              *d_diag = dd;
              date_row(st, COVGPU_DATE_POS_TEST)[i] = (float)t;
            }
          }
        }
      }
    }
    if (trace_on) {
      if (T.presumptive)
        trace = (date_row(st, COVGPU_DATE_TESTED)[i] == (float)t && (f & B_EXP)) ? 1u : 0u;
      else
        trace = (dd == (float)t) ? 1u : 0u;
    }
  }
  const uint32_t tm = __ballot_sync(0xffffffffu, trace);
  if (trace_on && lane == 0 && blk.begin + warp * 32 < blk.end) st.trace_bits[(blk.begin + warp * 32) >> 5] = tm;
  if (tm && T.cap_list) {  // the day's cases, for the capacity's selection (k_trace_cap)
    uint32_t base = 0u;
    if (lane == 0) base = atomicAdd(T.cap_count, (uint32_t)__popc(tm));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (trace) T.cap_list[base + __popc(tm & ((1u << lane) - 1u))] = (int32_t)(i - sp.agent_off);
  }
  tested_acc += tested;
  if (lane == 0 && tm) atomicAdd(st.trace_count + blk.sim, (unsigned)__popc(tm));
}

__device__ __forceinline__ void test_flush(const covgpu_state& st, int t, int sim, unsigned& tested_acc) {
  const unsigned n_tested = __reduce_add_sync(0xffffffffu, tested_acc);
  if ((threadIdx.x & 31) == 0 && n_tested)
    atomicAdd(reinterpret_cast<unsigned long long*>(&st.sims[sim].res_int[(int64_t)t * COVGPU_N_RES_INT + R_TESTS]),
              (unsigned long long)n_tested);
  tested_acc = 0;
}

// The per-sim preparation of day t's test pass, one block per sim:
// test_prob's swab-delay histogram is cleared (k_swab_hist fills it), and the
// day's influenza-like illnesses (interventions.py:941-947), drawn on the host
// (they do not depend on the state), are marked with t.
__global__ void k_test_prep(covgpu_state st, int t) {
  if (held(st, t)) return;
  const int s = blockIdx.x;
  if (s >= st.n_sims) return;
  const covgpu_testing& T = st.sims[s].testing;
  if (!day_active(t, T.test_start, T.test_end)) return;
  if (T.swab_pdf)
    for (int k = threadIdx.x; k <= T.swab_len; k += blockDim.x) T.swab_bins[k] = 0;
  if (T.cap_list && threadIdx.x == 0) *T.cap_count = 0u;
  if (!T.ili_mark) return;
  const int d = t - T.test_start;
  if (d < 0 || d >= T.ili_days) return;
  const int n = st.sims[s].n_agents;
  for (int64_t k = T.ili_off[d] + threadIdx.x; k < T.ili_off[d + 1]; k += blockDim.x) {
    const int32_t a = T.ili_inds[k];
    if (a >= 0 && a < n) T.ili_mark[a] = t;
  }
}

// The passes over agents run as (at most) one wave of blocks, each walking a
// contiguous range of agent blocks [b, b_end); counts are flushed once per sim.
__device__ __forceinline__ bool agent_range(const covgpu_state& st, int64_t& b, int64_t& b_end) {
  const int64_t nb = st.n_agent_blocks;
  const int64_t per = (nb + gridDim.x - 1) / gridDim.x;
  b = (int64_t)blockIdx.x * per;
  b_end = min(nb, b + per);
  return b < b_end;
}

// test_prob's swab-delay histogram of day t (interventions.py:931-932): the
// symptomatic agents by whole days since onset, and their total in the last bin
__global__ void __launch_bounds__(AGENT_THREADS) k_swab_hist(covgpu_state st, int t) {
  if (held(st, t)) return;
  int64_t b, b_end;
  if (!agent_range(st, b, b_end)) return;
  for (; b < b_end; ++b) {
    const covgpu_agent_block blk = st.agent_blocks[b];
    const covgpu_testing& T = st.sims[blk.sim].testing;
    if (!T.swab_pdf || !day_active(t, T.test_start, T.test_end)) continue;  // uniform over the agent block
    const int64_t i = blk.begin + threadIdx.x;
    if (i >= blk.end || !(st.flags[i] & B_SYMP)) continue;
    const int d = symp_days(st, i, t);
    if (d >= 0 && d < T.swab_len) atomicAdd(T.swab_bins + d, 1);
    atomicAdd(T.swab_bins + T.swab_len, 1);
  }
}

// contact_tracing's capacity (interventions.py:1074-1078), one block per sim: when
// the day's cases exceed int(capacity / scale), a radix select over their unique
// 64-bit keys finds the capacity-th smallest, and the trace bits of the cases above
// it are cleared (a uniform random subset of exactly that size)
__device__ __forceinline__ uint64_t cap_key(const covgpu_sim_params& sp, int32_t local, int t) {
  const uint4 w = philox(make_uint4((uint32_t)local, 2u, (uint32_t)t, TAG_TEST), sp.key0, sp.key1);
  return ((uint64_t)w.x << 32) | (uint32_t)local;
}
__global__ void k_trace_cap(covgpu_state st, int t) {
  if (held(st, t)) return;
  const int s = blockIdx.x;
  if (s >= st.n_sims) return;
  const covgpu_sim_params& sp = st.sims[s];
  const covgpu_testing& T = sp.testing;
  if (!T.cap_list || !day_active(t, T.trace_start, T.trace_end)) return;
  const double scale = sp.rescale_vec ? sp.rescale_vec[t] : T.cap_scale;
  const double capd = T.capacity / scale;
  const uint32_t c = *T.cap_count;
  const int64_t cap = capd < 0.0 ? 0 : (int64_t)capd;
  if ((int64_t)c <= cap) return;
  __shared__ unsigned int hist[256];
  __shared__ unsigned long long s_prefix;
  __shared__ unsigned int s_rank;
  unsigned long long prefix = 0ull, mask = 0ull;
  unsigned int rank = (unsigned int)cap;  // the rank (1-based) of the largest key kept
  if (rank > 0) {
    for (int shift = 56; shift >= 0; shift -= 8) {
      for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0u;
      __syncthreads();
      for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
        const uint64_t key = cap_key(sp, T.cap_list[j], t);
        if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned int cum = 0u;
        int d = 0;
        while (d < 255 && cum + hist[d] < rank) cum += hist[d++];
        s_prefix = prefix | ((unsigned long long)d << shift);
        s_rank = rank - cum;
      }
      __syncthreads();
      prefix = s_prefix;
      rank = s_rank;
      mask |= 0xFFull << shift;
      __syncthreads();
    }
  }
  for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
    const int32_t local = T.cap_list[j];
    if (cap == 0 || cap_key(sp, local, t) > prefix) {
      const int64_t i = sp.agent_off + local;
      atomicAnd(st.trace_bits + (i >> 5), ~(1u << (i & 31)));
    }
  }
  if (threadIdx.x == 0) st.trace_count[s] = (uint32_t)cap;
}

__global__ void __launch_bounds__(AGENT_THREADS) k_test_pass(covgpu_state st, int t) {
  if (held(st, t)) return;
  int64_t b, b_end;
  if (!agent_range(st, b, b_end)) return;
  int sim = st.agent_blocks[b].sim;
  unsigned tested_acc = 0;
  for (; b < b_end; ++b) {
    const covgpu_agent_block blk = st.agent_blocks[b];
    if (blk.sim != sim) {
      test_flush(st, t, sim, tested_acc);
      sim = blk.sim;
    }
    test_block(st, t, blk, tested_acc);
  }
  test_flush(st, t, sim, tested_acc);
}

__device__ __forceinline__ uint32_t bit_of(const uint32_t* __restrict__ bits, int32_t a) {
  return (__ldg(bits + (a >> 5)) >> (a & 31)) & 1u;
}

// contact_tracing.identify_contacts, the find_contacts half (utils.py:131-147):
// every edge of a stored layer without an index with a traced endpoint marks the
// other endpoint in its layer's bitmap (dynamic layers: k_trace_dyn)
template <int ROUNDS>
__global__ void __launch_bounds__(EDGE_THREADS) k_trace_scan(covgpu_state st, int t) {
  if (held(st, t)) return;
  constexpr int64_t TILE = (int64_t)ROUNDS * EDGE_ROUND;
  __shared__ int s_seg;
  if (threadIdx.x == 0) {
    int lo = 0, hi = st.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (st.segments[mid].tile_begin <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    s_seg = lo;
  }
  __syncthreads();
  const covgpu_layer* L = st.segments + s_seg;
  const covgpu_sim_params& sp = st.sims[L->sim];
  const covgpu_testing& T = sp.testing;
  if (!day_active(t, T.trace_start, T.trace_end) || T.thr_trace[L->layer] == 0 || st.trace_count[L->sim] == 0) return;
  if (L->rp1) return;  // indexed: k_trace_csr visits the traced agents' edges
  const int64_t words = (st.n + 31) >> 5;
  uint32_t* contact = st.contact_bits + (int64_t)L->layer * words;
  const int64_t e0 = ((int64_t)blockIdx.x - L->tile_begin) * TILE;
  const int64_t e1 = min(e0 + TILE, L->n_edges);
  const int32_t off = (int32_t)sp.agent_off;
  for (int r = 0; r < ROUNDS; ++r) {
    const int64_t eb = e0 + ((int64_t)r * EDGE_THREADS + threadIdx.x) * EDGE_VEC;
    if (eb >= e1) break;
    int32_t a[EDGE_VEC], b[EDGE_VEC];
#pragma unroll
    for (int j = 0; j < EDGE_VEC; ++j) {
      a[j] = eb + j < e1 ? __ldg(L->p1 + eb + j) : off;
      b[j] = eb + j < e1 ? __ldg(L->p2 + eb + j) : off;
    }
#pragma unroll
    for (int j = 0; j < EDGE_VEC; ++j) {
      if (eb + j >= e1) break;
      if (bit_of(st.trace_bits, a[j])) atomicOr(contact + (b[j] >> 5), 1u << (b[j] & 31));
      if (bit_of(st.trace_bits, b[j])) atomicOr(contact + (a[j] >> 5), 1u << (a[j] & 31));
    }
  }
}

// find_contacts through the index of each stored layer: a traced agent marks the
// other endpoint of each of its edges, as p1 and as p2
__device__ __forceinline__ void trace_csr_block(const covgpu_state& st, int t, const covgpu_agent_block& blk) {
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const covgpu_testing& T = sp.testing;
  if (!day_active(t, T.trace_start, T.trace_end) || st.trace_count[blk.sim] == 0) return;
  const int64_t i = blk.begin + threadIdx.x;
  if (i >= blk.end || !((st.trace_bits[i >> 5] >> (i & 31)) & 1u)) return;
  const int64_t words = (st.n + 31) >> 5;
  const int64_t local = i - sp.agent_off;
  for (int l = 0; l < sp.n_layers; ++l) {
    const int seg = sp.seg_of_layer[l];
    if (seg < 0 || T.thr_trace[l] == 0) continue;
    const covgpu_layer& L = st.segments[seg];
    if (L.dynamic || !L.rp1) continue;
    uint32_t* contact = st.contact_bits + (int64_t)l * words;
    for (uint32_t k = L.rp1[local]; k < L.rp1[local + 1]; ++k) {
      const int32_t b = L.p2[k];
      atomicOr(contact + (b >> 5), 1u << (b & 31));
    }
    for (uint32_t k = L.rp2[local]; k < L.rp2[local + 1]; ++k) {
      const int32_t a = L.p1[L.perm2[k]];
      atomicOr(contact + (a >> 5), 1u << (a & 31));
    }
  }
}
__global__ void __launch_bounds__(AGENT_THREADS) k_trace_csr(covgpu_state st, int t) {
  if (held(st, t)) return;
  int64_t b, b_end;
  if (!agent_range(st, b, b_end)) return;
  for (; b < b_end; ++b) trace_csr_block(st, t, st.agent_blocks[b]);
}

// find_contacts over the dynamic layers: one warp per agent block; each traced
// agent draws its two contact lists (the draws the edge pass makes for that agent
// as a source) and marks every partner
constexpr int TRACE_DYN_WARPS = 4;
__global__ void __launch_bounds__(TRACE_DYN_WARPS * 32) k_trace_dyn(covgpu_state st, int t) {
  if (held(st, t)) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * TRACE_DYN_WARPS + warp;
  if (b >= st.n_agent_blocks) return;  // warp-uniform
  const covgpu_agent_block blk = st.agent_blocks[b];
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const covgpu_testing& T = sp.testing;
  if (!day_active(t, T.trace_start, T.trace_end) || st.trace_count[blk.sim] == 0) return;
  const int64_t w0 = blk.begin >> 5;  // sims start at multiples of 32
  const int nw = (int)((blk.end - blk.begin + 31) >> 5);
  const WarpBits wb = warp_bits_scan(lane < nw ? st.trace_bits[w0 + lane] : 0u);
  if (wb.total == 0) return;
  const int64_t words = (st.n + 31) >> 5;
  const uint32_t n_local = (uint32_t)sp.n_agents, thr = bounded_thr(n_local);
  const int32_t off = (int32_t)sp.agent_off;
  for (int l = 0; l < sp.n_layers; ++l) {
    const int seg = sp.seg_of_layer[l];
    if (seg < 0 || T.thr_trace[l] == 0 || !st.segments[seg].dynamic) continue;
    const covgpu_layer& L = st.segments[seg];
    uint32_t* contact = st.contact_bits + (int64_t)l * words;
    for (int base = 0; base < wb.total; base += 32) {
      const int idx = base + lane;
      int bit;
      const int wl = warp_bits_nth(wb, nw, idx, bit);
      if (idx >= wb.total) continue;
      const uint32_t a = (uint32_t)((w0 + wl) * 32 + bit - off);
      int k[2];
      dyn_counts(L.dyn_cdf, L.dyn_k, a, (uint32_t)t, (uint32_t)l, sp.key0, sp.key1, k[0], k[1]);
      for (int d = 0; d < 2; ++d) {
        uint4 pw = make_uint4(0u, 0u, 0u, 0u);
        for (int j = 0; j < k[d]; ++j) {
          if ((j & 3) == 0) pw = dyn_partner_block(a, d, j, (uint32_t)t, (uint32_t)l, sp.key0, sp.key1);
          const int32_t g = off + (int32_t)dyn_partner(word_of(pw, j & 3), n_local, thr, a, d, j, (uint32_t)t,
                                                       (uint32_t)l, sp.key0, sp.key1);
          atomicOr(contact + (g >> 5), 1u << (g & 31));
        }
      }
    }
  }
}

// contact_tracing.notify_contacts (interventions.py:1120-1145) with the
// binomial_filter of identify_contacts, then update_states_post
// (people.py:189-196: check_diagnosed, check_quar, check_enter_iso)
// One agent block of the post pass; the day's diagnoses, quarantines and
// isolations are counted into the thread's accumulators
__device__ __forceinline__ void post_block(const covgpu_state& st, int t, const covgpu_agent_block& blk,
                                           unsigned& acc_diag, unsigned& acc_quar, unsigned& acc_iso) {
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const covgpu_testing& T = sp.testing;
  const int64_t i = blk.begin + threadIdx.x;
  const bool valid = i < blk.end;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t words = (st.n + 31) >> 5;
  const int64_t w = (blk.begin + warp * 32) >> 5;
  const bool warp_in = blk.begin + warp * 32 < blk.end;
  const float tf = (float)t;
  const int R = st.pending_slots;
  unsigned c_diag = 0, c_quar = 0, c_iso = 0;
  // the agent's fields the checks read, loaded together (one round trip): flags,
  // date_pos_test, date_diagnosed, today's pending-quarantine slot, date_end_quarantine
  const float nanf_ = __int_as_float(0x7fc00000);
  uint32_t f = 0u;
  float a_dpt = nanf_, a_dd = nanf_, a_deq = nanf_;
  int32_t a_pq = -1;
  int32_t* pq_today = st.pending_quar + (int64_t)(t % R) * st.n + i;
  if (valid) {
    f = st.flags[i];
    a_dpt = date_row(st, COVGPU_DATE_POS_TEST)[i];
    a_dd = date_row(st, COVGPU_DATE_DIAGNOSED)[i];
    a_pq = *pq_today;
    a_deq = date_row(st, COVGPU_DATE_END_QUARANTINE)[i];
  }
  const uint32_t f_in = f;

  // ---- notify the contacts found by the scan (only on tracing days)
  if (day_active(t, T.trace_start, T.trace_end) && warp_in) {
    for (int l = 0; l < sp.n_layers; ++l) {
      uint32_t* cw = st.contact_bits + (int64_t)l * words + w;
      const uint32_t word = *cw;
      __syncwarp();
      if (!word) continue;
      if (lane == 0) *cw = 0u;  // leave the bitmap clear for the next tracing day
      if (!valid || !((word >> lane) & 1u)) continue;
      const uint32_t local = (uint32_t)(i - sp.agent_off);
      const uint4 u = philox(make_uint4(local, (uint32_t)l, (uint32_t)t, TAG_TRACE), sp.key0, sp.key1);
      if (!bern52_thr(u.x, u.y, T.thr_trace[l]) || (f & B_DEAD)) continue;
      f |= B_KCONT;
      float* dkc = date_row(st, COVGPU_DATE_KNOWN_CONTACT) + i;
      const float cand = __double2float_rn(__dadd_rn((double)t, T.trace_time[l]));
      if (isnan(*dkc) || cand < *dkc) *dkc = cand;  // np.fmin
      const int start = t + T.trace_start_off[l];
      const int32_t end = start + T.trace_period[l];
      if (start == t) {  // today's slot: check_quar below reads it from a_pq
        if (a_pq < 0 || end > a_pq) a_pq = end;
        continue;
      }
      int32_t* pq = st.pending_quar + (int64_t)(start % R) * st.n + i;
      if (*pq < 0 || end > *pq) *pq = end;  // check_quar keeps the latest end of a day's requests
    }
  }

  if (valid) {
    // ---- check_diagnosed, people.py:315-332
    const float dd = a_dd;
    if (!(f & B_DIAG)) {
      if (defined(a_dpt) && tf >= a_dpt) { date_row(st, COVGPU_DATE_POS_TEST)[i] = nanf_; c_diag = 1; }
      if (defined(dd) && tf >= dd) f |= B_DIAG;
    }
    // ---- check_quar, people.py:335-358
    const int32_t end = a_pq;
    float deq = a_deq;
    if (end >= 0) {
      *pq_today = -1;
      if (f & B_QUAR) {
        if ((float)end > deq) deq = (float)end;  // max(current, end_day), first argument kept on ties/NaN
      } else if (!(f & (B_DEAD | B_REC | B_DIAG | B_ISO))) {
        f |= B_QUAR;
        date_row(st, COVGPU_DATE_QUARANTINED)[i] = tf;
        deq = (float)end;
        c_quar = 1;
      }
    }
    if ((f & B_QUAR) && dd == tf) deq = tf;
    if (__float_as_uint(deq) != __float_as_uint(a_deq)) date_row(st, COVGPU_DATE_END_QUARANTINE)[i] = deq;
    if ((f & B_QUAR) && defined(deq) && tf >= deq) f &= ~B_QUAR;
    // ---- check_enter_iso, people.py:361-366
    if (dd == tf) {
      f |= B_ISO;
      date_row(st, COVGPU_DATE_END_ISOLATION)[i] = date_row(st, COVGPU_DATE_RECOVERED)[i];
      c_iso = 1;
    }
    if (f != f_in) st.flags[i] = f;
    // a source's record carries its flags to the edge pass: keep its quarantine / isolation current
    if (((f ^ f_in) & (B_QUAR | B_ISO)) && ((st.roles[i >> 5] >> (i & 31)) & 1u)) st.src_rec[4 * i + 3] = __uint_as_float(f);
    // and a target's record carries its quarantine in the sign bit
    if (((f ^ f_in) & B_QUAR) && ((st.roles[words + (i >> 5)] >> (i & 31)) & 1u))
      for (int v = 0; v < sp.n_variants; ++v) {
        uint32_t* r = reinterpret_cast<uint32_t*>(st.tgt_rec + (int64_t)v * st.n + i);
        *r = (f & B_QUAR) ? (*r | 0x80000000u) : (*r & 0x7FFFFFFFu);
      }
  }
  acc_diag += c_diag;
  acc_quar += c_quar;
  acc_iso += c_iso;
  // the day's trace count is read only by the tracing passes, which have finished
  if (threadIdx.x == 0 && blk.begin == sp.agent_off) st.trace_count[blk.sim] = 0u;
}

__device__ __forceinline__ void post_flush(const covgpu_state& st, int t, int sim, unsigned& acc_diag,
                                           unsigned& acc_quar, unsigned& acc_iso) {
  const covgpu_sim_params& sp = st.sims[sim];
  const unsigned cd = __reduce_add_sync(0xffffffffu, acc_diag), cq = __reduce_add_sync(0xffffffffu, acc_quar),
                 ci = __reduce_add_sync(0xffffffffu, acc_iso);
  int64_t* res = sp.res_int + (int64_t)t * COVGPU_N_RES_INT;
  if ((threadIdx.x & 31) == 0 && t < sp.npts) {
    if (cd) atomicAdd(reinterpret_cast<unsigned long long*>(res + R_DIAGNOSES), (unsigned long long)cd);
    if (cq) atomicAdd(reinterpret_cast<unsigned long long*>(res + R_QUARANTINED), (unsigned long long)cq);
    if (ci) atomicAdd(reinterpret_cast<unsigned long long*>(res + R_ISOLATED), (unsigned long long)ci);
  }
  acc_diag = acc_quar = acc_iso = 0;
}

__global__ void __launch_bounds__(AGENT_THREADS) k_post_pass(covgpu_state st, int t) {
  if (held(st, t)) return;
  int64_t b, b_end;
  if (!agent_range(st, b, b_end)) return;
  int sim = st.agent_blocks[b].sim;
  unsigned acc_diag = 0, acc_quar = 0, acc_iso = 0;
  for (; b < b_end; ++b) {
    const covgpu_agent_block blk = st.agent_blocks[b];
    if (blk.sim != sim) {
      post_flush(st, t, sim, acc_diag, acc_quar, acc_iso);
      sim = blk.sim;
    }
    post_block(st, t, blk, acc_diag, acc_quar, acc_iso);
  }
  post_flush(st, t, sim, acc_diag, acc_quar, acc_iso);
}

// ------------------------------------------------------------ contact-tracing index
__global__ void k_row_ptr(const int32_t* p, int64_t n_edges, int64_t off, int64_t n_local, uint32_t* rp) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a > n_local) return;
  const int64_t key = off + a;  // first edge with p >= key
  int64_t lo = 0, hi = n_edges;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((int64_t)p[mid] < key) lo = mid + 1; else hi = mid;
  }
  rp[a] = (uint32_t)lo;
}
__global__ void k_rev_count(const int32_t* p2, int64_t n_edges, int64_t off, int64_t n_local, int64_t* counts) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_edges) return;
  const int64_t a = (int64_t)p2[e] - off;
  if (a >= 0 && a < n_local) atomicAdd(reinterpret_cast<unsigned long long*>(counts + a), 1ull);
}
__global__ void k_rev_offsets(const int64_t* offsets, int64_t n, uint32_t* rp2) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a <= n) rp2[a] = (uint32_t)offsets[a];
}
__global__ void k_rev_place(const int32_t* p2, int64_t n_edges, int64_t off, int64_t n_local, int64_t* cursor,
                            uint32_t* perm2) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_edges) return;
  const int64_t a = (int64_t)p2[e] - off;
  if (a < 0 || a >= n_local) return;
  const unsigned long long pos = atomicAdd(reinterpret_cast<unsigned long long*>(cursor + a), 1ull);
  perm2[pos] = (uint32_t)e;
}

}  // namespace

namespace covgpu {

int launch_test_trace(const covgpu_state* st, int t, cudaStream_t s) {
  if (!st->has_testing) return COVGPU_OK;
  k_test_prep<<<(unsigned)st->n_sims, 256, 0, s>>>(*st, t);
  if (st->has_testing & 2) {  // some sim has a swab delay
    static const int64_t hist_wave = wave_blocks(k_swab_hist, AGENT_THREADS);
    k_swab_hist<<<wave_grid(st, hist_wave), AGENT_THREADS, 0, s>>>(*st, t);
  }
  static const int64_t test_wave = wave_blocks(k_test_pass, AGENT_THREADS);
  k_test_pass<<<wave_grid(st, test_wave), AGENT_THREADS, 0, s>>>(*st, t);
  if (st->has_testing & 4) k_trace_cap<<<(unsigned)st->n_sims, 256, 0, s>>>(*st, t);  // a tracing capacity
  if (st->n_tiles > 0 && !(st->has_testing & 8)) {  // some stored layer is traced without an index
    const dim3 grid((unsigned)st->n_tiles);
    switch (st->edge_tile) {
      case 1024: k_trace_scan<1><<<grid, EDGE_THREADS, 0, s>>>(*st, t); break;
      case 2048: k_trace_scan<2><<<grid, EDGE_THREADS, 0, s>>>(*st, t); break;
      case 8192: k_trace_scan<8><<<grid, EDGE_THREADS, 0, s>>>(*st, t); break;
      default: k_trace_scan<4><<<grid, EDGE_THREADS, 0, s>>>(*st, t); break;
    }
  }
  static const int64_t csr_wave = wave_blocks(k_trace_csr, AGENT_THREADS);
  k_trace_csr<<<wave_grid(st, csr_wave), AGENT_THREADS, 0, s>>>(*st, t);
  if (st->n_dynamic)
    k_trace_dyn<<<(unsigned)((st->n_agent_blocks + TRACE_DYN_WARPS - 1) / TRACE_DYN_WARPS), TRACE_DYN_WARPS * 32, 0,
                  s>>>(*st, t);
  static const int64_t post_wave = wave_blocks(k_post_pass, AGENT_THREADS);
  k_post_pass<<<wave_grid(st, post_wave), AGENT_THREADS, 0, s>>>(*st, t);
  return launch_status();
}

}  // namespace covgpu

extern "C" {

int covgpu_test_trace(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF) return COVGPU_BADARG;
  return launch_test_trace(st, t, S(stream));
}

int64_t covgpu_trace_index_scratch(int64_t n_local) {
  return 2 * (n_local + 1) + (int64_t)scan_blocks_for(n_local, SCAN_TILE) + 1;
}

int covgpu_trace_index(const int32_t* p1, const int32_t* p2, int64_t n_edges, int64_t agent_off, int64_t n_local,
                       uint32_t* rp1, uint32_t* rp2, uint32_t* perm2, int64_t* scratch, void* stream) {
  if (n_edges < 1 || n_edges > 0xFFFFFFFFLL || n_local < 1 || agent_off < 0 || !p1 || !p2 || !rp1 || !rp2 ||
      !perm2 || !scratch)
    return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  int64_t* counts = scratch;
  int64_t* offsets = scratch + (n_local + 1);
  int64_t* tiles = scratch + 2 * (n_local + 1);
  k_row_ptr<<<grid_for(n_local + 1, 256, 1 << 30), 256, 0, s>>>(p1, n_edges, agent_off, n_local, rp1);
  if (cudaMemsetAsync(counts, 0, sizeof(int64_t) * (size_t)n_local, s) != cudaSuccess) return COVGPU_CUDA_ERROR;
  k_rev_count<<<grid_for(n_edges, 256, 1 << 30), 256, 0, s>>>(p2, n_edges, agent_off, n_local, counts);
  int rc = scan_i64(counts, offsets, n_local, tiles, s);
  if (rc) return rc;
  k_rev_offsets<<<grid_for(n_local + 1, 256, 1 << 30), 256, 0, s>>>(offsets, n_local, rp2);
  k_rev_place<<<grid_for(n_edges, 256, 1 << 30), 256, 0, s>>>(p2, n_edges, agent_off, n_local, offsets, perm2);
  return launch_status();
}

}  // extern "C"
