// covgpu_dropin: the day path's functions one at a time, for callers that use
// the reference's own call sequence instead of the fused day kernels:
//   k_check            People.check_infectious / check_symptomatic / check_severe /
//                      check_critical / check_recovery / check_death / check_exit_iso
//                      (people.py:222-312, 368-374), returning the agents changed;
//   k_check_immunity   check_immunity (immunity.py:303-350);
//   k_update_nab       update_nab (immunity.py:205-213);
//   k_update_peak_nab  update_peak_nab (immunity.py:138-202).
// Each writes the same state words and arrays as the fused agent and infect
// passes, with the same arithmetic (covgpu_imm.cuh, covgpu_ff.cuh).
#include <cuda_runtime.h>
#include <stdint.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_ff.cuh"
#include "covgpu_imm.cuh"
#include "covgpu_launch.cuh"

using namespace covgpu;

namespace {

constexpr int DROPIN_THREADS = 256;

// one People.check_* for agent i (flags f, vstate vs); returns whether it changed
// the agent. filt: the reference's is_exp filter (the exposed flag, which is the
// reference's start-of-day snapshot for each check run in update_states_pre's order)
__device__ __forceinline__ bool check_one(const covgpu_state& st, int nv, bool waning, int which, bool filt,
                                          bool forced, int64_t i, float tf, uint32_t& f, uint32_t& vs, bool& kd) {
  uint32_t ev = vs & 0xFFu, iv = (vs >> 8) & 0xFFu, rv = (vs >> 16) & 0xFFu;
  const bool pass = !filt || (f & B_EXP);
  bool hit = false;
  switch (which) {
    case COVGPU_CHECK_INFECTIOUS: {  // people.py:222-232
      const float d = date_row(st, COVGPU_DATE_INFECTIOUS)[i];
      if (pass && !(f & B_INF) && defined(d) && tf >= d) {
        f |= B_INF;
        iv = ev;
        if (iv < (uint32_t)nv) f |= 1u << (INFV_SHIFT + iv);
        hit = true;
      }
      break;
    }
    case COVGPU_CHECK_SYMPTOMATIC:  // people.py:235-253
    case COVGPU_CHECK_SEVERE:
    case COVGPU_CHECK_CRITICAL: {
      const int row = which == COVGPU_CHECK_SYMPTOMATIC ? COVGPU_DATE_SYMPTOMATIC
                    : (which == COVGPU_CHECK_SEVERE ? COVGPU_DATE_SEVERE : COVGPU_DATE_CRITICAL);
      const uint32_t bit = which == COVGPU_CHECK_SYMPTOMATIC ? B_SYMP : (which == COVGPU_CHECK_SEVERE ? B_SEV : B_CRIT);
      const float d = date_row(st, row)[i];
      if (pass && !(f & bit) && defined(d) && tf >= d) {
        f |= bit;
        hit = true;
      }
      break;
    }
    case COVGPU_CHECK_RECOVERY: {  // people.py:256-291 (forced: an explicit inds argument)
      const float d = date_row(st, COVGPU_DATE_RECOVERED)[i];
      if (forced || (pass && !(f & B_REC) && defined(d) && tf >= d)) {
        f &= ~(B_EXP | B_INF | B_SYMP | B_SEV | B_CRIT | BYVAR_MASK);
        f |= B_REC;
        rv = ev;
        iv = NOV;
        ev = NOV;
        if (waning) { f |= B_SUS; f &= ~B_DIAG; }
        hit = true;
      }
      break;
    }
    case COVGPU_CHECK_DEATH: {  // people.py:294-312
      const float d = date_row(st, COVGPU_DATE_DEAD)[i];
      if (pass && !(f & B_DEAD) && defined(d) && tf >= d) {
        f |= B_DEAD;
        if (f & B_DIAG) { f |= B_KDEAD; kd = true; }
        f &= ~(B_SUS | B_EXP | B_INF | B_SYMP | B_SEV | B_CRIT | B_KCONT | B_QUAR | B_REC);
        iv = ev = rv = NOV;
        hit = true;
      }
      break;
    }
    default: {  // COVGPU_CHECK_EXIT_ISO, people.py:368-374
      const float d = date_row(st, COVGPU_DATE_END_ISOLATION)[i];
      if ((f & B_ISO) && defined(d) && tf >= d) {
        f &= ~B_ISO;
        hit = true;
      }
      break;
    }
  }
  vs = (vs & 0xFF000000u) | (rv << 16) | (iv << 8) | ev;
  return hit;
}

__global__ void __launch_bounds__(DROPIN_THREADS) k_check(covgpu_state st, int t, int which, int sim, int filt,
                                                           const int32_t* inds, int64_t n, int32_t* out, int64_t cap,
                                                           int64_t* counts) {
  const covgpu_sim_params& sp = st.sims[sim];
  const int lane = threadIdx.x & 31;
  const float tf = (float)t;
  // uniform trip count per block (the append ballots need every lane)
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    bool hit = false, kd = false;
    int32_t local = 0;
    if (j < n) {
      local = inds ? inds[j] : (int32_t)j;
      if (local >= 0 && local < sp.n_agents) {
        const int64_t i = sp.agent_off + local;
        uint32_t f = st.flags[i], vs = st.vstate[i];
        hit = check_one(st, sp.n_variants, sp.use_waning != 0, which, filt != 0, inds != nullptr, i, tf, f, vs, kd);
        if (hit) { st.flags[i] = f; st.vstate[i] = vs; }
      } else {
        atomicOr(st.status, COVGPU_BADARG);
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit), mk = __ballot_sync(0xffffffffu, kd);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    unsigned long long pos = 0;
    if (lane == leader) {
      pos = atomicAdd(reinterpret_cast<unsigned long long*>(counts), (unsigned long long)__popc(m));
      if (mk) atomicAdd(reinterpret_cast<unsigned long long*>(counts + 1), (unsigned long long)__popc(mk));
    }
    pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(m & ((1u << lane) - 1u));
    if (hit) {
      if ((int64_t)pos < cap) out[pos] = local;
      else atomicOr(st.status, COVGPU_OVERFLOW);
    }
  }
}

// check_immunity for every agent of one sim and the variants of vmask
__global__ void __launch_bounds__(DROPIN_THREADS) k_check_immunity(covgpu_state st, int t, int sim, uint32_t vmask) {
  const covgpu_sim_params& sp = st.sims[sim];
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < sp.n_agents;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = sp.agent_off + j;
    const uint32_t f = st.flags[i];
    const bool was_inf = (float)t >= date_row(st, COVGPU_DATE_RECOVERED)[i];  // false for NaN
    const uint32_t rv = (st.vstate[i] >> 16) & 0xFFu;
    const float nab = st.nab[i];
    ff ln_nab = ff{0.0f, 0.0f};
    bool have_ln = false;
    for (int v = 0; v < sp.n_variants; ++v) {
      if (!((vmask >> v) & 1u)) continue;
      ff ln_imm;
      const float imm = imm_of(st, sp, i, v, f, was_inf, rv, ln_imm);
      float a = 0.0f, b = 0.0f, c = 0.0f;
      if (nab > 0.0f && imm > 0.0f) {
        if (!have_ln) { ln_nab = ff_log(nab, COVGPU_LN_TAB, COVGPU_LN_INV); have_ln = true; }
        const ff ln_eff = ff_add(ln_nab, ln_imm);
        a = ve_axis(sp, 0, ln_eff, COVGPU_EXP_TAB);
        b = ve_axis(sp, 1, ln_eff, COVGPU_EXP_TAB);
        c = ve_axis(sp, 2, ln_eff, COVGPU_EXP_TAB);
      }
      const int64_t off = (int64_t)v * st.n + i;
      st.sus_imm[off] = a;
      st.symp_imm[off] = b;
      st.sev_imm[off] = c;
    }
  }
}

// update_nab for the listed agents (local indices of one sim)
__global__ void __launch_bounds__(DROPIN_THREADS) k_update_nab(covgpu_state st, int t, int sim, const int32_t* inds,
                                                               int64_t n) {
  const covgpu_sim_params& sp = st.sims[sim];
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t local = inds[j];
    if (local < 0 || local >= sp.n_agents) { atomicOr(st.status, COVGPU_BADARG); continue; }
    const int64_t i = sp.agent_off + local;
    int k = t - st.t_nab_event[i];
    if (k < 0 || k >= sp.nab_kin_len) {
      atomicOr(st.status, COVGPU_BADARG);
      k = k < 0 ? 0 : sp.nab_kin_len - 1;
    }
    st.nab[i] = update_nab_ff(st.nab[i], st.peak_nab[i], sp.nab_kin[2 * k], sp.nab_kin[2 * k + 1]);
  }
}

// update_peak_nab for the listed agents: a boost where NAbs are present, else
// 2^init (init ~ nab_init, a standard normal from Philox (agent, 3, day,
// TAG_INFECT | call_tag), the block infect()'s own draws leave unused), scaled
// by the symptom class's rel_imm_symp and norm_factor when symp_class is given
__global__ void __launch_bounds__(DROPIN_THREADS) k_update_peak_nab(covgpu_state st, int t, int sim,
                                                                    const int32_t* inds, int64_t n,
                                                                    const int8_t* symp_class, covgpu_dur_par init,
                                                                    float boost, double norm, int call_tag) {
  const covgpu_sim_params& sp = st.sims[sim];
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t local = inds[j];
    if (local < 0 || local >= sp.n_agents) { atomicOr(st.status, COVGPU_BADARG); continue; }
    const int64_t i = sp.agent_off + local;
    if (st.nab[i] > 0.0f) {
      st.peak_nab[i] = __fmul_rn(st.peak_nab[i], boost);
    } else {
      const uint4 w = philox(make_uint4((uint32_t)local, 3u, (uint32_t)t, TAG_INFECT | (uint32_t)call_tag), sp.key0,
                             sp.key1);
      ff z0, z1;
      box_muller_ff(w.x, w.y, COVGPU_LN_TAB, COVGPU_LN_INV, COVGPU_SINCOS_TAB, z0, z1);
      double peak = exp2_ff(d2ff(sample_ff(init, z0)));
      if (symp_class) {
        const int c = symp_class[j];
        const double rel = c == 0 ? sp.rel_imm_asymp : (c == 1 ? sp.rel_imm_mild : sp.rel_imm_severe);
        peak = __dmul_rn(__dmul_rn(peak, rel), norm);
      }
      st.peak_nab[i] = (float)peak;
    }
    st.t_nab_event[i] = t;
  }
}

int check_sim(const covgpu_state* st, int32_t sim) {
  const int rc = check_state(st);
  if (rc) return rc;
  return (sim < 0 || sim >= st->n_sims) ? COVGPU_BADARG : COVGPU_OK;
}

}  // namespace

extern "C" {

int covgpu_check(const covgpu_state* st, int32_t t, int32_t which, int32_t sim, int32_t filter_exposed,
                 const int32_t* inds, int64_t n_inds, int64_t n_agents, int32_t* out, int64_t capacity,
                 int64_t* counts, void* stream) {
  int rc = check_sim(st, sim);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF || which < 0 || which > COVGPU_CHECK_EXIT_ISO || !out || !counts || capacity < 0 ||
      (inds && which != COVGPU_CHECK_RECOVERY) || (inds ? n_inds < 0 : n_agents < 0))
    return COVGPU_BADARG;
  cudaStream_t s = S(stream);
  if (cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), s) != cudaSuccess) return COVGPU_CUDA_ERROR;
  const int64_t n = inds ? n_inds : n_agents;
  if (n == 0) return COVGPU_OK;
  k_check<<<grid_for(n, DROPIN_THREADS), DROPIN_THREADS, 0, s>>>(*st, t, which, sim, filter_exposed, inds, n, out,
                                                                  capacity, counts);
  return launch_status();
}

int covgpu_check_immunity(const covgpu_state* st, int32_t t, int32_t sim, uint32_t variant_mask, void* stream) {
  int rc = check_sim(st, sim);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF) return COVGPU_BADARG;
  k_check_immunity<<<grid_for(1 << 22, DROPIN_THREADS), DROPIN_THREADS, 0, S(stream)>>>(*st, t, sim, variant_mask);
  return launch_status();
}

int covgpu_update_nab(const covgpu_state* st, int32_t t, int32_t sim, const int32_t* inds, int64_t n_inds,
                      void* stream) {
  int rc = check_sim(st, sim);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF || n_inds < 0 || (n_inds && !inds)) return COVGPU_BADARG;
  if (n_inds == 0) return COVGPU_OK;
  k_update_nab<<<grid_for(n_inds, DROPIN_THREADS), DROPIN_THREADS, 0, S(stream)>>>(*st, t, sim, inds, n_inds);
  return launch_status();
}

int covgpu_update_peak_nab(const covgpu_state* st, int32_t t, int32_t sim, const int32_t* inds, int64_t n_inds,
                           const int8_t* symp_class, covgpu_dur_par nab_init, float nab_boost, double norm_factor,
                           int32_t call_tag, void* stream) {
  int rc = check_sim(st, sim);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF || n_inds < 0 || (n_inds && !inds) || call_tag < 0 || call_tag > 0xFFFF)
    return COVGPU_BADARG;
  if (n_inds == 0) return COVGPU_OK;
  k_update_peak_nab<<<grid_for(n_inds, DROPIN_THREADS), DROPIN_THREADS, 0, S(stream)>>>(
      *st, t, sim, inds, n_inds, symp_class, nab_init, nab_boost, norm_factor, call_tag);
  return launch_status();
}

}  // extern "C"
