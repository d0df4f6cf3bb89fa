// covgpu: GB300-native (sm_103a) kernels for Covasim 3.1.7's per-day step.
//
// Kernels (all HBM/L2-bound integer and float32 work; no tensor cores):
//   k_agent_step     one dense pass per agent per day (one wave of blocks walking
//       agent-block ranges): update_states_pre (people.py:164-312,368-374) +
//       check_immunity (immunity.py:303-350) + update_nab (immunity.py:205-213) +
//       stocks/flows (sim.py:651-674) + viral load, source/target role bitmaps and
//       the source and target records of the edge passes;
//   k_edge_wave      every stored layer segment and variant of every sim, one wave
//       of blocks over balanced tile ranges (k_edge_pass: one block per tile;
//       k_edge_pass_res: the source bitmap in shared memory): edges streamed with
//       128-bit reads, source->target candidates queued per warp in shared memory,
//       then compute_trans_sus folded in lane-packed, Philox Bernoullis,
//       warp-ballot compaction of events, atomicMin first-infector claim;
//   k_dyn_pass       the redrawn layers (base.py:1849-1876): the day's sources'
//       contact lists drawn from Philox and thinned, the same candidates' path;
//       on quiet days its second half of blocks walks the stored layers from the
//       sources instead of the tile pass (k_src_pass: the walk on its own);
//   k_infect_claims / k_infect_list   People.infect (people.py:435-586) +
//       update_peak_nab (immunity.py:138-202).
// The reference's standalone numba functions are in covgpu_reference.cu, the
// testing and tracing passes in covgpu_testing.cu, the population builders in
// covgpu_pop.cu.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <stddef.h>
#include <math.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_ff.cuh"
#include "covgpu_launch.cuh"
#include "covgpu_imm.cuh"

using namespace covgpu;

namespace {

// Programmatic dependent launch for the day's kernels: a kernel launched with
// launch_pdl may be scheduled while its stream predecessor's last blocks finish
// (inside a captured graph the edge becomes a programmatic one); pdl_wait, the
// first statement of each such kernel, holds it until the predecessor has
// completed and its writes are visible. Launched the ordinary way, pdl_wait
// returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// A block's signal that the next kernel's blocks may be scheduled once every block
// of this grid has given it or exited: their set-up before pdl_wait (tables,
// read-only descriptors) then overlaps this grid's last blocks.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <typename... K, typename... A>
void launch_pdl(void (*kernel)(K...), unsigned grid, unsigned block, size_t smem, cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

// resident blocks per SM that the register budget of the agent pass must allow
// (0: the compiler's choice); the pass's grid is one wave of them. Three blocks
// ran a whole 1M-agent run (one CUDA graph) 0.8 ms faster than four and 2.3 ms
// faster than five (both spilling); bounding the infect pass the same way
// changed nothing.
#ifndef COVGPU_AGENT_MIN_BLOCKS
#define COVGPU_AGENT_MIN_BLOCKS 3
#endif
#if COVGPU_AGENT_MIN_BLOCKS
#define AGENT_BOUNDS __launch_bounds__(AGENT_THREADS, COVGPU_AGENT_MIN_BLOCKS)
#else
#define AGENT_BOUNDS __launch_bounds__(AGENT_THREADS)
#endif
constexpr int EQ_ROUND = 32 * EDGE_VEC;  // most candidates one warp appends per round (one per edge)
#ifndef COVGPU_EQ_CAP
#define COVGPU_EQ_CAP 256
#endif
constexpr int EQ_CAP = COVGPU_EQ_CAP;  // candidate queue entries per warp (drained when a round could overflow);
                                       // 192 and 160, which leave L1 more room, measured slower
static_assert(2 * EDGE_TILE_MAX <= 65536, "queue entries pack (edge within the tile, direction) in 16 bits");
constexpr int CALL_TAG_SEED = 1;       // covgpu_infect_list call_tag of the day-0 seed infections
constexpr int CALL_TAG_IMPORT = 2;     // the daily importations (variant importations: 2 + variant)
constexpr int IMPORT_BLOCKS = 4;       // k_import_day grid (a day imports a handful of agents)


// ============================================================ fused agent pass


// One agent's inputs that (nearly) every agent needs: the state words, rel_sus, the
// recovery date and the NAb fields, loaded one agent block ahead of its processing.
struct AgentIn {
  uint32_t f, vs;
  float rs, dr, nab, peak;
  int tne;
};

__device__ __forceinline__ AgentIn agent_load(const covgpu_state& st, int64_t i, bool valid, bool waning) {
  AgentIn a{0u, 0xFFFFFFFFu, 0.0f, f32nan(), 0.0f, 0.0f, 0};
  if (valid) {
    a.f = st.flags[i];
    a.vs = st.vstate[i];
    a.rs = st.rel_sus[i];
    a.dr = date_row(st, COVGPU_DATE_RECOVERED)[i];
    if (waning) {
      a.nab = st.nab[i];
      a.peak = st.peak_nab[i];
      a.tne = st.t_nab_event[i];
    }
  }
  return a;
}

// The block's counters: [0, N_RES_INT) day-t ints, then the day t-1 stocks, then
// the variant slots [slot][v], and the warps' fixed-point sums.
struct AgentCounters {
  unsigned int cnt[COVGPU_N_RES_INT];  // day t flows + severe/critical now
  unsigned int prev[N_STOCKS];         // day t-1 stocks
  unsigned int var[COVGPU_N_RES_VAR * COVGPU_MAX_VARIANTS];
  long long f[AGENT_THREADS / 32][3];
};

__device__ __forceinline__ void agent_counters_clear(AgentCounters& c) {
  for (int k = threadIdx.x; k < COVGPU_N_RES_INT; k += blockDim.x) c.cnt[k] = 0;
  for (int k = threadIdx.x; k < N_STOCKS; k += blockDim.x) c.prev[k] = 0;
  for (int k = threadIdx.x; k < COVGPU_N_RES_VAR * COVGPU_MAX_VARIANTS; k += blockDim.x) c.var[k] = 0;
}

// Bits of an agent's day word (agent_block_step): the day's flows, the severe and
// critical now, the variant of a new infectious agent (bit 16 + v) and the two
// edge-pass roles, the last two stored as the role bitmaps' words.
constexpr int DW_FLOWS = 9, DW_VAR = 16, DW_SRC = 30, DW_TGT = 31;
// result slots of day-word bits 0-8, six bits each
constexpr uint64_t FLOW_SLOTS =
    (uint64_t)R_INFECTIOUS | (uint64_t)R_SYMPTOMATIC << 6 |
    (uint64_t)R_SEVERE << 12 | (uint64_t)R_CRITICAL << 18 | (uint64_t)R_RECOVERIES << 24 |
    (uint64_t)R_DEATHS << 30 | (uint64_t)R_KNOWN_DEATHS << 36 | (uint64_t)COVGPU_RES_SEVERE_NOW << 42 |
    (uint64_t)COVGPU_RES_CRITICAL_NOW << 48;
static_assert(COVGPU_N_RES_INT <= 64, "six-bit slots");
static_assert(DW_VAR + COVGPU_MAX_VARIANTS <= DW_SRC, "day-word layout");

// One agent block (up to 256 agents of one sim, thread k on agent begin + k):
// closes day t-1 and runs day t's checks for its agents. Counts go to per-lane
// accumulators: the agents' flag words (for the stocks) and day words (for the
// flows) are bit-transposed across the warp, so lane b counts bit b
// (acc_prev: flag bit b, acc_day: day-word bit b) with one popcount, and the
// sums reach the block's counters once per agent_flush. Sums of levels go to the
// thread's fixed-point sums (2^24 for NAbs, 2^32 for efficacies: exact integer
// reductions, independent of order, and no float64 work per agent). full_imm: also store sev_imm (read only by infect(), which
// recomputes it for the agents it infects; stored on the last day of a launch
// sequence, so that the state a caller reads afterwards holds the reference's array).
__device__ __forceinline__ void agent_block_step(const covgpu_state& st, const covgpu_agent_block& blk,
                                                 const AgentIn& in, int t, int do_prev, int do_day, int full_imm,
                                                 int steady,
                                                 const float (*s_ln_tab)[2], const float* s_ln_inv,
                                                 const float (*s_exp_tab)[2],
                                                 long long& nab_fx, long long& sus_fx, long long& symp_fx,
                                                 unsigned& acc_prev, unsigned& acc_day) {
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const int nv = sp.n_variants;
  const int64_t i = blk.begin + threadIdx.x;
  const bool valid = i < blk.end;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tp = t - 1;
  const bool waning = sp.use_waning != 0;
  uint32_t f = in.f, vs = in.vs;
  const float a_rs = in.rs, a_dr = in.dr, a_nab = in.nab, a_peak = in.peak;
  const int a_tne = in.tne;
  const uint32_t f_in = f, vs_in = vs;
  float nab_now = a_nab;  // the NAb level after the closing pass's update_nab

  // A warp of steady agents (susceptible and naive and nothing else: never infected,
  // so without NAbs, and not tested, quarantined, isolated or vaccinated): their day
  // changes none of their fields, records or role bits, and closing the day before
  // counts them as susceptible and naive. Their role words and target records are
  // those an earlier full pass of the launch sequence wrote (steady: not its first
  // day), since every kernel that changes an agent's flags or quarantine keeps them
  // current; so only the stocks are counted.
  if (steady && __all_sync(0xffffffffu, !valid || f == (B_SUS | B_NAIVE))) {
    if (do_prev) acc_prev += (((B_SUS | B_NAIVE) >> lane) & 1u) * (unsigned)__popc(__ballot_sync(0xffffffffu, valid));
    return;
  }

  // ---------------------------------------------------------- close day t-1
  if (do_prev) {
    // sim.py:652-656: stocks at the end of day t-1, one flag bit each, and the
    // exposed / infectious by variant (flag bits EXPV_SHIFT + v, INFV_SHIFT + v)
    acc_prev += __popc(warp_transpose32(valid ? f : 0u));
    if (valid) {
      float nab = 0.0f;
      if (waning) {
        nab = a_nab;
        if (a_peak != 0.0f) {  // sim.py:666-669 -> immunity.py:205-213 at t-1
          int k = tp - a_tne;
          if (k < 0 || k >= sp.nab_kin_len) {
            atomicOr(st.status, COVGPU_BADARG);
            k = k < 0 ? 0 : sp.nab_kin_len - 1;
          }
          nab = update_nab_ff(nab, a_peak, sp.nab_kin[2 * k], sp.nab_kin[2 * k + 1]);
          st.nab[i] = nab;
          nab_now = nab;
        }
      }
      if (!(f & B_DEAD) && nab != 0.0f) nab_fx += __float2ll_rn(__fmul_rn(nab, 16777216.0f));  // sim.py:672
    }
  }

  // ---------------------------------------------------------- day t
  uint32_t src_bit = 0, tgt_bit = 0;
  if (do_day) {
    unsigned c_inf = 0, c_symp = 0, c_sev = 0, c_crit = 0, c_rec = 0, c_dead = 0, c_kdead = 0;
    int inf_v = -1;
    if (valid) {
      const float tf = (float)t;
      uint32_t ev = vs & 0xFFu, iv = (vs >> 8) & 0xFFu, rv = (vs >> 16) & 0xFFu;
      const bool is_exp = f & B_EXP;  // people.py:170 snapshot
      // the exposed agents' dates and rel_trans (the infectious are among them), and
      // the isolated agents' end date, loaded together before the checks use them
      float d_inf = 0.0f, d_sym = 0.0f, d_sev = 0.0f, d_crit = 0.0f, d_dead = 0.0f, d_iso = 0.0f, a_rt = 0.0f;
      if (is_exp) {
        d_inf = date_row(st, COVGPU_DATE_INFECTIOUS)[i];
        d_sym = date_row(st, COVGPU_DATE_SYMPTOMATIC)[i];
        d_sev = date_row(st, COVGPU_DATE_SEVERE)[i];
        d_crit = date_row(st, COVGPU_DATE_CRITICAL)[i];
        d_dead = date_row(st, COVGPU_DATE_DEAD)[i];
        a_rt = st.rel_trans[i];
      }
      if (f & B_ISO) d_iso = date_row(st, COVGPU_DATE_END_ISOLATION)[i];
      if (is_exp) {
        if (!(f & B_INF)) {  // check_infectious, people.py:222-232
          const float d = d_inf;
          if (defined(d) && tf >= d) {
            f |= B_INF;
            iv = ev;
            if (iv < (uint32_t)nv) { f |= 1u << (INFV_SHIFT + iv); inf_v = (int)iv; }
            c_inf = 1;
          }
        }
        if (!(f & B_SYMP)) {  // check_symptomatic, people.py:235-239
          const float d = d_sym;
          if (defined(d) && tf >= d) { f |= B_SYMP; c_symp = 1; }
        }
        if (!(f & B_SEV)) {  // check_severe, people.py:242-246
          const float d = d_sev;
          if (defined(d) && tf >= d) { f |= B_SEV; c_sev = 1; }
        }
        if (!(f & B_CRIT)) {  // check_critical, people.py:249-253
          const float d = d_crit;
          if (defined(d) && tf >= d) { f |= B_CRIT; c_crit = 1; }
        }
        if (!(f & B_REC)) {  // check_recovery, people.py:256-291
          const float d = a_dr;
          if (defined(d) && tf >= d) {
            f &= ~(B_EXP | B_INF | B_SYMP | B_SEV | B_CRIT | BYVAR_MASK);
            f |= B_REC;
            rv = ev;
            iv = NOV;
            ev = NOV;
            if (waning) { f |= B_SUS; f &= ~B_DIAG; }
            c_rec = 1;
          }
        }
      }
      if (f & B_ISO) {  // check_exit_iso, people.py:368-374
        const float d = d_iso;
        if (defined(d) && tf >= d) f &= ~B_ISO;
      }
      if (is_exp && !(f & B_DEAD)) {  // check_death, people.py:294-312
        const float d = d_dead;
        if (defined(d) && tf >= d) {
          f |= B_DEAD;
          if (f & B_DIAG) { f |= B_KDEAD; c_kdead = 1; }
          f &= ~(B_SUS | B_EXP | B_INF | B_SYMP | B_SEV | B_CRIT | B_KCONT | B_QUAR | B_REC);
          iv = ev = rv = NOV;
          c_dead = 1;
        }
      }
      vs = (vs & 0xFF000000u) | (rv << 16) | (iv << 8) | ev;

      // an edge-pass target (susceptible, rel_sus nonzero) gets its susceptibility per
      // variant, rel_sus * (1 - sus_imm[v]) as compute_trans_sus forms it unquarantined
      // (utils.py:87), with the sign bit set when quarantined
      const float rs = (f & B_SUS) ? a_rs : 0.0f;
      const bool is_tgt = rs != 0.0f;
      const uint32_t tq = (f & B_QUAR) ? 0x80000000u : 0u;
      if (waning && a_peak == 0.0f && nab_now == 0.0f) {
        // an agent that never had NAbs: every efficacy is 0, as the state has held
        // them since initialisation (nothing to store; infect() reads symp_imm as 0
        // for it, symp_imm_of), and the target record is rel_sus itself
        if (is_tgt)
          for (int v = 0; v < nv; ++v) st.tgt_rec[(int64_t)v * st.n + i] = __uint_as_float(__float_as_uint(rs) | tq);
      } else if (waning) {  // check_immunity, immunity.py:303-350 (float-float, one rounding)
        const bool was_inf = tf >= a_dr;  // false for NaN
        const float nab = nab_now;
        ff ln_nab = ff{0.0f, 0.0f};
        bool have_ln = false;
        for (int v = 0; v < nv; ++v) {
          ff ln_imm;  // imm = max(natural, vaccine); ln(imm) from the host's tables
          const float imm = imm_of(st, sp, i, v, f, was_inf, rv, ln_imm);
          float a = 0.0f, b = 0.0f, c = 0.0f;
          if (nab > 0.0f && imm > 0.0f) {  // eff = nab * imm > 0; else every efficacy is 0
            if (!have_ln) { ln_nab = ff_log(nab, s_ln_tab, s_ln_inv); have_ln = true; }
            const ff ln_eff = ff_add(ln_nab, ln_imm);
            a = ve_axis(sp, 0, ln_eff, s_exp_tab);
            b = ve_axis(sp, 1, ln_eff, s_exp_tab);
            if (full_imm) c = ve_axis(sp, 2, ln_eff, s_exp_tab);
          }
          const int64_t off = (int64_t)v * st.n + i;
          st.sus_imm[off] = a;
          st.symp_imm[off] = b;
          if (full_imm) st.sev_imm[off] = c;
          if (is_tgt) st.tgt_rec[off] = __uint_as_float(__float_as_uint(__fmul_rn(rs, __fsub_rn(1.0f, a))) | tq);
          if (a != 0.0f || b != 0.0f) {
            sus_fx += __float2ll_rn(__fmul_rn(a, 4294967296.0f));
            symp_fx += __float2ll_rn(__fmul_rn(b, 4294967296.0f));
          }
        }
      }

      // viral load (sim.py:601-608) and edge-pass roles for the infectious / susceptible,
      // with the records the edge pass gathers for its candidates (one 16-byte load
      // per endpoint instead of one per field)
      if (f & B_INF) {
        const float rt = a_rt;
        const float vl = viral_load_one(t, d_inf, a_dr, d_dead, sp.frac_time, sp.load_ratio, sp.high_cap);
        st.viral_load[i] = vl;
        src_bit = (rt != 0.0f && iv < (uint32_t)nv) ? 1u : 0u;
        if (src_bit)
          reinterpret_cast<float4*>(st.src_rec)[i] = make_float4(rt, vl, __uint_as_float(vs), __uint_as_float(f));
      }
      // exclusive by construction (the infectious are never susceptible); the edge
      // pass relies on it to queue at most one direction per edge
      if (is_tgt) {
        tgt_bit = 1u;
        if (!waning)
          for (int v = 0; v < nv; ++v) {
            const int64_t off = (int64_t)v * st.n + i;
            st.tgt_rec[off] = __uint_as_float(__float_as_uint(__fmul_rn(rs, __fsub_rn(1.0f, st.sus_imm[off]))) | tq);
          }
      }
      if (f != f_in) st.flags[i] = f;
      if (vs != vs_in) st.vstate[i] = vs;
    }
    // flows (people.py:172-180), the severe/critical counts of sim.py:579-580, the
    // new infectious by variant and the roles, one bit each of the day word;
    // transposed, lanes 30 and 31 hold the role bitmaps' words of this warp's 32
    // agents (the 32-aligned word (i - lane) / 32)
    const uint32_t dw = valid ? (c_inf | c_symp << 1 | c_sev << 2 | c_crit << 3 | c_rec << 4 | c_dead << 5 |
                                 c_kdead << 6 | ((f & B_SEV) ? 1u << 7 : 0u) | ((f & B_CRIT) ? 1u << 8 : 0u) |
                                 (inf_v >= 0 ? 1u << (DW_VAR + inf_v) : 0u) | src_bit << DW_SRC |
                                 tgt_bit << DW_TGT)
                              : 0u;
    const uint32_t col = warp_transpose32(dw);
    if (lane < DW_SRC) {
      acc_day += __popc(col);
    } else if (blk.begin + warp * 32 < blk.end) {
      const int64_t w = (blk.begin + warp * 32) >> 5;
      st.roles[(lane == DW_SRC ? 0 : roles_words(st)) + w] = col;  // source / target bitmap
    }
  }
}

// Adds the block's counters and fixed-point sums of sim `sim` to its results:
// integer atomics, bit-reproducible. With `clear` the counters restart at zero
// for the next sim's agent blocks.
__device__ __noinline__ void agent_flush(const covgpu_state& st, int sim, int t, int do_prev, int do_day,
                                         AgentCounters& sc, long long& nab_fx, long long& sus_fx, long long& symp_fx,
                                         unsigned& acc_prev, unsigned& acc_day, bool clear) {
  const covgpu_sim_params& sp = st.sims[sim];
  const int nv = sp.n_variants;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tp = t - 1;
  unsigned int* s_cnt = sc.cnt;
  unsigned int* s_prev = sc.prev;
  unsigned int* s_var = sc.var;
  nab_fx = warp_sum_fx(nab_fx);
  sus_fx = warp_sum_fx(sus_fx);
  symp_fx = warp_sum_fx(symp_fx);
  if (lane == 0) { sc.f[warp][0] = nab_fx; sc.f[warp][1] = sus_fx; sc.f[warp][2] = symp_fx; }
  if (acc_prev) {  // lane b: flag bit b
    if (lane >= INFV_SHIFT) atomicAdd(&s_var[RV_N_INFECTIOUS * COVGPU_MAX_VARIANTS + lane - INFV_SHIFT], acc_prev);
    else if (lane >= EXPV_SHIFT) atomicAdd(&s_var[RV_N_EXPOSED * COVGPU_MAX_VARIANTS + lane - EXPV_SHIFT], acc_prev);
    else
      for (int k = 0; k < N_STOCKS; ++k)
        if (STOCK_BITS[k] == 1u << lane) atomicAdd(&s_prev[k], acc_prev);
  }
  if (acc_day) {  // lane b: day-word bit b
    if (lane >= DW_VAR) atomicAdd(&s_var[RV_INFECTIOUS * COVGPU_MAX_VARIANTS + lane - DW_VAR], acc_day);
    else if (lane < DW_FLOWS) atomicAdd(&s_cnt[(FLOW_SLOTS >> (6 * lane)) & 63u], acc_day);
  }
  acc_prev = acc_day = 0;
  __syncthreads();
  const int npts = sp.npts;
  int64_t* res_t = sp.res_int + (int64_t)t * COVGPU_N_RES_INT;
  int64_t* res_tp = sp.res_int + (int64_t)tp * COVGPU_N_RES_INT;
  if (do_day && t < npts) {
    for (int k = threadIdx.x; k < COVGPU_N_RES_INT; k += blockDim.x)
      if (s_cnt[k]) atomicAdd(reinterpret_cast<unsigned long long*>(&res_t[k]), (unsigned long long)s_cnt[k]);
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
      const unsigned c = s_var[RV_INFECTIOUS * COVGPU_MAX_VARIANTS + v];
      if (c) atomicAdd(reinterpret_cast<unsigned long long*>(&sp.res_var[((int64_t)t * COVGPU_N_RES_VAR + RV_INFECTIOUS) * nv + v]),
                       (unsigned long long)c);
    }
  }
  if (do_prev && tp >= 0) {
    for (int k = threadIdx.x; k < N_STOCKS; k += blockDim.x)
      if (s_prev[k]) atomicAdd(reinterpret_cast<unsigned long long*>(&res_tp[R_N_FIRST + k]), (unsigned long long)s_prev[k]);
    for (int k = threadIdx.x; k < 2 * nv; k += blockDim.x) {
      const int slot = k < nv ? RV_N_EXPOSED : RV_N_INFECTIOUS, v = k < nv ? k : k - nv;
      const unsigned c = s_var[slot * COVGPU_MAX_VARIANTS + v];
      if (c) atomicAdd(reinterpret_cast<unsigned long long*>(&sp.res_var[((int64_t)tp * COVGPU_N_RES_VAR + slot) * nv + v]),
                       (unsigned long long)c);
    }
  }
  // block totals of the fixed-point sums, added with integer atomics (bit-reproducible)
  if (threadIdx.x == 0) {
    long long a = 0, b = 0, c = 0;
    for (int w = 0; w < AGENT_THREADS / 32; ++w) { a += sc.f[w][0]; b += sc.f[w][1]; c += sc.f[w][2]; }
    if (do_prev && tp >= 0 && a != 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(&sp.res_fx[(int64_t)tp * COVGPU_N_RES_F + 0]),
                (unsigned long long)a);
    if (do_day && t < npts && (b != 0 || c != 0)) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&sp.res_fx[(int64_t)t * COVGPU_N_RES_F + 1]),
                (unsigned long long)b);
      atomicAdd(reinterpret_cast<unsigned long long*>(&sp.res_fx[(int64_t)t * COVGPU_N_RES_F + 2]),
                (unsigned long long)c);
    }
  }
  nab_fx = sus_fx = symp_fx = 0;
  if (clear) {
    __syncthreads();
    agent_counters_clear(sc);
    __syncthreads();
  }
}

// The fused agent pass. It runs as (at most) one wave of resident blocks, each
// walking a contiguous range of agent blocks: the next agent block's loads are in
// flight while the current one is processed, no barrier separates agent blocks of
// one sim, and the counters go to the results once per sim a block touched
// instead of once per 256 agents.
__global__ void AGENT_BOUNDS k_agent_step(covgpu_state st, int t, int do_prev, int do_day, int full_imm, int steady) {
  const int64_t nb = st.n_agent_blocks;
  const int64_t per = (nb + gridDim.x - 1) / gridDim.x;
  int64_t b = (int64_t)blockIdx.x * per;
  const int64_t b_end = min(nb, b + per);
  if (b >= b_end) return;  // block-uniform

  // set-up that reads nothing an earlier kernel writes: before pdl_wait
  __shared__ AgentCounters sc;
  __shared__ float s_ln_tab[COVGPU_LN_N][2];
  __shared__ float s_ln_inv[COVGPU_LN_N];
  __shared__ float s_exp_tab[COVGPU_EXP_N][2];
  for (int k = threadIdx.x; k < 2 * COVGPU_LN_N; k += blockDim.x) (&s_ln_tab[0][0])[k] = (&COVGPU_LN_TAB[0][0])[k];
  for (int k = threadIdx.x; k < COVGPU_LN_N; k += blockDim.x) s_ln_inv[k] = COVGPU_LN_INV[k];
  for (int k = threadIdx.x; k < 2 * COVGPU_EXP_N; k += blockDim.x) (&s_exp_tab[0][0])[k] = (&COVGPU_EXP_TAB[0][0])[k];
  agent_counters_clear(sc);
  covgpu_agent_block blk = st.agent_blocks[b];
  int sim = blk.sim;
  __syncthreads();

  pdl_wait();
  if (st.hold) {  // a held day t - 1 has nothing to close; a held day t closes day t - 1 only
    const int h = *st.hold;
    if (h <= t - 1) return;
    if (h <= t) do_day = 0;
    if (!do_prev && !do_day) return;
  }
  if (do_day && blockIdx.x == 0 && threadIdx.x == 0) *st.event_count = 0ull;
  AgentIn cur = agent_load(st, blk.begin + threadIdx.x, blk.begin + threadIdx.x < blk.end,
                           st.sims[sim].use_waning != 0);

  long long nab_fx = 0, sus_fx = 0, symp_fx = 0;
  unsigned acc_prev = 0, acc_day = 0;
  for (;;) {
    const bool more = b + 1 < b_end;
    covgpu_agent_block nblk = blk;
    AgentIn nxt = cur;
    if (more) {
      nblk = st.agent_blocks[b + 1];
      const int64_t ni = nblk.begin + threadIdx.x;
      nxt = agent_load(st, ni, ni < nblk.end, st.sims[nblk.sim].use_waning != 0);
    }
    agent_block_step(st, blk, cur, t, do_prev, do_day, full_imm, steady, s_ln_tab, s_ln_inv, s_exp_tab, nab_fx, sus_fx,
                     symp_fx, acc_prev, acc_day);
    if (!more) break;
    ++b;
    if (nblk.sim != sim) {
      agent_flush(st, sim, t, do_prev, do_day, sc, nab_fx, sus_fx, symp_fx, acc_prev, acc_day, true);
      sim = nblk.sim;
    }
    blk = nblk;
    cur = nxt;
  }
  pdl_trigger();
  agent_flush(st, sim, t, do_prev, do_day, sc, nab_fx, sus_fx, symp_fx, acc_prev, acc_day, false);
}

// ============================================================ fused edge pass
//
// One block per tile of ROUNDS * 1024 edges of one layer segment. Phase A streams
// the tile (128-bit loads of p1/p2, or the dynamic layer's endpoints from
// Philox), reads both endpoints' role words and appends every candidate
// direction source -> target to its warp's queue in shared memory. Phase B
// drains the queue one candidate per lane, so the gathers of
// compute_trans_sus run lane-packed instead of serialising the whole warp on
// the few lanes that hold a source.

// source bit (infectious with a variant and rel_trans != 0) and target bit
// (susceptible with rel_sus != 0) of agent a: two separate bitmaps, so that the
// source bitmap (n/8 bytes), tested for both endpoints of every edge, stays in L1
__device__ __forceinline__ uint32_t src_bit(const uint32_t* __restrict__ roles, int32_t a) {
  return (ld_keep_u32(roles + (a >> 5)) >> (a & 31)) & 1u;
}
__device__ __forceinline__ uint32_t tgt_bit(const covgpu_state& st, int32_t a) {
  return (__ldg(st.roles + roles_words(st) + (a >> 5)) >> (a & 31)) & 1u;
}

// per-tile constants, hoisted out of the segment and sim records
struct SegCtx {
  const covgpu_layer* L;
  const float* edge_beta;    // per-edge layer weights, or null for beta_const
  const float* beta_t;       // beta_tab row of day t ([n_variants])
  float beta_const, beta_layer, quar_factor, iso_factor, asymp_factor;
  float rse_max;             // dynamic layers: the thinning bound (covgpu_layer.dyn_rse_max)
  uint32_t key0, key1;
  int nv, layer, seg, sim;
  int64_t n_edges;
};

// per-thread likelihood sums of one tile (one sim, one layer), float-float
struct LikAcc {
  ff ll{0.0f, 0.0f}, g{0.0f, 0.0f};
};

__device__ __forceinline__ ff ff_mul_f(ff x, float f) {
  const ff p = two_prod(x.hi, f);
  return fast_two_sum(p.hi, __fmaf_rn(x.lo, f, p.lo));
}
// ln of a positive float-float: ln(hi) + lo / hi (|lo / hi| <= 2^-24, so the
// dropped term is below 2^-49)
__device__ __forceinline__ ff ff_log_ff(ff x) {
  const ff l = ff_log(x.hi, COVGPU_LN_TAB, COVGPU_LN_INV);
  return fast_two_sum(l.hi, __fadd_rn(l.lo, __fdiv_rn(x.lo, x.hi)));
}
__device__ __forceinline__ double ff_to_d(ff x) { return __dadd_rn((double)x.hi, (double)x.lo); }

// The likelihood terms of one candidate direction s -> g (see covgpu_lik):
// the outcome `hit` is the edge pass's own draw on the float32 p32; the
// terms use p recomputed from the unrounded factors and F in float-float
// (~2^-44 relative; GB300's float64 rate is a small fraction of its float32
// rate), capped at 1 (a draw u < p with p >= 1 is certain, and its
// probability does not change with the parameters).
__device__ __forceinline__ void lik_terms(const covgpu_state& st, const SegCtx& c, int t, uint32_t v, int32_t g,
                                          uint32_t fs, uint32_t fg, float rt, float vl, float rs, float lb, float si,
                                          float p32, bool hit, LikAcc& acc) {
  const covgpu_lik& K = st.lik;
  ff r{rt, 0.0f};
  if (fs & B_QUAR) r = ff_mul_f(r, c.quar_factor);
  if (!(fs & B_SYMP)) r = ff_mul_f(r, c.asymp_factor);
  if (fs & B_ISO) r = ff_mul_f(r, c.iso_factor);
  r = ff_mul_f(r, vl);
  ff q{rs, 0.0f};
  if (fg & B_QUAR) q = ff_mul_f(q, c.quar_factor);
  q = ff_mul(q, two_sum(1.0f, -si));
  const float* Fp = K.factor + 2 * ((((int64_t)c.sim * K.npts_max + t) * K.n_layers_max + c.layer) * K.nv_max + v);
  ff p = ff_mul(ff_mul(ff_mul_f(ff{Fp[0], Fp[1]}, lb), r), q);
  if (p.hi > 1.0f || (p.hi == 1.0f && p.lo >= 0.0f)) {
    if (hit) {  // certain transmission: log p = 0, no sensitivity; the target is surely infected
      atomicAdd(K.logq + g, -INFINITY);
      return;
    }
    p = ff{p32, 0.0f};  // not infected, so p32 < 1: p crossed 1 only by rounding
  }
  ff om = two_sum(1.0f, -p.hi);  // 1 - p, exact in float-float
  om = fast_two_sum(om.hi, __fsub_rn(om.lo, p.lo));
  const ff l1m = ff_log_ff(om);
  const ff odds = ff_div(p, om);
  if (hit) {
    acc.ll = ff_add(acc.ll, ff_log_ff(p));
    acc.g = ff_add(acc.g, ff{1.0f, 0.0f});
  } else {
    acc.ll = ff_add(acc.ll, l1m);
    acc.g = ff_add(acc.g, ff{-odds.hi, -odds.lo});
  }
  atomicAdd(K.logq + g, ff_to_d(l1m));
  if (K.g_exp) atomicAdd(K.w + (int64_t)c.layer * st.n + g, ff_to_d(odds));
}

// compute_trans_sus folded into compute_infections for one direction s -> g
// (utils.py:88-89 then 117-123); returns true on a transmission. Every gather
// is issued before the first use so that they overlap. LIK: also the
// likelihood terms of the direction, from the same gathered values. INJ: a
// stored layer's edge, which takes the injected uniforms of test mode. THIN: a
// dynamic layer's list entry, which transmits only if it was a potential
// transmission (ph, covgpu_device.cuh "Thinning") and then with probability
// p * 2^m against the edge's uniform.
template <bool LIK, bool INJ = true, bool THIN = false>
__device__ __forceinline__ bool edge_try(const covgpu_state& st, const SegCtx& c, int t, int64_t e, int dir,
                                         int32_t s, int32_t g, uint32_t& v_out, LikAcc& acc, bool ph = true) {
  const float4 sr = __ldg(reinterpret_cast<const float4*>(st.src_rec) + s);
  const uint32_t fs = __float_as_uint(sr.w);
  const float lb = c.edge_beta ? __ldg(c.edge_beta + e) : c.beta_const;
  const float rt = sr.x, vl = sr.y;
  const uint32_t v = (__float_as_uint(sr.z) >> 8) & 0xFFu;
  const uint32_t vc = v < (uint32_t)c.nv ? v : 0u;
  const int64_t gv = (int64_t)vc * st.n + g;
  const float beta = __ldg(c.beta_t + vc);
  // the target: its record (rel_sus * (1 - sus_imm), sign bit = quarantined); the
  // quarantined, and the likelihood's terms, take the fields themselves
  const uint32_t tr = __float_as_uint(__ldg(st.tgt_rec + gv));
  const bool tquar = tr >> 31;
  uint32_t fg = tquar ? B_QUAR : 0u;
  float rs = 0.0f, si = 0.0f;
  if (LIK || tquar) {
    fg = __ldg(st.flags + g);
    rs = __ldg(st.rel_sus + g);
    si = __ldg(st.sus_imm + gv);
  }
  if (v >= (uint32_t)c.nv) return false;
  float rte = rt;
  if (fs & B_QUAR) rte = __fmul_rn(rte, c.quar_factor);
  if (!(fs & B_SYMP)) rte = __fmul_rn(rte, c.asymp_factor);
  if (fs & B_ISO) rte = __fmul_rn(rte, c.iso_factor);
  rte = __fmul_rn(rte, c.beta_layer);
  rte = __fmul_rn(rte, vl);
  float rse = __uint_as_float(tr & 0x7FFFFFFFu);
  if (tquar) rse = __fmul_rn(__fmul_rn(rs, c.quar_factor), __fsub_rn(1.0f, si));
  const float p = __fmul_rn(__fmul_rn(__fmul_rn(beta, lb), rte), rse);
  if (p == 0.0f) return false;
  v_out = v;
  bool hit;
  if (INJ && st.edge_uniforms) {  // injected draws (test mode)
    hit = st.edge_uniforms[c.seg][((int64_t)v * 2 + dir) * c.n_edges + e] < (double)p;
  } else if (THIN) {
    hit = false;
    if (ph) {
      const int m = thin_shift(__fmul_rn(__fmul_rn(__fmul_rn(beta, lb), rte), c.rse_max));
      const float ps = __fmul_rn(p, __int_as_float((127 + m) << 23));  // p * 2^m, exact
      const uint4 w = philox(make_uint4((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)t,
                                        TAG_EDGE | (v << 8) | (uint32_t)c.layer), c.key0, c.key1);
      hit = dir ? bern52(w.z, w.w, ps) : bern52(w.x, w.y, ps);
    }
  } else {
    // one Philox block per (edge, day, variant, layer): words x,y draw direction 0, z,w direction 1
    const uint4 w = philox(make_uint4((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)t,
                                      TAG_EDGE | (v << 8) | (uint32_t)c.layer), c.key0, c.key1);
    hit = dir ? bern52(w.z, w.w, p) : bern52(w.x, w.y, p);  // u < p in float64, decided in integers
  }
  if (LIK) lik_terms(st, c, t, v, g, fs, fg, rt, vl, rs, lb, si, p, hit, acc);
  return hit;
}

__device__ __forceinline__ uint64_t event_key(int t, uint32_t v, int layer, int dir, int64_t e) {
  return ((uint64_t)(0xFFFFu - (uint32_t)t) << 48) | ((uint64_t)v << 45) | ((uint64_t)layer << 41) |
         ((uint64_t)dir << 40) | (uint64_t)e;
}

// warp-aggregated append of (key, target, source); all lanes of the warp call it
__device__ __forceinline__ void emit(const covgpu_state& st, bool has, uint64_t key, int32_t tgt, int32_t src) {
  const unsigned m = __ballot_sync(0xffffffffu, has);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  const int leader = __ffs(m) - 1;
  if (lane == leader) base = atomicAdd(st.event_count, (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (has) {
    atomicMin(reinterpret_cast<unsigned long long*>(st.claim + tgt), (unsigned long long)key);
    const unsigned long long pos = base + __popc(m & ((1u << lane) - 1u));
    if ((int64_t)pos < st.event_capacity) {
      covgpu_event ev;
      ev.key = key; ev.target = tgt; ev.source = src;
      st.events[pos] = ev;
    } else {
      atomicOr(st.status, COVGPU_OVERFLOW);
    }
  }
}

struct EdgeQueue {               // candidate directions of one warp
  int32_t s[EQ_CAP];             // source agent
  int32_t g[EQ_CAP];             // target agent
  uint16_t m[EQ_CAP];            // (edge within the tile) << 1 | direction
};

// warp-aggregated append of one candidate per lane with `has`
__device__ __forceinline__ void queue_push(EdgeQueue& q, int& qn, bool has, int32_t s, int32_t g, uint32_t m) {
  const unsigned mask = __ballot_sync(0xffffffffu, has);
  if (has) {
    const int pos = qn + __popc(mask & ((1u << (threadIdx.x & 31)) - 1u));
    q.s[pos] = s; q.g[pos] = g; q.m[pos] = (uint16_t)m;
  }
  qn += __popc(mask);
}

// phase B: one candidate per lane, then the warp-aggregated event append
// (LIK: with the likelihood terms)
template <bool LIK>
__device__ __forceinline__ void queue_drain(const covgpu_state& st, const SegCtx& c, int t, int64_t e0,
                                            EdgeQueue& q, int qn, LikAcc& acc) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < qn; base += 32) {
    const int i = base + lane;
    bool hit = false;
    uint32_t v = 0;
    int32_t s = 0, g = 0;
    uint32_t m = 0;
    if (i < qn) {
      s = q.s[i]; g = q.g[i]; m = q.m[i];
      hit = edge_try<LIK>(st, c, t, e0 + (m >> 1), (int)(m & 1u), s, g, v, acc);
    }
    emit(st, hit, hit ? event_key(t, v, c.layer, (int)(m & 1u), e0 + (m >> 1)) : 0ull, g, s);
  }
  __syncwarp();
}

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// The segment owning a tile: the last segment with tile_begin <= tile.
__device__ __forceinline__ int segment_of_tile(const covgpu_layer* segs, int n_segments, int64_t tile) {
  int lo = 0, hi = n_segments - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The fields of a sim's parameter block that the edge pass reads
struct SimLite {
  const float* beta_tab;
  const float* beta_layer_tab;
  int64_t n_agents, agent_off;
  float asymp_factor;
  uint32_t key0, key1;
  int32_t nv, n_layers;
};
__device__ __forceinline__ void load_sim_lite(SimLite& o, const covgpu_sim_params& sp) {
  o.beta_tab = sp.beta_tab;
  o.beta_layer_tab = sp.beta_layer_tab;
  o.n_agents = sp.n_agents;
  o.agent_off = sp.agent_off;
  o.asymp_factor = sp.asymp_factor;
  o.key0 = sp.key0;
  o.key1 = sp.key1;
  o.nv = sp.n_variants;
  o.n_layers = sp.n_layers;
}

// The segment context of a stored segment's tiles (edge_tile, edge_span).
__device__ __forceinline__ void seg_ctx(const covgpu_state& st, int t, int seg, const covgpu_layer* L,
                                        const SimLite* sp, SegCtx& c) {
  c.L = st.segments + seg;
  c.seg = seg;
  c.layer = L->layer;
  c.n_edges = L->n_edges;
  c.edge_beta = L->beta;
  c.beta_const = L->beta_const;
  c.quar_factor = L->quar_factor;
  c.iso_factor = L->iso_factor;
  c.asymp_factor = sp->asymp_factor;
  c.nv = sp->nv;
  c.key0 = sp->key0;
  c.key1 = sp->key1;
  c.beta_t = sp->beta_tab + (int64_t)t * c.nv;
  c.beta_layer = sp->beta_layer_tab[(int64_t)t * sp->n_layers + c.layer];
  c.sim = L->sim;
}

// One round of phase A for this thread's edges eb .. eb + 3 (pa: their p1, pb: their
// p2; those at or past e_hi are masked off): the sources first (every edge: shared
// memory, or the L1-resident bitmap), then the other endpoint's target bit only
// where one endpoint is a source (roles are exclusive, so an edge has at most one
// candidate direction), and the warp-aggregated queue appends, with offsets from e0.
template <bool RES>
__device__ __forceinline__ void edge_round(const covgpu_state& st, const uint32_t* s_src, const int4& pa,
                                           const int4& pb, int64_t eb, int64_t e_hi, int64_t e0, EdgeQueue& q,
                                           int& qn) {
  int32_t a[EDGE_VEC], b[EDGE_VEC];
  a[0] = pa.x; a[1] = pa.y; a[2] = pa.z; a[3] = pa.w;
  b[0] = pb.x; b[1] = pb.y; b[2] = pb.z; b[3] = pb.w;
  uint32_t sa[EDGE_VEC], sb[EDGE_VEC];
#pragma unroll
  for (int j = 0; j < EDGE_VEC; ++j) {
    if (RES) {
      sa[j] = (s_src[a[j] >> 5] >> (a[j] & 31)) & 1u;
      sb[j] = (s_src[b[j] >> 5] >> (b[j] & 31)) & 1u;
    } else {
      sa[j] = src_bit(st.roles, a[j]);
      sb[j] = src_bit(st.roles, b[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < EDGE_VEC; ++j) {
    const bool in = eb + j < e_hi;
    const uint32_t m = (uint32_t)(eb + j - e0) << 1;
    const bool d1 = sb[j] != 0u;  // direction p2 -> p1
    bool cand = false;
    if (in && (sa[j] | sb[j])) cand = tgt_bit(st, d1 ? a[j] : b[j]) != 0u;
    queue_push(q, qn, cand, d1 ? b[j] : a[j], d1 ? a[j] : b[j], m | (d1 ? 1u : 0u));
  }
}

// One tile (TILE edges) of one stored segment, NT threads: phase A streams the
// edges and queues the candidate directions of each warp, phase B drains the queues.
// The segment record L and its sim's constants sp are shared-memory copies.
// RES: the sim's source bitmap is resident in shared memory (s_src, one sim).
template <bool LIK, int NT, int64_t TILE, bool RES>
__device__ __forceinline__ void edge_tile(const covgpu_state& st, int t, int seg, int64_t tile, const covgpu_layer* L,
                                          const SimLite* sp, const uint32_t* s_src, EdgeQueue& q, LikAcc& acc) {
  constexpr int ROUNDS = (int)(TILE / ((int64_t)NT * EDGE_VEC));
  static_assert(ROUNDS >= 1 && TILE % ((int64_t)NT * EDGE_VEC) == 0, "whole rounds per tile");
  SegCtx c;
  seg_ctx(st, t, seg, L, sp, c);
  const int32_t* p1 = L->p1;
  const int32_t* p2 = L->p2;
  const int64_t e0 = (tile - L->tile_begin) * TILE;
  const int64_t e1 = min(e0 + TILE, c.n_edges);
  const int32_t off = (int32_t)sp->agent_off;
  int qn = 0;  // warp-uniform queue length
  // each round's edge lists are loaded one round ahead, so that their latency
  // overlaps the previous round's lookups and queue drain
  auto fetch = [&](int r, int4& xa, int4& xb) {
    const int64_t eb = e0 + ((int64_t)r * NT + threadIdx.x) * EDGE_VEC;
    if (eb + EDGE_VEC <= e1) {
      xa = ld_stream_v4(p1 + eb);
      xb = ld_stream_v4(p2 + eb);
    } else {
      xa.x = eb < e1 ? p1[eb] : off;         xb.x = eb < e1 ? p2[eb] : off;
      xa.y = eb + 1 < e1 ? p1[eb + 1] : off; xb.y = eb + 1 < e1 ? p2[eb + 1] : off;
      xa.z = eb + 2 < e1 ? p1[eb + 2] : off; xb.z = eb + 2 < e1 ? p2[eb + 2] : off;
      xa.w = eb + 3 < e1 ? p1[eb + 3] : off; xb.w = eb + 3 < e1 ? p2[eb + 3] : off;
    }
  };
  static_assert(EDGE_VEC == 4, "one int4 of each list per thread and round");
  int4 na, nb;
  fetch(0, na, nb);
  for (int r = 0; r < ROUNDS; ++r) {
    const int64_t eb = e0 + ((int64_t)r * NT + threadIdx.x) * EDGE_VEC;
    const int4 pa = na, pb = nb;
    if (r + 1 < ROUNDS) fetch(r + 1, na, nb);
    edge_round<RES>(st, s_src, pa, pb, eb, e1, e0, q, qn);
    if (qn > EQ_CAP - EQ_ROUND) {
      queue_drain<LIK>(st, c, t, e0, q, qn, acc);
      qn = 0;
    }
  }
  if (qn > 0) queue_drain<LIK>(st, c, t, e0, q, qn, acc);
}

// Tiles [k_lo, k_hi) of one stored segment (L, its sim's constants sp) as one
// stream of rounds: each round's edge lists are loaded one round ahead, across
// the tiles' boundaries, and the warp's queue entries count edges from a base
// that moves on (the queue drained first) when a round would reach past the
// 2^15 edges their offsets hold.
template <bool LIK, int64_t TILE>
__device__ __forceinline__ void edge_span(const covgpu_state& st, int t, int seg, int64_t k_lo, int64_t k_hi,
                                          const covgpu_layer* L, const SimLite* sp, EdgeQueue& q, LikAcc& acc) {
  constexpr int64_t ROUND = (int64_t)EDGE_THREADS * EDGE_VEC;
  constexpr int64_t SPAN = 32768;
  static_assert(TILE % ROUND == 0 && SPAN % ROUND == 0, "whole rounds");
  SegCtx c;
  seg_ctx(st, t, seg, L, sp, c);
  const int32_t* p1 = L->p1;
  const int32_t* p2 = L->p2;
  const int64_t e_lo = k_lo * TILE;
  const int64_t e_hi = min(k_hi * TILE, c.n_edges);
  const int32_t off = (int32_t)sp->agent_off;
  auto fetch = [&](int64_t rb, int4& xa, int4& xb) {
    const int64_t eb = rb + (int64_t)threadIdx.x * EDGE_VEC;
    if (eb + EDGE_VEC <= e_hi) {
      xa = ld_stream_v4(p1 + eb);
      xb = ld_stream_v4(p2 + eb);
    } else {
      xa.x = eb < e_hi ? p1[eb] : off;         xb.x = eb < e_hi ? p2[eb] : off;
      xa.y = eb + 1 < e_hi ? p1[eb + 1] : off; xb.y = eb + 1 < e_hi ? p2[eb + 1] : off;
      xa.z = eb + 2 < e_hi ? p1[eb + 2] : off; xb.z = eb + 2 < e_hi ? p2[eb + 2] : off;
      xa.w = eb + 3 < e_hi ? p1[eb + 3] : off; xb.w = eb + 3 < e_hi ? p2[eb + 3] : off;
    }
  };
  int qn = 0;
  int64_t e0 = e_lo;
  int4 na, nb;
  fetch(e_lo, na, nb);
  for (int64_t rb = e_lo; rb < e_hi; rb += ROUND) {
    if (rb + ROUND - e0 > SPAN) {
      if (qn > 0) {
        queue_drain<LIK>(st, c, t, e0, q, qn, acc);
        qn = 0;
      }
      e0 = rb;
    }
    const int4 pa = na, pb = nb;
    if (rb + ROUND < e_hi) fetch(rb + ROUND, na, nb);
    edge_round<false>(st, nullptr, pa, pb, rb + (int64_t)threadIdx.x * EDGE_VEC, e_hi, e0, q, qn);
    if (qn > EQ_CAP - EQ_ROUND) {
      queue_drain<LIK>(st, c, t, e0, q, qn, acc);
      qn = 0;
    }
  }
  if (qn > 0) queue_drain<LIK>(st, c, t, e0, q, qn, acc);
}

// the likelihood sums of one warp for one (sim, layer), then reset
__device__ __forceinline__ void lik_flush_warp(const covgpu_state& st, int t, int sim, int layer, LikAcc& acc) {
  const double a = warp_sum_d(ff_to_d(acc.ll)), b = warp_sum_d(ff_to_d(acc.g));
  if ((threadIdx.x & 31) == 0) {
    const covgpu_lik& K = st.lik;
    const int64_t day = (int64_t)sim * K.npts_max + t;
    if (a != 0.0) atomicAdd(K.ll + day, a);
    if (K.g_ll && b != 0.0) atomicAdd(K.g_ll + day * K.n_layers_max + layer, b);
  }
  acc = LikAcc();
}

// Stored layers on quiet days. A stored layer segment with an agent index (rp1,
// rp2, perm2: each agent's edges as p1 and as p2) is walked from the day's
// sources (k_src_pass) instead of streamed edge by edge (the tile passes) while
// its sim's infectious agents times st.src_walk are fewer than its agents (0:
// never, -1: always): the number infectious at the end of day t-1 plus day t's
// new infectious, less its recoveries and deaths, from the results the agent
// pass of day t has written. The walk visits each source's edges (about 2 E x
// prevalence entries, each a few dependent loads) where the tile pass tests both
// endpoints of all E edges. Both queue the same candidates and draw, key and
// claim them alike, so the choice moves only the cost.
__device__ __forceinline__ bool seg_walked(const covgpu_state& st, const covgpu_layer& L, int t) {
  if (L.dynamic || !L.rp1 || st.src_walk == 0) return false;
  if (st.src_walk < 0) return true;
  const covgpu_sim_params& sp = st.sims[L.sim];
  if (t < 0 || t >= sp.npts) return false;
  const int64_t* r = sp.res_int + (int64_t)t * COVGPU_N_RES_INT;
  int64_t inf = r[R_INFECTIOUS] - r[R_RECOVERIES] - r[R_DEATHS];
  if (t > 0) inf += (r - COVGPU_N_RES_INT)[R_N_FIRST + 2];  // n_infectious, end of day t-1
  return inf * (int64_t)st.src_walk < sp.n_agents;
}

// One block per tile (none for a segment walked from its sources today).
template <bool LIK, int ROUNDS>
__global__ void __launch_bounds__(EDGE_THREADS) k_edge_pass(covgpu_state st, int t) {
  pdl_wait();
  if (held(st, t)) return;
  constexpr int64_t TILE = (int64_t)ROUNDS * EDGE_ROUND;
  __shared__ int s_seg;
  __shared__ covgpu_layer s_L;
  __shared__ SimLite s_sp;
  __shared__ EdgeQueue s_q[EDGE_THREADS / 32];
  if (threadIdx.x == 0) {
    const int seg = segment_of_tile(st.segments, st.n_segments, (int64_t)blockIdx.x);
    s_seg = seg;
    s_L = st.segments[seg];
    load_sim_lite(s_sp, st.sims[s_L.sim]);
  }
  __syncthreads();
  if (seg_walked(st, s_L, t)) return;  // block-uniform
  LikAcc acc;
  edge_tile<LIK, EDGE_THREADS, TILE, false>(st, t, s_seg, (int64_t)blockIdx.x, &s_L, &s_sp, nullptr,
                                            s_q[threadIdx.x >> 5], acc);
  pdl_trigger();
  if (LIK) {  // the tile's sums: one sim, one layer
    __shared__ double s_acc[EDGE_THREADS / 32][2];
    const double a = warp_sum_d(ff_to_d(acc.ll)), b = warp_sum_d(ff_to_d(acc.g));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_acc[warp][0] = a; s_acc[warp][1] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double x = 0.0, y = 0.0;
      for (int k = 0; k < EDGE_THREADS / 32; ++k) { x += s_acc[k][0]; y += s_acc[k][1]; }
      const covgpu_lik& K = st.lik;
      const int64_t day = (int64_t)s_L.sim * K.npts_max + t;
      if (x != 0.0) atomicAdd(K.ll + day, x);
      if (K.g_ll && y != 0.0) atomicAdd(K.g_ll + day * K.n_layers_max + s_L.layer, y);
    }
  }
}

// The stored layers as one wave of resident blocks (covgpu_state.edge_wave): of the
// T tiles, block b walks [b T / G, (b + 1) T / G), a contiguous share that differs
// from the others' by at most one tile, segment by segment, its edge lists loaded a
// round ahead across the tiles' boundaries. Against one block per tile it leaves
// no partial last wave and no per-tile start (segment lookup, first round's
// latency); the tile size only sets how finely the shares are balanced.
template <bool LIK, int ROUNDS>
__global__ void __launch_bounds__(EDGE_THREADS) k_edge_wave(covgpu_state st, int t) {
  constexpr int64_t TILE = (int64_t)ROUNDS * EDGE_ROUND;
  const int64_t lo = st.n_tiles * (int64_t)blockIdx.x / gridDim.x;
  const int64_t hi = st.n_tiles * ((int64_t)blockIdx.x + 1) / gridDim.x;
  if (lo >= hi) return;  // block-uniform
  __shared__ covgpu_layer s_L;
  __shared__ SimLite s_sp;
  __shared__ EdgeQueue s_q[EDGE_THREADS / 32];
  __shared__ double s_acc[EDGE_THREADS / 32][2];
  int seg = segment_of_tile(st.segments, st.n_segments, lo);  // the segment table is read-only
  pdl_wait();
  if (held(st, t)) return;
  int64_t tile = lo;
  for (;;) {
    if (threadIdx.x == 0) {
      s_L = st.segments[seg];
      load_sim_lite(s_sp, st.sims[s_L.sim]);
    }
    __syncthreads();
    const int64_t seg_end = seg + 1 < st.n_segments ? st.segments[seg + 1].tile_begin : st.n_tiles;
    const int64_t stop = min(hi, seg_end);  // >= tile: seg is the last segment starting at or before tile
    if (tile < stop && !seg_walked(st, s_L, t)) {  // block-uniform
      LikAcc acc;
      edge_span<LIK, TILE>(st, t, seg, tile - s_L.tile_begin, stop - s_L.tile_begin, &s_L, &s_sp,
                           s_q[threadIdx.x >> 5], acc);
      if (LIK) {  // this segment's sums: one sim, one layer
        const double a = warp_sum_d(ff_to_d(acc.ll)), b = warp_sum_d(ff_to_d(acc.g));
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) { s_acc[warp][0] = a; s_acc[warp][1] = b; }
        __syncthreads();
        if (threadIdx.x == 0) {
          double x = 0.0, y = 0.0;
          for (int k = 0; k < EDGE_THREADS / 32; ++k) { x += s_acc[k][0]; y += s_acc[k][1]; }
          const covgpu_lik& K = st.lik;
          const int64_t day = (int64_t)s_L.sim * K.npts_max + t;
          if (x != 0.0) atomicAdd(K.ll + day, x);
          if (K.g_ll && y != 0.0) atomicAdd(K.g_ll + day * K.n_layers_max + s_L.layer, y);
        }
      }
    }
    if (stop > tile) tile = stop;
    if (tile >= hi || seg + 1 >= st.n_segments) break;
    ++seg;
    __syncthreads();  // every thread has read s_L (and s_acc) before they are replaced
  }
  pdl_trigger();
}

// Resident-bitmap variant for a single sim: one block of RES_THREADS per SM
// loads the sim's source bitmap into shared memory once, then walks the tiles
// with a stride of the grid (stored and redrawn layers interleave, which
// balances the blocks); the per-warp queues follow the bitmap in shared memory.
constexpr int RES_THREADS = 1024;
constexpr int RES_MAX_SEGS = COVGPU_MAX_LAYERS;  // one sim: at most one segment per layer
template <bool LIK, int64_t TILE>
__global__ void __launch_bounds__(RES_THREADS, 1) k_edge_pass_res(covgpu_state st, int t) {
  pdl_wait();
  if (held(st, t)) return;
  extern __shared__ uint4 s_dyn[];
  __shared__ covgpu_layer s_segs[RES_MAX_SEGS];
  __shared__ SimLite s_sp;
  uint32_t* s_src = reinterpret_cast<uint32_t*>(s_dyn);
  const int64_t words = (st.n + 31) >> 5;
  const int n_segs = st.n_segments;
  __shared__ uint32_t s_walk;  // bit k: segment k is walked from its sources today
  if (threadIdx.x < n_segs) s_segs[threadIdx.x] = st.segments[threadIdx.x];
  if (threadIdx.x == 0) s_walk = 0u;
  __syncthreads();
  if (threadIdx.x < n_segs && seg_walked(st, s_segs[threadIdx.x], t)) atomicOr(&s_walk, 1u << threadIdx.x);
  __syncthreads();
  uint32_t streamed = 0u;  // the stored segments left to this pass
  for (int k = 0; k < n_segs; ++k)
    if (!s_segs[k].dynamic && !((s_walk >> k) & 1u)) streamed |= 1u << k;
  if (!streamed) return;  // block-uniform
  // bitmap words four at a time (the bitmap has room for whole uint4s)
  const uint4* g4 = reinterpret_cast<const uint4*>(st.roles);
  for (int64_t k = threadIdx.x; k < (words >> 2); k += RES_THREADS) s_dyn[k] = __ldg(g4 + k);
  for (int64_t k = (words & ~3ll) + threadIdx.x; k < words; k += RES_THREADS) s_src[k] = __ldg(st.roles + k);
  if (threadIdx.x == 0) load_sim_lite(s_sp, st.sims[0]);
  EdgeQueue* s_q = reinterpret_cast<EdgeQueue*>(s_dyn + ((words + 3) >> 2));
  EdgeQueue& q = s_q[threadIdx.x >> 5];
  __syncthreads();
  LikAcc acc;
  for (int64_t tile = blockIdx.x; tile < st.n_tiles; tile += gridDim.x) {
    const int seg = segment_of_tile(s_segs, n_segs, tile);
    if (!((streamed >> seg) & 1u)) continue;
    edge_tile<LIK, RES_THREADS, TILE, true>(st, t, seg, tile, s_segs + seg, &s_sp, s_src, q, acc);
    if (LIK) lik_flush_warp(st, t, s_segs[seg].sim, s_segs[seg].layer, acc);
  }
  pdl_trigger();
}

// ============================================================ redrawn layers
//
// Transmission over the dynamic layers (base.py:1849-1876 redrawn daily, then
// utils.py:93-128): one warp per agent block of one sim, or two (source_split), on its
// source-bitmap words. The words' sources are handed to the lanes 32 at a time; for each
// dynamic layer of the sim every lane draws its source's two list lengths
// (covgpu_device.cuh, "redrawn layers, per agent"), and the lists' four-entry
// blocks of all 32 sources are then spread over the lanes (a prefix count and a
// search for each block's source), so that the Philox blocks of a warp with few
// sources still run on full lanes. Entries are thinned (covgpu_device.cuh
// "Thinning"): only the potential transmissions, about pmax of them, have their
// partner drawn, and those whose partner is a target are queued; the queue
// drains through edge_try as the stored layers' does. The work follows the
// day's sources, not the layer's edges: a quiet day costs a read of the source
// bitmap.
constexpr int DYN_WARPS = 8;  // warps per thread block
// Warps per agent block of the per-source passes (SPLIT, a template parameter: each
// warp takes 8 / SPLIT of the agent block's eight source-bitmap words). One warp
// per agent block ran a 1M-agent run 2.7% faster than two (16.8 against 17.26 ms):
// half the warps to launch and scan on the quiet days, when the pass is all
// scanning; a state of fewer agent blocks than SPLIT_ONE_MIN keeps two, for the
// parallelism of its busy days.
constexpr int AB_WORDS = AGENT_THREADS / 32;  // source-bitmap words of an agent block
constexpr int64_t SPLIT_ONE_MIN = 2048;
inline int source_split(const covgpu_state* st) { return st->n_agent_blocks >= SPLIT_ONE_MIN ? 1 : 2; }

// the segment constants of dynamic layer segment seg for day t
__device__ __forceinline__ void dyn_ctx(const covgpu_state& st, const covgpu_sim_params& sp, int seg, int t, SegCtx& c) {
  const covgpu_layer* L = st.segments + seg;
  c.L = L;
  c.seg = seg;
  c.layer = L->layer;
  c.n_edges = L->n_edges;
  c.edge_beta = nullptr;
  c.beta_const = L->beta_const;
  c.quar_factor = L->quar_factor;
  c.iso_factor = L->iso_factor;
  c.asymp_factor = sp.asymp_factor;
  c.rse_max = L->dyn_rse_max;
  c.nv = sp.n_variants;
  c.key0 = sp.key0;
  c.key1 = sp.key1;
  c.beta_t = sp.beta_tab + (int64_t)t * c.nv;
  c.beta_layer = sp.beta_layer_tab[(int64_t)t * sp.n_layers + c.layer];
  c.sim = L->sim;
}

// the thinning shift of source s (covgpu_device.cuh "Thinning"): pmax = beta *
// lb * rel_trans'(s) * rse_max, formed as edge_try forms p; -1 when the source
// cannot transmit in this layer
__device__ __forceinline__ int dyn_shift(const covgpu_state& st, const SegCtx& c, int32_t s) {
  const float4 sr = __ldg(reinterpret_cast<const float4*>(st.src_rec) + s);
  const uint32_t fs = __float_as_uint(sr.w);
  const uint32_t v = (__float_as_uint(sr.z) >> 8) & 0xFFu;
  if (v >= (uint32_t)c.nv) return -1;
  float rte = sr.x;
  if (fs & B_QUAR) rte = __fmul_rn(rte, c.quar_factor);
  if (!(fs & B_SYMP)) rte = __fmul_rn(rte, c.asymp_factor);
  if (fs & B_ISO) rte = __fmul_rn(rte, c.iso_factor);
  rte = __fmul_rn(rte, c.beta_layer);
  rte = __fmul_rn(rte, sr.y);
  const float q = __fmul_rn(__fmul_rn(__ldg(c.beta_t + v), c.beta_const), rte);
  return q == 0.0f ? -1 : thin_shift(__fmul_rn(q, c.rse_max));
}

// phase B of the redrawn layers: one candidate per lane (entry j of list d of
// source s, potential transmission ph; m = j << 2 | ph << 1 | d), then the
// warp-aggregated event append
template <bool LIK>
__device__ __forceinline__ void dyn_drain(const covgpu_state& st, const SegCtx& c, int t, int64_t agent_off,
                                          EdgeQueue& q, int qn, LikAcc& acc) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < qn; base += 32) {
    const int i = base + lane;
    bool hit = false;
    uint32_t v = 0, m = 0;
    int32_t s = 0, g = 0;
    uint64_t e = 0;
    if (i < qn) {
      s = q.s[i]; g = q.g[i]; m = q.m[i];
      e = dyn_edge_id((uint32_t)(s - agent_off), m >> 2, (uint32_t)t, (uint32_t)c.layer);
      hit = edge_try<LIK, false, true>(st, c, t, (int64_t)e, (int)(m & 1u), s, g, v, acc, (m >> 1) & 1u);
    }
    emit(st, hit, hit ? event_key(t, v, c.layer, (int)(m & 1u), (int64_t)e) : 0ull, g, s);
  }
  __syncwarp();
}

// The redrawn layers of the day's sources for one block's worth (vblock) of
// agent blocks: SPLIT warps per agent block, each on AB_WORDS / SPLIT source-bitmap words.
template <bool LIK, int SPLIT>
__device__ __forceinline__ void dyn_body(const covgpu_state& st, int t, int64_t vblock, EdgeQueue* s_q) {
  constexpr int DYN_WORDS = AB_WORDS / SPLIT;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t gw = vblock * DYN_WARPS + warp;
  const int64_t b = gw / SPLIT;  // SPLIT warps per agent block
  if (b >= st.n_agent_blocks) return;  // warp-uniform
  const covgpu_agent_block blk = st.agent_blocks[b];
  const int w_lo = (int)(gw % SPLIT) * DYN_WORDS;
  const int nwb = (int)((blk.end - blk.begin + 31) >> 5);
  if (w_lo >= nwb) return;
  const int nw = min(DYN_WORDS, nwb - w_lo);
  const int64_t w0 = (blk.begin >> 5) + w_lo;  // sims start at multiples of 32
  const WarpBits wb = warp_bits_scan(lane < nw ? __ldg(st.roles + w0 + lane) : 0u);
  if (wb.total == 0) return;
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const uint32_t n_local = (uint32_t)sp.n_agents, thr = bounded_thr(n_local);
  const int32_t off = (int32_t)sp.agent_off;
  const uint32_t day = (uint32_t)t;
  EdgeQueue& q = s_q[warp];
  LikAcc acc;
  for (int l = 0; l < sp.n_layers; ++l) {
    const int seg = sp.seg_of_layer[l];
    if (seg < 0 || !st.segments[seg].dynamic) continue;
    SegCtx c;
    dyn_ctx(st, sp, seg, t, c);
    int qn = 0;
    for (int base = 0; base < wb.total; base += 32) {
      const int idx = base + lane;
      int bit;
      const int wl = warp_bits_nth(wb, nw, idx, bit);
      const int32_t s = (int32_t)((w0 + wl) * 32 + bit);
      int k0 = 0, k1 = 0, m = -1;
      if (idx < wb.total) {
        m = dyn_shift(st, c, s);
        if (m >= 0 || LIK) dyn_counts(c.L->dyn_cdf, c.L->dyn_k, (uint32_t)(s - off), day, (uint32_t)l, c.key0, c.key1, k0, k1);
      }
      // the lanes' four-entry blocks of both lists (one Philox block of potential
      // transmissions each), flattened across the warp: item j belongs to the
      // first lane whose inclusive prefix count exceeds j
      const uint32_t nb0 = (uint32_t)(k0 + 3) >> 2, nb = nb0 + ((uint32_t)(k1 + 3) >> 2);
      uint32_t pre = nb;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += y;
      }
      const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
      for (uint32_t j0 = 0; j0 < total; j0 += 32) {
        const uint32_t j = j0 + (uint32_t)lane;
        int owner = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (__shfl_sync(0xffffffffu, pre, owner + step - 1) <= j) owner += step;
        const int32_t os = __shfl_sync(0xffffffffu, s, owner);
        const int om = __shfl_sync(0xffffffffu, m, owner);
        const int ok0 = __shfl_sync(0xffffffffu, k0, owner), ok1 = __shfl_sync(0xffffffffu, k1, owner);
        const uint32_t onb0 = __shfl_sync(0xffffffffu, nb0, owner);
        const uint32_t obeg = __shfl_sync(0xffffffffu, pre - nb, owner);
        uint32_t pm = 0u, tb = 0u;
        int d = 0, je = 0;
        int32_t g[4] = {0, 0, 0, 0};
        if (j < total) {
          const uint32_t r = j - obeg;
          d = r >= onb0 ? 1 : 0;
          je = 4 * (int)(d ? r - onb0 : r);
          const int kd = d ? ok1 : ok0;
          const uint32_t oa = (uint32_t)(os - off);
          if (om >= 0) {  // potential transmissions among entries je .. je + 3
            const uint4 hw = dyn_hit_block(oa, d, je, day, (uint32_t)l, c.key0, c.key1);
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4)
              if (je + r4 < kd && thin_potential(word_of(hw, r4), om)) pm |= 1u << r4;
          }
          // partners: of the potential entries (all entries for the likelihood)
          const uint32_t want = LIK ? (0xFu >> max(0, 4 - (kd - je))) : pm;
          if (want) {
            const uint4 pw = dyn_partner_block(oa, d, je, day, (uint32_t)l, c.key0, c.key1);
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4)
              if ((want >> r4) & 1u) {
                g[r4] = off + (int32_t)dyn_partner(word_of(pw, r4), n_local, thr, oa, d, je + r4, day, (uint32_t)l,
                                                   c.key0, c.key1);
                tb |= tgt_bit(st, g[r4]) << r4;
              }
          }
        }
        if (!__any_sync(0xffffffffu, tb != 0u)) continue;
#pragma unroll
        for (int r4 = 0; r4 < 4; ++r4)
          queue_push(q, qn, (tb >> r4) & 1u, os, g[r4],
                     ((uint32_t)(je + r4) << 2) | (((pm >> r4) & 1u) << 1) | (uint32_t)d);
        if (qn > EQ_CAP - 4 * 32) {
          dyn_drain<LIK>(st, c, t, sp.agent_off, q, qn, acc);
          qn = 0;
        }
      }
    }
    if (qn > 0) dyn_drain<LIK>(st, c, t, sp.agent_off, q, qn, acc);
    if (LIK) lik_flush_warp(st, t, blk.sim, l, acc);
  }
}

// The walk of the stored layers from the day's sources (seg_walked): the warps and
// source-bitmap words of the redrawn layers' pass. For each indexed stored
// layer the warp's sources' edges (as p1: [rp1[a], rp1[a + 1]); as p2: the edges
// perm2[rp2[a] .. rp2[a + 1])) are flattened across the lanes 32 at a time, each
// lane finding its source by a search over the lanes' prefix counts; an edge whose
// other endpoint is a target is queued with its index and direction (1: the
// source is p2, as in the tile pass) and drained through edge_try.
constexpr int SRC_WARPS = 8;
struct SrcQueue {
  int32_t s[EQ_CAP];   // source agent
  int32_t g[EQ_CAP];   // target agent | direction << 31
  uint32_t e[EQ_CAP];  // edge index in the layer
};

__device__ __forceinline__ void src_push(SrcQueue& q, int& qn, bool has, int32_t s, int32_t gd, uint32_t e) {
  const unsigned mask = __ballot_sync(0xffffffffu, has);
  if (has) {
    const int pos = qn + __popc(mask & ((1u << (threadIdx.x & 31)) - 1u));
    q.s[pos] = s; q.g[pos] = gd; q.e[pos] = e;
  }
  qn += __popc(mask);
}

template <bool LIK>
__device__ __forceinline__ void src_drain(const covgpu_state& st, const SegCtx& c, int t, SrcQueue& q, int qn,
                                          LikAcc& acc) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < qn; base += 32) {
    const int i = base + lane;
    bool hit = false;
    uint32_t v = 0;
    int32_t s = 0, g = 0;
    int d = 0;
    int64_t e = 0;
    if (i < qn) {
      s = q.s[i];
      const uint32_t gd = (uint32_t)q.g[i];
      g = (int32_t)(gd & 0x7FFFFFFFu);
      d = (int)(gd >> 31);
      e = (int64_t)q.e[i];
      hit = edge_try<LIK>(st, c, t, e, d, s, g, v, acc);
    }
    emit(st, hit, hit ? event_key(t, v, c.layer, d, e) : 0ull, g, s);
  }
  __syncwarp();
}

template <bool LIK, int SPLIT>
__device__ __forceinline__ void src_body(const covgpu_state& st, int t, int64_t vblock, SrcQueue* s_q) {
  constexpr int DYN_WORDS = AB_WORDS / SPLIT;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t gw = vblock * SRC_WARPS + warp;
  const int64_t b = gw / SPLIT;  // SPLIT warps per agent block
  if (b >= st.n_agent_blocks) return;  // warp-uniform
  const covgpu_agent_block blk = st.agent_blocks[b];
  const covgpu_sim_params& sp = st.sims[blk.sim];
  int first = -1;  // the sim's first walked layer
  for (int l = 0; l < sp.n_layers && first < 0; ++l) {
    const int seg = sp.seg_of_layer[l];
    if (seg >= 0 && seg_walked(st, st.segments[seg], t)) first = l;
  }
  if (first < 0) return;
  const int w_lo = (int)(gw % SPLIT) * DYN_WORDS;
  const int nwb = (int)((blk.end - blk.begin + 31) >> 5);
  if (w_lo >= nwb) return;
  const int nw = min(DYN_WORDS, nwb - w_lo);
  const int64_t w0 = (blk.begin >> 5) + w_lo;  // sims start at multiples of 32
  const WarpBits wb = warp_bits_scan(lane < nw ? __ldg(st.roles + w0 + lane) : 0u);
  if (wb.total == 0) return;
  const int32_t off = (int32_t)sp.agent_off;
  SrcQueue& q = s_q[warp];
  LikAcc acc;
  for (int l = first; l < sp.n_layers; ++l) {
    const int seg = sp.seg_of_layer[l];
    if (seg < 0) continue;
    const covgpu_layer& L = st.segments[seg];
    if (!seg_walked(st, L, t)) continue;
    SegCtx c;
    dyn_ctx(st, sp, seg, t, c);
    c.edge_beta = L.beta;
    const int32_t* p1 = L.p1;
    const int32_t* p2 = L.p2;
    int qn = 0;
    for (int base = 0; base < wb.total; base += 32) {
      const int idx = base + lane;
      int bit;
      const int wl = warp_bits_nth(wb, nw, idx, bit);
      const int32_t s = (int32_t)((w0 + wl) * 32 + bit);
      uint32_t k1 = 0, n1 = 0, k2 = 0, n = 0;
      if (idx < wb.total) {
        const uint32_t a = (uint32_t)(s - off);
        k1 = __ldg(L.rp1 + a);
        n1 = __ldg(L.rp1 + a + 1) - k1;
        k2 = __ldg(L.rp2 + a);
        n = n1 + (__ldg(L.rp2 + a + 1) - k2);
      }
      uint32_t pre = n;  // inclusive prefix of the lanes' entry counts
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += y;
      }
      const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
      for (uint32_t j0 = 0; j0 < total; j0 += 32) {
        const uint32_t j = j0 + (uint32_t)lane;
        int owner = 0;  // the first lane whose inclusive prefix exceeds j
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (__shfl_sync(0xffffffffu, pre, owner + step - 1) <= j) owner += step;
        owner = min(owner, 31);
        const int32_t os = __shfl_sync(0xffffffffu, s, owner);
        const uint32_t ok1 = __shfl_sync(0xffffffffu, k1, owner), on1 = __shfl_sync(0xffffffffu, n1, owner);
        const uint32_t ok2 = __shfl_sync(0xffffffffu, k2, owner);
        const uint32_t obeg = __shfl_sync(0xffffffffu, pre - n, owner);
        bool has = false;
        int32_t g = 0;
        uint32_t e = 0, d = 0;
        if (j < total) {
          const uint32_t r = j - obeg;
          if (r < on1) {
            e = ok1 + r;
            g = __ldg(p2 + e);
          } else {
            e = __ldg(L.perm2 + ok2 + (r - on1));
            g = __ldg(p1 + e);
            d = 1u;
          }
          has = tgt_bit(st, g) != 0u;
        }
        src_push(q, qn, has, os, (int32_t)((uint32_t)g | (d << 31)), e);
        if (qn > EQ_CAP - 32) {
          src_drain<LIK>(st, c, t, q, qn, acc);
          qn = 0;
        }
      }
    }
    if (qn > 0) src_drain<LIK>(st, c, t, q, qn, acc);
    if (LIK) lik_flush_warp(st, t, blk.sim, l, acc);
  }
}

static_assert(SRC_WARPS == DYN_WARPS, "the per-source passes share their launch shape");

// The redrawn layers' pass (dyn_body), and with WALK also the walk of the stored
// layers from the day's sources (src_body) in blocks [dyn_blocks, 2 dyn_blocks)
// of the same launch: both start from the day's source bitmap, so on the days the
// stored layers are walked the walk runs beside the redrawn layers' draws instead
// of after the stored layers' (then empty) tile pass. Four resident blocks per SM
// (64 registers): the redrawn layers' pass over a 100-day 1M-agent run took
// 2.70 ms of kernel time against 2.89 ms with three (80 registers).
// resident blocks per SM the per-source passes' registers must allow (three, 80
// registers without spills, ran the 1M run 0.05 ms slower than four)
#ifndef COVGPU_DYN_MIN_BLOCKS
#define COVGPU_DYN_MIN_BLOCKS 4
#endif
template <bool LIK, bool WALK, int SPLIT>
__global__ void __launch_bounds__(DYN_WARPS * 32, COVGPU_DYN_MIN_BLOCKS) k_dyn_pass(covgpu_state st, int t,
                                                                                   int dyn_blocks) {
  if (held(st, t)) return;
  __shared__ union {
    EdgeQueue e[DYN_WARPS];
    SrcQueue s[SRC_WARPS];
  } s_q;
  if (!WALK || (int)blockIdx.x < dyn_blocks) dyn_body<LIK, SPLIT>(st, t, blockIdx.x, s_q.e);
  else src_body<LIK, SPLIT>(st, t, (int64_t)blockIdx.x - dyn_blocks, s_q.s);
}

// The walk alone (a state without redrawn layers, or the stored layers' pass on
// its own).
template <bool LIK, int SPLIT>
__global__ void __launch_bounds__(SRC_WARPS * 32) k_src_pass(covgpu_state st, int t) {
  if (held(st, t)) return;
  __shared__ SrcQueue s_q[SRC_WARPS];
  src_body<LIK, SPLIT>(st, t, blockIdx.x, s_q);
}

unsigned source_pass_blocks(const covgpu_state* st) {
  return (unsigned)((source_split(st) * st->n_agent_blocks + DYN_WARPS - 1) / DYN_WARPS);
}

int launch_src_pass(const covgpu_state* st, int t, cudaStream_t s) {
  if (st->n_tiles == 0 || st->src_walk == 0) return COVGPU_OK;
  const unsigned grid = source_pass_blocks(st);
  const bool one = source_split(st) == 1;
  void (*k)(covgpu_state, int) = st->lik.factor ? (one ? k_src_pass<true, 1> : k_src_pass<true, 2>)
                                                : (one ? k_src_pass<false, 1> : k_src_pass<false, 2>);
  k<<<grid, SRC_WARPS * 32, 0, s>>>(*st, t);
  return launch_status();
}

// the redrawn layers' pass; with_walk: also the walk of the stored layers (when
// src_walk is on), in the same launch
int launch_dyn_pass(const covgpu_state* st, int t, cudaStream_t s, bool with_walk) {
  if (st->n_dynamic == 0) return COVGPU_OK;
  const unsigned g = source_pass_blocks(st);
  const bool walk = with_walk && st->n_tiles > 0 && st->src_walk != 0;
  const unsigned grid = walk ? 2 * g : g;
  void (*k)(covgpu_state, int, int);
  if (source_split(st) == 1)
    k = st->lik.factor ? (walk ? k_dyn_pass<true, true, 1> : k_dyn_pass<true, false, 1>)
                       : (walk ? k_dyn_pass<false, true, 1> : k_dyn_pass<false, false, 1>);
  else
    k = st->lik.factor ? (walk ? k_dyn_pass<true, true, 2> : k_dyn_pass<true, false, 2>)
                       : (walk ? k_dyn_pass<false, true, 2> : k_dyn_pass<false, false, 2>);
  k<<<grid, DYN_WARPS * 32, 0, s>>>(*st, t, (int)g);
  return launch_status();
}

// covgpu_layer_lists: one thread per agent; counts (offsets NULL) or partners
__global__ void k_layer_lists(covgpu_state st, int seg, int t, int64_t begin, int64_t n, int32_t* counts,
                              const int64_t* offsets, int32_t* partners) {
  const covgpu_layer& L = st.segments[seg];
  const covgpu_sim_params& sp = st.sims[L.sim];
  const uint32_t n_local = (uint32_t)sp.n_agents, thr = bounded_thr(n_local);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t a = (uint32_t)(begin + i);
    int k[2];
    dyn_counts(L.dyn_cdf, L.dyn_k, a, (uint32_t)t, (uint32_t)L.layer, sp.key0, sp.key1, k[0], k[1]);
    if (!offsets) {
      counts[2 * i] = k[0];
      counts[2 * i + 1] = k[1];
      continue;
    }
    for (int d = 0; d < 2; ++d) {
      int32_t* out = partners + offsets[2 * i + d];
      uint4 pw = make_uint4(0u, 0u, 0u, 0u);
      for (int j = 0; j < k[d]; ++j) {
        if ((j & 3) == 0) pw = dyn_partner_block(a, d, j, (uint32_t)t, (uint32_t)L.layer, sp.key0, sp.key1);
        out[j] = (int32_t)dyn_partner(word_of(pw, j & 3), n_local, thr, a, d, j, (uint32_t)t, (uint32_t)L.layer,
                                      sp.key0, sp.key1);
      }
    }
  }
}

// shared memory of the resident-bitmap variant, 0 when it cannot run
int64_t edge_res_smem(const covgpu_state* st) {
  if (st->n_sims != 1 || st->edge_tile < RES_THREADS * EDGE_VEC || st->n_segments > RES_MAX_SEGS) return 0;
  const int64_t words = (st->n + 31) >> 5;
  const int64_t static_bytes = (int64_t)sizeof(covgpu_layer) * RES_MAX_SEGS + (int64_t)sizeof(SimLite) + 64;
  const int64_t bytes = 16 * ((words + 3) >> 2) + (int64_t)(RES_THREADS / 32) * (int64_t)sizeof(EdgeQueue);
  static int max_optin = -1;
  if (max_optin < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      max_optin = 0;
  }
  return bytes + static_bytes <= max_optin ? bytes : 0;
}

int n_sms() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
  }
  return sms;
}

// raise the resident variant's dynamic shared-memory limit (before any capture)
template <bool LIK>
int configure_res(int64_t smem) {
  const void* fns[2] = {reinterpret_cast<const void*>(k_edge_pass_res<LIK, 4096>),
                        reinterpret_cast<const void*>(k_edge_pass_res<LIK, 8192>)};
  for (const void* f : fns)
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return COVGPU_CUDA_ERROR;
  return COVGPU_OK;
}
int configure_edge_pass(const covgpu_state* st) {
  if (!st->edge_resident) return COVGPU_OK;
  const int64_t smem = edge_res_smem(st);
  if (!smem) return COVGPU_BADARG;
  const int rc = configure_res<false>(smem);
  return rc ? rc : configure_res<true>(smem);
}

// one wave of k_edge_wave<LIK, R>: at most st->edge_wave blocks per SM
template <bool LIK, int R>
void launch_edge_wave_r(const covgpu_state* st, int t, cudaStream_t s) {
  static int64_t per_sm = -1;
  if (per_sm < 0) per_sm = wave_blocks(k_edge_wave<LIK, R>, EDGE_THREADS) / n_sms();
  const int64_t wave = (int64_t)n_sms() * (st->edge_wave < per_sm ? st->edge_wave : per_sm);
  const unsigned grid = (unsigned)(st->n_tiles < wave ? st->n_tiles : wave);
  launch_pdl(k_edge_wave<LIK, R>, grid, EDGE_THREADS, 0, s, *st, t);
}

template <bool LIK>
void launch_edge_tiles(const covgpu_state* st, int t, cudaStream_t s) {
  if (st->edge_wave > 0) {
    switch (st->edge_tile) {
      case 1024: launch_edge_wave_r<LIK, 1>(st, t, s); break;
      case 2048: launch_edge_wave_r<LIK, 2>(st, t, s); break;
      case 8192: launch_edge_wave_r<LIK, 8>(st, t, s); break;
      default: launch_edge_wave_r<LIK, 4>(st, t, s); break;
    }
    return;
  }
  const dim3 grid((unsigned)st->n_tiles);
  switch (st->edge_tile) {
    case 1024: launch_pdl(k_edge_pass<LIK, 1>, grid.x, EDGE_THREADS, 0, s, *st, t); break;
    case 2048: launch_pdl(k_edge_pass<LIK, 2>, grid.x, EDGE_THREADS, 0, s, *st, t); break;
    case 8192: launch_pdl(k_edge_pass<LIK, 8>, grid.x, EDGE_THREADS, 0, s, *st, t); break;
    default: launch_pdl(k_edge_pass<LIK, 4>, grid.x, EDGE_THREADS, 0, s, *st, t); break;
  }
}

template <bool LIK>
void launch_edge_res(const covgpu_state* st, int t, cudaStream_t s) {
  const int64_t smem = edge_res_smem(st);
  const unsigned grid = (unsigned)(st->n_tiles < n_sms() ? st->n_tiles : n_sms());
  if (st->edge_tile == 8192) launch_pdl(k_edge_pass_res<LIK, 8192>, grid, RES_THREADS, (size_t)smem, s, *st, t);
  else launch_pdl(k_edge_pass_res<LIK, 4096>, grid, RES_THREADS, (size_t)smem, s, *st, t);
}

// the stored layers' tile pass; with_walk: then the walk from the sources (when
// src_walk is on) as its own launch
int launch_stored_pass(const covgpu_state* st, int t, cudaStream_t s, bool with_walk) {
  if (st->n_tiles == 0) return COVGPU_OK;
  if (st->edge_resident) {
    if (st->lik.factor) launch_edge_res<true>(st, t, s);
    else launch_edge_res<false>(st, t, s);
  } else if (st->lik.factor) {
    launch_edge_tiles<true>(st, t, s);
  } else {
    launch_edge_tiles<false>(st, t, s);
  }
  const int rc = launch_status();
  return (rc || !with_walk) ? rc : launch_src_pass(st, t, s);
}

// the stored layers' tiles, then the redrawn layers' sources (parts: 0 both, 1 or 2
// one of them); the walk of the stored layers goes with the redrawn layers' pass
// when both run, else with the stored layers'
int launch_edge_pass(const covgpu_state* st, int t, cudaStream_t s, int parts = 0) {
  const bool walk_with_dyn = parts == 0 && st->n_dynamic > 0;
  const int rc = parts == 2 ? COVGPU_OK : launch_stored_pass(st, t, s, !walk_with_dyn);
  return (rc || parts == 1) ? rc : launch_dyn_pass(st, t, s, walk_with_dyn);
}

// The same two passes side by side: they read the same start-of-day state and
// only append events and claims with atomics, so the redrawn layers' pass runs
// on a side stream forked from s and joined back before anything after it
// (inside a capture the fork and join become edges of the graph).
cudaStream_t g_side_stream = nullptr;
cudaEvent_t g_fork_ev = nullptr, g_join_ev = nullptr;
int launch_edge_pass_forked(const covgpu_state* st, int t, cudaStream_t s) {
  if (st->n_tiles == 0 || st->n_dynamic == 0) return launch_edge_pass(st, t, s);
  if (!g_side_stream) {
    if (cudaStreamCreateWithFlags(&g_side_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&g_fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g_join_ev, cudaEventDisableTiming) != cudaSuccess)
      return COVGPU_CUDA_ERROR;
  }
  if (cudaEventRecord(g_fork_ev, s) != cudaSuccess || cudaStreamWaitEvent(g_side_stream, g_fork_ev, 0) != cudaSuccess)
    return COVGPU_CUDA_ERROR;
  int rc = launch_dyn_pass(st, t, g_side_stream, true);
  if (rc) return rc;
  if (cudaEventRecord(g_join_ev, g_side_stream) != cudaSuccess) return COVGPU_CUDA_ERROR;
  rc = launch_stored_pass(st, t, s, false);
  if (rc) return rc;
  return cudaStreamWaitEvent(s, g_join_ev, 0) == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
}

// per target: expected = 1 - prod(1 - p) and its per-layer sensitivities from
// the sums the likelihood edge pass left, which are cleared for the next day
__global__ void __launch_bounds__(AGENT_THREADS) k_lik_agents(covgpu_state st, int t) {
  constexpr int WARPS = AGENT_THREADS / 32;
  const covgpu_agent_block blk = st.agent_blocks[blockIdx.x];
  const covgpu_sim_params& sp = st.sims[blk.sim];
  const covgpu_lik& K = st.lik;
  const int64_t i = blk.begin + threadIdx.x;
  const bool valid = i < blk.end;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nl = sp.n_layers;
  __shared__ double s_e[WARPS];
  __shared__ double s_h[WARPS][COVGPU_MAX_LAYERS];
  const double lq = valid ? K.logq[i] : 0.0;
  const bool hit = lq != 0.0;  // a target of some candidate direction today
  double qprod = 0.0, e = 0.0;
  if (hit) {
    qprod = exp(lq);  // 0 for a certain transmission (lq = -inf)
    e = 1.0 - qprod;
    K.logq[i] = 0.0;
  }
  const bool any = __any_sync(0xffffffffu, hit);  // most warps have no target: skip the reductions
  if (lane == 0) s_e[warp] = 0.0;
  if (any) {
    e = warp_sum_d(e);
    if (lane == 0) s_e[warp] = e;
  }
  if (K.g_exp) {
    for (int l = 0; l < nl; ++l) {
      double h = 0.0;
      if (hit) {  // read and clear every layer's sum of a target, also when its product is 0
        double* wl = K.w + (int64_t)l * st.n + i;
        const double x = *wl;
        if (x != 0.0) { h = qprod * x; *wl = 0.0; }
      }
      if (any) h = warp_sum_d(h);
      if (lane == 0) s_h[warp][l] = any ? h : 0.0;
    }
  }
  __syncthreads();
  const int64_t day = (int64_t)blk.sim * K.npts_max + t;
  if (threadIdx.x == 0) {
    double x = 0.0;
    for (int k = 0; k < WARPS; ++k) x += s_e[k];
    if (x != 0.0) atomicAdd(K.expected + day, x);
  }
  if (K.g_exp && threadIdx.x < nl) {
    double x = 0.0;
    for (int k = 0; k < WARPS; ++k) x += s_h[k][threadIdx.x];
    if (x != 0.0) atomicAdd(K.g_exp + day * K.n_layers_max + threadIdx.x, x);
  }
}

int launch_lik_targets(const covgpu_state* st, int t, cudaStream_t s) {
  if (!st->lik.factor) return COVGPU_OK;
  k_lik_agents<<<(unsigned)st->n_agent_blocks, AGENT_THREADS, 0, s>>>(*st, t);
  return launch_status();
}

// ============================================================ infect

struct DrawSet {
  ff z[6];           // the six standard normals, float-float
  double u[4];       // injected uniforms (test mode)
  uint32_t uw[4];    // Philox words of the uniforms
  uint32_t w23[2];   // Philox words of the (sym2sev, sev2crit) normal pair, transformed on demand
  bool injected;
  // u_k < p exactly as float64 compares them (integer test for Philox words)
  __device__ __forceinline__ bool lt(int k, float p) const { return injected ? (u[k] < (double)p) : bern32(uw[k], p); }
  // the normals of the severe branch: only severe cases need them
  __device__ __forceinline__ void severe_normals() {
    if (!injected) box_muller_ff(w23[0], w23[1], COVGPU_LN_TAB, COVGPU_LN_INV, COVGPU_SINCOS_TAB, z[2], z[3]);
  }
};

__device__ __forceinline__ void get_draws(const covgpu_state& st, const covgpu_sim_params& sp, int64_t i,
                                          int64_t local, int t, int call_tag, DrawSet& d) {
  if (st.draw_table) {
    const double* r = st.draw_table + i * COVGPU_N_DRAWS;
#pragma unroll
    for (int k = 0; k < 6; ++k) d.z[k] = d2ff(r[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) d.u[k] = r[6 + k];
    d.injected = true;
    return;
  }
  d.injected = false;
  const uint32_t tag = TAG_INFECT | (uint32_t)call_tag;
  const uint4 b0 = philox(make_uint4((uint32_t)local, 0u, (uint32_t)t, tag), sp.key0, sp.key1);
  const uint4 b1 = philox(make_uint4((uint32_t)local, 1u, (uint32_t)t, tag), sp.key0, sp.key1);
  const uint4 b2 = philox(make_uint4((uint32_t)local, 2u, (uint32_t)t, tag), sp.key0, sp.key1);
  box_muller_ff(b0.x, b0.y, COVGPU_LN_TAB, COVGPU_LN_INV, COVGPU_SINCOS_TAB, d.z[0], d.z[1]);
  d.w23[0] = b0.z;
  d.w23[1] = b0.w;
  box_muller_ff(b1.x, b1.y, COVGPU_LN_TAB, COVGPU_LN_INV, COVGPU_SINCOS_TAB, d.z[4], d.z[5]);
  d.uw[0] = b1.z;
  d.uw[1] = b1.w;
  d.uw[2] = b2.x;
  d.uw[3] = b2.y;
}

// sev_imm[v] of agent i (flags f) as day t's check_immunity (immunity.py:303-350)
// forms it in the agent pass, from the same inputs (NAb, recovery date and
// variant, vaccination: infect() changes none of them before it reads this), for
// infect() alone reads it; the agent pass stores the array only on the last day
// of a launch sequence. Without waning the array is as set.
// (the same from the agent's nab, date_recovered and vstate, already loaded)
__device__ float sev_imm_with(const covgpu_state& st, const covgpu_sim_params& sp, int64_t i, int t, int v, uint32_t f,
                              float nab, float d_rec, uint32_t vs) {
  if (!sp.use_waning) return st.sev_imm[(int64_t)v * st.n + i];
  if (!(nab > 0.0f)) return 0.0f;
  ff ln_imm;
  const float imm = imm_of(st, sp, i, v, f, (float)t >= d_rec, (vs >> 16) & 0xFFu, ln_imm);
  if (!(imm > 0.0f)) return 0.0f;
  return ve_axis(sp, 2, ff_add(ff_log(nab, COVGPU_LN_TAB, COVGPU_LN_INV), ln_imm), COVGPU_EXP_TAB);
}
__device__ float sev_imm_of(const covgpu_state& st, const covgpu_sim_params& sp, int64_t i, int t, int v, uint32_t f) {
  if (!sp.use_waning) return st.sev_imm[(int64_t)v * st.n + i];
  return sev_imm_with(st, sp, i, t, v, f, st.nab[i], date_row(st, COVGPU_DATE_RECOVERED)[i], st.vstate[i]);
}

// people.py:435-586 for one agent (already deduplicated), plus update_peak_nab
// outcome bits of one infect_one call, tallied per warp by infect_tally
constexpr uint32_t O_INF = 1u, O_COUNT = 2u, O_REINF = 4u, O_SYMP = 8u, O_SEV = 16u;

__device__ uint32_t infect_one(const covgpu_state& st, const covgpu_sim_params& sp, int sim, int64_t i, int t, int v,
                               int32_t source, int layer_tag, int call_tag, bool hosp_max, bool icu_max) {
  uint32_t f = st.flags[i];
  if (!(f & B_SUS)) return 0u;  // people.py:468-472: keep only susceptibles
  const int64_t local = i - sp.agent_off;
  // people.py:486-491: breakthrough infections (peak_nab defined)
  const bool breakthrough = st.peak_nab[i] != 0.0f;
  if (breakthrough && st.n_breakthroughs[i] == 0) st.rel_trans[i] = __fmul_rn(st.rel_trans[i], sp.trans_redux);
  // people.py:494-505
  float* d_rec = date_row(st, COVGPU_DATE_RECOVERED);
  const bool reinfection = defined(d_rec[i]);
  f &= ~(B_SUS | B_NAIVE | B_REC | B_DIAG);
  f |= B_EXP | (1u << (EXPV_SHIFT + v));
  st.n_infections[i] += 1;
  if (breakthrough) st.n_breakthroughs[i] += 1;
  st.vstate[i] = (st.vstate[i] & 0xFFFFFF00u) | (uint32_t)v;
  // seed infections happen before update_states_pre resets the day's flows
  // (sim.py:571-577, people.py:171), so they are not counted; the counts and
  // the infection log record (people.py:508-511) are written by infect_tally
  const bool count = call_tag != CALL_TAG_SEED;
  uint32_t out = O_INF | (count ? O_COUNT : 0u) | (reinfection ? O_REINF : 0u);
  DrawSet d;
  get_draws(st, sp, i, local, t, call_tag, d);
  float* d_inf = date_row(st, COVGPU_DATE_INFECTIOUS);
  float* d_sym = date_row(st, COVGPU_DATE_SYMPTOMATIC);
  float* d_sev = date_row(st, COVGPU_DATE_SEVERE);
  float* d_crit = date_row(st, COVGPU_DATE_CRITICAL);
  float* d_dead = date_row(st, COVGPU_DATE_DEAD);
  float* u_exp2inf = dur_row(st, COVGPU_DUR_EXP2INF);
  float* u_inf2sym = dur_row(st, COVGPU_DUR_INF2SYM);
  float* u_sym2sev = dur_row(st, COVGPU_DUR_SYM2SEV);
  float* u_sev2crit = dur_row(st, COVGPU_DUR_SEV2CRIT);
  float* u_disease = dur_row(st, COVGPU_DUR_DISEASE);
  const float nanf_ = f32nan();
  const float tf = (float)t;
  // people.py:514-520
  const float de = (float)sample_ff(sp.dur[COVGPU_D_EXP2INF], d.z[0]);
  u_exp2inf[i] = de;
  date_row(st, COVGPU_DATE_EXPOSED)[i] = tf;
  const float di = __fadd_rn(de, tf);
  d_inf[i] = di;
  d_sym[i] = nanf_; d_sev[i] = nanf_; d_crit[i] = nanf_;
  date_row(st, COVGPU_DATE_DIAGNOSED)[i] = nanf_;
  float rec = nanf_;
  int symp_class;  // 0 asymptomatic, 1 mild, 2 severe (immunity.py:185-188)
  // people.py:523-527
  const float sp_symp = __fmul_rn(__fmul_rn(sp.rel_symp[v], st.symp_prob[i]),
                                  __fsub_rn(1.0f, symp_imm_of(st, i, v)));
  if (!d.lt(0, sp_symp)) {  // CASE 1: asymptomatic, people.py:530-532
    const double dr = sample_ff(sp.dur[COVGPU_D_ASYM2REC], d.z[4]);
    rec = (float)__dadd_rn((double)di, dr);
    u_disease[i] = (float)__dadd_rn((double)de, dr);
    symp_class = 0;
  } else {  // CASE 2: symptomatic, people.py:535-541
    const float dis = (float)sample_ff(sp.dur[COVGPU_D_INF2SYM], d.z[1]);
    u_inf2sym[i] = dis;
    const float ds = __fadd_rn(di, dis);
    d_sym[i] = ds;
    out |= O_SYMP;
    const float p_sev = __fmul_rn(__fmul_rn(sp.rel_severe[v], st.severe_prob[i]),
                                  __fsub_rn(1.0f, sev_imm_of(st, sp, i, t, v, f)));
    if (!d.lt(1, p_sev)) {  // CASE 2.1 mild, people.py:544-547
      const double dr = sample_ff(sp.dur[COVGPU_D_MILD2REC], d.z[4]);
      rec = (float)__dadd_rn((double)ds, dr);
      u_disease[i] = (float)__dadd_rn((double)__fadd_rn(de, dis), dr);
      symp_class = 1;
    } else {  // CASE 2.2 severe, people.py:550-554
      d.severe_normals();
      out |= O_SEV;
      const float dss = (float)sample_ff(sp.dur[COVGPU_D_SYM2SEV], d.z[2]);
      u_sym2sev[i] = dss;
      const float dsev = __fadd_rn(ds, dss);
      d_sev[i] = dsev;
      const float p_crit = __fmul_rn(__fmul_rn(sp.rel_crit[v], st.crit_prob[i]), hosp_max ? sp.no_hosp_factor : 1.0f);
      symp_class = 2;
      if (!d.lt(2, p_crit)) {  // CASE 2.2.1 not critical, people.py:557-559
        const double dr = sample_ff(sp.dur[COVGPU_D_SEV2REC], d.z[4]);
        rec = (float)__dadd_rn((double)dsev, dr);
        u_disease[i] = (float)__dadd_rn((double)__fadd_rn(__fadd_rn(de, dis), dss), dr);
      } else {  // CASE 2.2.2 critical, people.py:562-566
        const float dsc = (float)sample_ff(sp.dur[COVGPU_D_SEV2CRIT], d.z[3]);
        u_sev2crit[i] = dsc;
        const float dcrit = __fadd_rn(dsev, dsc);
        d_crit[i] = dcrit;
        const float p_death = __fmul_rn(__fmul_rn(sp.rel_death[v], st.death_prob[i]), icu_max ? sp.no_icu_factor : 1.0f);
        const float dsum = __fadd_rn(__fadd_rn(__fadd_rn(de, dis), dss), dsc);
        if (!d.lt(3, p_death)) {  // CASE 2.2.2.1 alive, people.py:569-571
          const double dr = sample_ff(sp.dur[COVGPU_D_CRIT2REC], d.z[4]);
          rec = (float)__dadd_rn((double)dcrit, dr);
          u_disease[i] = (float)__dadd_rn((double)dsum, dr);
        } else {  // CASE 2.2.2.2 dead, people.py:574-577
          const double dr = sample_ff(sp.dur[COVGPU_D_CRIT2DIE], d.z[4]);
          d_dead[i] = (float)__dadd_rn((double)dcrit, dr);
          u_disease[i] = (float)__dadd_rn((double)dsum, dr);
          rec = nanf_;
        }
      }
    }
  }
  d_rec[i] = rec;
  // people.py:580-584 -> immunity.py:138-202 update_peak_nab (natural infection)
  if (sp.use_waning) {
    if (st.nab[i] > 0.0f) {
      st.peak_nab[i] = __fmul_rn(st.peak_nab[i], sp.nab_boost);
    } else {
      const double init = sample_ff(sp.nab_init, d.z[5]);
      const double rel = symp_class == 0 ? sp.rel_imm_asymp : (symp_class == 1 ? sp.rel_imm_mild : sp.rel_imm_severe);
      st.peak_nab[i] = (float)__dmul_rn(__dmul_rn(exp2_ff(d2ff(init)), rel), sp.nab_norm);
    }
    st.t_nab_event[i] = t;
  }
  st.flags[i] = f;
  // no longer a target for the rest of the day (matters for infections before the edge pass)
  atomicAnd(st.roles + roles_words(st) + (i >> 5), ~(1u << (i & 31)));
  return out;
}

// infect_one split over a group of IG = 4 lanes (k_infect_claims). The draws of
// one infection are independent until the final sums: every lane derives the
// branch (symptomatic / severe / critical / dead) from the uniforms of Philox
// blocks 1 and 2, then lane 0 samples exp2inf and inf2sym (normals z0, z1),
// lane 1 sym2sev and sev2crit (z2, z3), lane 2 the recovery or death duration
// (z4) and lane 3 the initial NAb (z5); lane 0 gathers them with shuffles and
// does infect_one's sums and stores in infect_one's order, so the results are
// bit-identical to infect_one's. All 32 lanes of the warp must call it
// (shuffles); lanes of a group share i, win and the arguments. Returns the
// outcome bits in the group's lane 0, 0 elsewhere.
constexpr int IG = 4;  // lanes per infection (8, one sample per lane, measured 16% slower)
__device__ uint32_t infect_group(const covgpu_state& st, const covgpu_sim_params& sp, bool win, int64_t i, int t,
                                 int v, int call_tag, bool hosp_max, bool icu_max) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, r = lane & (IG - 1), g0 = lane & ~(IG - 1);
  const uint32_t f0 = win ? st.flags[i] : 0u;
  const bool act = win && (f0 & B_SUS);  // people.py:468-472: keep only susceptibles
  const int64_t local = i - sp.agent_off;
  const bool injected = st.draw_table != nullptr;
  const double* tab = injected ? st.draw_table + i * COVGPU_N_DRAWS : nullptr;
  const uint32_t tag = TAG_INFECT | (uint32_t)call_tag;
  // the agent's fields that the branch, the samples and the writes read, loaded
  // together with its flags: one round trip instead of one per level of the branch
  float a_symp = 0.0f, a_sev = 0.0f, a_crit = 0.0f, a_death = 0.0f, a_peak = 0.0f, a_nab = 0.0f, a_simm = 0.0f;
  float a_drec = 0.0f, a_rt = 0.0f;
  uint32_t a_vs = 0u;
  int32_t a_ninf = 0, a_nbt = 0;
  if (win) {
    a_symp = st.symp_prob[i];
    a_sev = st.severe_prob[i];
    a_crit = st.crit_prob[i];
    a_death = st.death_prob[i];
    a_peak = st.peak_nab[i];
    a_nab = st.nab[i];
    a_simm = st.symp_imm[(int64_t)v * st.n + i];
    a_drec = date_row(st, COVGPU_DATE_RECOVERED)[i];
    a_vs = st.vstate[i];
    a_ninf = st.n_infections[i];  // and the counters the writes update
    a_nbt = st.n_breakthroughs[i];
    a_rt = st.rel_trans[i];
  }
  // the branch: every lane of the group (people.py:523-566)
  bool symp = false, sev = false, crit = false, dead = false;
  uint4 b1 = make_uint4(0u, 0u, 0u, 0u);
  if (act) {
    uint32_t uw[4] = {0u, 0u, 0u, 0u};
    if (!injected) {
      b1 = philox(make_uint4((uint32_t)local, 1u, (uint32_t)t, tag), sp.key0, sp.key1);
      const uint4 b2 = philox(make_uint4((uint32_t)local, 2u, (uint32_t)t, tag), sp.key0, sp.key1);
      uw[0] = b1.z; uw[1] = b1.w; uw[2] = b2.x; uw[3] = b2.y;
    }
    auto lt = [&](int k, float p) { return injected ? (tab[6 + k] < (double)p) : bern32(uw[k], p); };
    // symp_imm as symp_imm_of reads it: 0 for an agent that never had NAbs
    const float sp_symp = __fmul_rn(__fmul_rn(sp.rel_symp[v], a_symp), __fsub_rn(1.0f, a_peak == 0.0f ? 0.0f : a_simm));
    symp = lt(0, sp_symp);
    if (symp) {
      const float p_sev = __fmul_rn(__fmul_rn(sp.rel_severe[v], a_sev),
                                    __fsub_rn(1.0f, sev_imm_with(st, sp, i, t, v, f0, a_nab, a_drec, a_vs)));
      sev = lt(1, p_sev);
      if (sev) {
        const float p_crit = __fmul_rn(__fmul_rn(sp.rel_crit[v], a_crit), hosp_max ? sp.no_hosp_factor : 1.0f);
        crit = lt(2, p_crit);
        if (crit) {
          const float p_death = __fmul_rn(__fmul_rn(sp.rel_death[v], a_death), icu_max ? sp.no_icu_factor : 1.0f);
          dead = lt(3, p_death);
        }
      }
    }
  }
  // This lane's normals and samples, in converged code: every lane of an acting
  // group runs the same Philox, Box-Muller and sampler instructions on its own
  // inputs (divergent per-lane branches would run one after another).
  // Lane 0: exp2inf, inf2sym (normals z0, z1); lane 1: sym2sev, sev2crit (z2, z3);
  // lane 2: the recovery or death duration (z4); lane 3: the initial NAb (z5).
  double s0 = 0.0, s1 = 0.0;
  float peak = 0.0f;
  if (act) {
    ff za, zb;
    if (injected) {
      const int k = 2 * (r < 2 ? r : 2);
      za = d2ff(tab[k]);
      zb = d2ff(tab[k + 1]);
    } else {
      const uint4 b0 = philox(make_uint4((uint32_t)local, 0u, (uint32_t)t, tag), sp.key0, sp.key1);
      const uint32_t wa = r == 0 ? b0.x : (r == 1 ? b0.z : b1.x);
      const uint32_t wb = r == 0 ? b0.y : (r == 1 ? b0.w : b1.y);
      box_muller_ff(wa, wb, COVGPU_LN_TAB, COVGPU_LN_INV, COVGPU_SINCOS_TAB, za, zb);
    }
    const int rec_d = !symp ? COVGPU_D_ASYM2REC : (!sev ? COVGPU_D_MILD2REC : (!crit ? COVGPU_D_SEV2REC
                                                                                : (dead ? COVGPU_D_CRIT2DIE
                                                                                        : COVGPU_D_CRIT2REC)));
    // first sample of every lane; the second of lanes 0 and 1 (the others repeat a
    // harmless one to stay converged)
    const covgpu_dur_par& p0 = r == 0 ? sp.dur[COVGPU_D_EXP2INF]
                                      : (r == 1 ? sp.dur[COVGPU_D_SYM2SEV] : (r == 2 ? sp.dur[rec_d] : sp.nab_init));
    const covgpu_dur_par& p1 = r == 0 ? sp.dur[COVGPU_D_INF2SYM] : (r == 1 ? sp.dur[COVGPU_D_SEV2CRIT] : p0);
    s0 = sample_ff(p0, r == 3 ? zb : za);
    s1 = sample_ff(p1, r < 2 ? zb : (r == 3 ? zb : za));
    if (r == 3 && sp.use_waning) {  // immunity.py:138-202 update_peak_nab (natural infection)
      if (a_nab > 0.0f) {
        peak = __fmul_rn(a_peak, sp.nab_boost);
      } else {
        const double rel = !symp ? sp.rel_imm_asymp : (!sev ? sp.rel_imm_mild : sp.rel_imm_severe);
        peak = (float)__dmul_rn(__dmul_rn(exp2_ff(d2ff(s0)), rel), sp.nab_norm);
      }
    }
  }
  const double v_exp2inf = __shfl_sync(full, s0, g0), v_inf2sym = __shfl_sync(full, s1, g0);
  const double v_sym2sev = __shfl_sync(full, s0, g0 + 1), v_sev2crit = __shfl_sync(full, s1, g0 + 1);
  const double v_rec = __shfl_sync(full, s0, g0 + 2);
  const float v_peak = __shfl_sync(full, peak, g0 + 3);
  if (r != 0 || !act) return 0u;

  uint32_t f = f0;
  // people.py:486-491: breakthrough infections (peak_nab defined)
  const bool breakthrough = a_peak != 0.0f;
  if (breakthrough && a_nbt == 0) st.rel_trans[i] = __fmul_rn(a_rt, sp.trans_redux);
  float* d_rec = date_row(st, COVGPU_DATE_RECOVERED);
  const bool reinfection = defined(a_drec);
  f &= ~(B_SUS | B_NAIVE | B_REC | B_DIAG);
  f |= B_EXP | (1u << (EXPV_SHIFT + v));
  st.n_infections[i] = a_ninf + 1;
  if (breakthrough) st.n_breakthroughs[i] = a_nbt + 1;
  st.vstate[i] = (a_vs & 0xFFFFFF00u) | (uint32_t)v;
  const bool count = call_tag != CALL_TAG_SEED;
  uint32_t out = O_INF | (count ? O_COUNT : 0u) | (reinfection ? O_REINF : 0u);
  float* d_inf = date_row(st, COVGPU_DATE_INFECTIOUS);
  float* d_sym = date_row(st, COVGPU_DATE_SYMPTOMATIC);
  float* d_sev = date_row(st, COVGPU_DATE_SEVERE);
  float* d_crit = date_row(st, COVGPU_DATE_CRITICAL);
  float* d_dead = date_row(st, COVGPU_DATE_DEAD);
  float* u_disease = dur_row(st, COVGPU_DUR_DISEASE);
  const float nanf_ = f32nan();
  const float tf = (float)t;
  const float de = (float)v_exp2inf;  // people.py:514-520
  dur_row(st, COVGPU_DUR_EXP2INF)[i] = de;
  date_row(st, COVGPU_DATE_EXPOSED)[i] = tf;
  const float di = __fadd_rn(de, tf);
  d_inf[i] = di;
  d_sym[i] = nanf_; d_sev[i] = nanf_; d_crit[i] = nanf_;
  date_row(st, COVGPU_DATE_DIAGNOSED)[i] = nanf_;
  float rec = nanf_;
  const double dr = v_rec;
  if (!symp) {  // CASE 1: asymptomatic, people.py:530-532
    rec = (float)__dadd_rn((double)di, dr);
    u_disease[i] = (float)__dadd_rn((double)de, dr);
  } else {  // CASE 2: symptomatic, people.py:535-541
    const float dis = (float)v_inf2sym;
    dur_row(st, COVGPU_DUR_INF2SYM)[i] = dis;
    const float ds = __fadd_rn(di, dis);
    d_sym[i] = ds;
    out |= O_SYMP;
    if (!sev) {  // CASE 2.1 mild, people.py:544-547
      rec = (float)__dadd_rn((double)ds, dr);
      u_disease[i] = (float)__dadd_rn((double)__fadd_rn(de, dis), dr);
    } else {  // CASE 2.2 severe, people.py:550-554
      out |= O_SEV;
      const float dss = (float)v_sym2sev;
      dur_row(st, COVGPU_DUR_SYM2SEV)[i] = dss;
      const float dsev = __fadd_rn(ds, dss);
      d_sev[i] = dsev;
      if (!crit) {  // CASE 2.2.1 not critical, people.py:557-559
        rec = (float)__dadd_rn((double)dsev, dr);
        u_disease[i] = (float)__dadd_rn((double)__fadd_rn(__fadd_rn(de, dis), dss), dr);
      } else {  // CASE 2.2.2 critical, people.py:562-566
        const float dsc = (float)v_sev2crit;
        dur_row(st, COVGPU_DUR_SEV2CRIT)[i] = dsc;
        const float dcrit = __fadd_rn(dsev, dsc);
        d_crit[i] = dcrit;
        const float dsum = __fadd_rn(__fadd_rn(__fadd_rn(de, dis), dss), dsc);
        if (!dead) {  // CASE 2.2.2.1 alive, people.py:569-571
          rec = (float)__dadd_rn((double)dcrit, dr);
          u_disease[i] = (float)__dadd_rn((double)dsum, dr);
        } else {  // CASE 2.2.2.2 dead, people.py:574-577
          d_dead[i] = (float)__dadd_rn((double)dcrit, dr);
          u_disease[i] = (float)__dadd_rn((double)dsum, dr);
        }
      }
    }
  }
  d_rec[i] = rec;
  if (sp.use_waning) {  // people.py:580-584
    st.peak_nab[i] = v_peak;
    st.t_nab_event[i] = t;
  }
  st.flags[i] = f;
  // no longer a target for the rest of the day
  atomicAnd(st.roles + roles_words(st) + (i >> 5), ~(1u << (i & 31)));
  return out;
}

// The day's counts (people.py:172-180 flows of infect) and the infection-log
// records of one warp's infect_one calls: one log atomic per warp, and one
// atomic per counter for each group of lanes with the same sim and variant.
// All 32 lanes call it (lanes without an infection pass out = 0).
__device__ void infect_tally(const covgpu_state& st, int t, uint32_t out, int sim, int v, int32_t source,
                             int32_t target_local, int layer_tag) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const bool inf = out & O_INF;
  if (st.log) {
    const unsigned m = __ballot_sync(full, inf);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(st.log_count, (unsigned long long)__popc(m));
      base = __shfl_sync(full, base, leader);
      if (inf) {
        const unsigned long long pos = base + __popc(m & ((1u << lane) - 1u));
        if ((int64_t)pos < st.log_capacity) {
          covgpu_log_rec r;
          r.source = source; r.target = target_local; r.day = t;
          r.layer_variant = (layer_tag & 0xFF) | (v << 8) | (sim << 16);
          st.log[pos] = r;
        } else {
          atomicOr(st.status, COVGPU_OVERFLOW);
        }
      }
    }
  }
  const bool cnt = inf && (out & O_COUNT);
  const unsigned b_inf = __ballot_sync(full, cnt);
  if (!b_inf) return;
  const unsigned grp = __match_any_sync(full, cnt ? (((unsigned)sim << 8) | (unsigned)v) : 0xffffffffu);
  const unsigned b_re = __ballot_sync(full, cnt && (out & O_REINF));
  const unsigned b_sy = __ballot_sync(full, cnt && (out & O_SYMP));
  const unsigned b_sv = __ballot_sync(full, cnt && (out & O_SEV));
  if (!cnt || lane != __ffs(grp) - 1) return;  // one leader per (sim, variant) group
  const covgpu_sim_params& sp = st.sims[sim];
  const int nv = sp.n_variants;
  unsigned long long* ri = reinterpret_cast<unsigned long long*>(sp.res_int + (int64_t)t * COVGPU_N_RES_INT);
  unsigned long long* rv = reinterpret_cast<unsigned long long*>(sp.res_var + (int64_t)t * COVGPU_N_RES_VAR * nv);
  const unsigned n_inf = __popc(b_inf & grp), n_re = __popc(b_re & grp), n_sy = __popc(b_sy & grp),
                 n_sv = __popc(b_sv & grp);
  atomicAdd(ri + R_INFECTIONS, (unsigned long long)n_inf);
  if (n_re) atomicAdd(ri + R_REINFECTIONS, (unsigned long long)n_re);
  atomicAdd(rv + RV_INFECTIONS * nv + v, (unsigned long long)n_inf);
  if (n_sy) atomicAdd(rv + RV_SYMPTOMATIC * nv + v, (unsigned long long)n_sy);
  if (n_sv) atomicAdd(rv + RV_SEVERE * nv + v, (unsigned long long)n_sv);
}

__device__ __forceinline__ int sim_of(const covgpu_state& st, int64_t i) {
  int lo = 0, hi = st.n_sims - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (st.sims[mid].agent_off <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// sim.py:579-580: beds exceeded, from the severe/critical counts after the day's transitions
__device__ __forceinline__ void hosp_icu(const covgpu_state& st, const covgpu_sim_params& sp, int s, int t,
                                         bool& hosp, bool& icu) {
  if (st.hospicu) { hosp = st.hospicu[2 * s] != 0; icu = st.hospicu[2 * s + 1] != 0; return; }
  const int64_t* r = sp.res_int + (int64_t)t * COVGPU_N_RES_INT;
  hosp = sp.n_beds_hosp >= 0 && r[COVGPU_RES_SEVERE_NOW] > sp.n_beds_hosp;
  icu = sp.n_beds_icu >= 0 && r[COVGPU_RES_CRITICAL_NOW] > sp.n_beds_icu;
}

__global__ void k_infect_claims(covgpu_state st, int t) {
  pdl_wait();
  pdl_trigger();  // the next day's agent pass may set up while the infections run
  if (held(st, t)) return;
  const unsigned long long cnt = *st.event_count;
  const int64_t n = (int64_t)cnt < st.event_capacity ? (int64_t)cnt : st.event_capacity;
  // IG lanes per event, 32 / IG events per warp and iteration; warp-uniform trip
  // count (the shuffles of infect_group and the ballots of infect_tally need every lane)
  constexpr int EPW = 32 / IG;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * EPW; base < n; base += n_warps * EPW) {
    const int64_t j = base + lane / IG;
    bool win = false;
    int s = 0, v = 0, layer = 0;
    int32_t src = -1, tgt = 0;
    int64_t target = 0;
    if (j < n) {
      const covgpu_event ev = st.events[j];
      win = st.claim[ev.target] == ev.key;  // the first infector of this target
      if (win) {
        target = ev.target;
        s = sim_of(st, ev.target);
        v = (int)((ev.key >> 45) & 7u);
        layer = (int)((ev.key >> 41) & 15u);
        src = (int32_t)(ev.source - st.sims[s].agent_off);
        tgt = (int32_t)(ev.target - st.sims[s].agent_off);
      }
    }
    const covgpu_sim_params& sp = st.sims[s];
    bool hosp = false, icu = false;
    if (win) hosp_icu(st, sp, s, t, hosp, icu);
    const uint32_t out = infect_group(st, sp, win, target, t, v, 0, hosp, icu);
    infect_tally(st, t, out, s, v, src, tgt, layer);
  }
}

__global__ void k_infect_list(covgpu_state st, int t, const int32_t* inds, const int32_t* sources, int64_t n, int sim,
                              int v, int layer_tag, int call_tag, uint8_t* infected) {
  const covgpu_sim_params& sp = st.sims[sim];
  bool hosp, icu;
  hosp_icu(st, sp, sim, t, hosp, icu);
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    uint32_t out = 0;
    int32_t tgt = 0, src = -1;
    if (j < n) {
      tgt = (int32_t)(inds[j] - sp.agent_off);
      if (sources) src = sources[j];
      out = infect_one(st, sp, sim, inds[j], t, v, src, layer_tag, call_tag, hosp, icu);
      if (infected) infected[j] = (out & O_INF) ? 1 : 0;
    }
    infect_tally(st, t, out, sim, v, src, tgt, layer_tag);
  }
}

// sim.py:582-587: the agents drawn for day t (every sim's, precomputed on the
// host: neither the Poisson count nor the choice depends on the state) are
// infected with the wild type from the importation "layer", on infection
// stream CALL_TAG_IMPORT. The trip count is uniform across each block (the
// ballots of infect_tally need every lane); lanes of one warp may belong to
// different sims.
__global__ void k_import_day(covgpu_state st, int t) {
  if (held(st, t)) return;
  const int64_t b = st.import_day_off[t], e = st.import_day_off[t + 1];
  for (int64_t base = b + (int64_t)blockIdx.x * blockDim.x; base < e; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    uint32_t out = 0;
    int32_t tgt = 0, s = 0;
    if (j < e) {
      const int64_t i = st.imports[j];
      s = st.import_sims[j];
      if (s >= 0 && s < st.n_sims && i >= st.sims[s].agent_off && i < st.sims[s].agent_off + st.sims[s].n_agents) {
        const covgpu_sim_params& sp = st.sims[s];
        bool hosp, icu;
        hosp_icu(st, sp, s, t, hosp, icu);
        tgt = (int32_t)(i - sp.agent_off);
        out = infect_one(st, sp, s, i, t, 0, -1, COVGPU_MAX_LAYERS + 1, CALL_TAG_IMPORT, hosp, icu);
      } else {
        atomicOr(st.status, COVGPU_BADARG);
        s = 0;
      }
    }
    infect_tally(st, t, out, s, 0, -1, tgt, COVGPU_MAX_LAYERS + 1);
  }
}

// sim.py:535-547, the test only: is a rescaling due at the start of day t? The
// count of agents not naive grows by the day's first infections (infections
// less reinfections; an agent's first infection clears naive, and only a
// recovered agent is reinfected); the host sets it after seeding and after
// each rescaling. One thread per sim.
__global__ void k_rescale_check(covgpu_state st, int t) {
  if (held(st, t)) return;
  for (int s = threadIdx.x; s < st.n_sims; s += blockDim.x) {
    const covgpu_sim_params& sp = st.sims[s];
    if (!sp.rescale_vec || t >= sp.npts) continue;
    int64_t nn = sp.nonnaive[0];
    for (int64_t d = sp.nonnaive[1] + 1; d <= t - 1; ++d) {
      const int64_t* r = sp.res_int + d * COVGPU_N_RES_INT;
      nn += r[R_INFECTIONS] - r[R_REINFECTIONS];
    }
    if (sp.nonnaive[1] < t - 1) {
      sp.nonnaive[0] = nn;
      sp.nonnaive[1] = t - 1;
    }
    if (sp.nonnaive[2] >= t) continue;
    if (sp.rescale_vec[t] < sp.pop_scale && (double)nn / (double)sp.n_agents > sp.rescale_threshold)
      atomicMin(st.hold, t);
    else
      sp.nonnaive[2] = t;
  }
}

// ------------------------------------------------------------ graph cache for covgpu_run_days
// An entry is made the first time a (state, range) is run, which launches the
// days directly: a run made once does not pay for the capture (about 5 ms for
// 181 days of a 1M-agent sim, against 1.4 ms of launch time the graph saves).
// The second run captures and instantiates the graph, later runs replay it.
struct GraphEntry {
  bool used = false;
  covgpu_state st;
  int t0 = 0, t1 = 0, open_prev = 0, close_last = 0;
  cudaGraphExec_t exec = nullptr;  // null: run once, not captured yet
};
// entries: the checkpoint segments of a likelihood run in both modes, or a few
// hundred sims each run on its own state
constexpr int N_GRAPHS = 320;
GraphEntry g_graphs[N_GRAPHS];
int g_graph_next = 0;
cudaStream_t g_capture_stream = nullptr;  // private stream for captures (the legacy stream cannot capture)

// Grid of the agent pass: one wave of resident blocks (the SM count of the current
// device times the blocks per SM the pass's registers allow), or fewer when the
// state has fewer agent blocks. Any grid gives the same results.
unsigned agent_grid(const covgpu_state* st) {
  static const int64_t wave = [] {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent_step, AGENT_THREADS, 0) != cudaSuccess) {
      cudaGetLastError();
      return (int64_t)1 << 30;  // no wave bound: one block per agent block
    }
    return (int64_t)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  }();
  const int64_t nb = st->n_agent_blocks;
  return (unsigned)(nb < wave ? (nb > 0 ? nb : 1) : wave);
}

int enqueue_days(const covgpu_state* st, int t0, int t1, int open_prev, int close_last, cudaStream_t s) {
  for (int t = t0; t < t1; ++t) {
    if (st->hold) k_rescale_check<<<1, 128, 0, s>>>(*st, t);
    launch_pdl(k_agent_step, agent_grid(st), AGENT_THREADS, 0, s, *st, t, (t > t0 || open_prev) ? 1 : 0, 1,
               t == t1 - 1 ? 1 : 0, t > t0 ? 1 : 0);
    if (t < st->import_days) k_import_day<<<IMPORT_BLOCKS, 256, 0, s>>>(*st, t);
    launch_test_trace(st, t, s);
    const int rc = launch_edge_pass_forked(st, t, s);
    if (rc) return rc;
    launch_lik_targets(st, t, s);
    launch_pdl(k_infect_claims, (unsigned)grid_for(st->n / 8 + 1, 256, 152 * 4), 256, 0, s, *st, t);
  }
  if (close_last) launch_pdl(k_agent_step, agent_grid(st), AGENT_THREADS, 0, s, *st, t1, 1, 0, 0, 1);
  return launch_status();
}

}  // namespace

// ============================================================ C ABI

namespace covgpu {

int check_state(const covgpu_state* st) {
  if (!st || st->n <= 0 || st->n_sims <= 0 || st->n_agent_blocks <= 0) return COVGPU_BADARG;
  if (!st->flags || !st->vstate || !st->sims || !st->agent_blocks || !st->roles || !st->claim || !st->src_rec ||
      !st->tgt_rec ||
      !st->events ||
      !st->event_count || !st->status)
    return COVGPU_BADARG;
  if ((st->n_tiles > 0 || st->n_dynamic > 0) && (!st->segments || st->n_segments <= 0)) return COVGPU_BADARG;
  if (st->n_dynamic < 0 || st->n_dynamic > st->n_segments) return COVGPU_BADARG;
  if (st->n_agent_blocks > 0x7FFFFFFF || st->n_tiles > 0x7FFFFFFF) return COVGPU_BADARG;
  if (st->edge_tile != 1024 && st->edge_tile != 2048 && st->edge_tile != 4096 && st->edge_tile != 8192)
    return COVGPU_BADARG;
  if (st->edge_resident && (!edge_res_smem(st) || (reinterpret_cast<uintptr_t>(st->roles) & 15u))) return COVGPU_BADARG;
  if (st->edge_wave < 0 || (st->edge_wave > 0 && st->edge_resident)) return COVGPU_BADARG;
  if (st->has_testing && (!st->trace_bits || !st->contact_bits || !st->pending_quar || !st->trace_count ||
                          st->pending_slots < 1 || st->n_contact_layers < 1))
    return COVGPU_BADARG;
  if (st->import_days < 0 || (st->import_days > 0 && (!st->import_day_off || !st->imports || !st->import_sims)))
    return COVGPU_BADARG;
  const covgpu_lik& K = st->lik;
  if (K.factor && (!K.ll || !K.expected || !K.logq || (K.g_exp && !K.w) || K.npts_max < 1 ||
                   K.n_layers_max < 1 || K.n_layers_max > COVGPU_MAX_LAYERS || K.nv_max < 1))
    return COVGPU_BADARG;
  return COVGPU_OK;
}

}  // namespace covgpu


extern "C" {

int covgpu_version(void) { return 1; }

int covgpu_abi_layout(int64_t* out, int32_t n) {
  const int64_t v[] = {(int64_t)sizeof(covgpu_sim_params), (int64_t)sizeof(covgpu_layer),
                       (int64_t)sizeof(covgpu_agent_block), (int64_t)sizeof(covgpu_event),
                       (int64_t)sizeof(covgpu_log_rec), (int64_t)sizeof(covgpu_state),
                       (int64_t)offsetof(covgpu_state, sims), (int64_t)offsetof(covgpu_state, edge_uniforms),
                       (int64_t)offsetof(covgpu_sim_params, res_fx), (int64_t)sizeof(covgpu_testing),
                       (int64_t)offsetof(covgpu_sim_params, testing), (int64_t)offsetof(covgpu_state, pending_quar),
                       (int64_t)offsetof(covgpu_state, trace_count), (int64_t)sizeof(covgpu_lik),
                       (int64_t)offsetof(covgpu_state, lik), (int64_t)offsetof(covgpu_state, import_day_off),
                       (int64_t)offsetof(covgpu_sim_params, pop_scale), (int64_t)offsetof(covgpu_state, hold)};
  const int m = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n && i < m; ++i) out[i] = v[i];
  return m;
}


int covgpu_agent_step(const covgpu_state* st, int32_t t, int32_t do_prev, int32_t do_day, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF) return COVGPU_BADARG;
  if (do_day & ~(1 | COVGPU_DAY_STEADY)) return COVGPU_BADARG;
  const int day = do_day & 1, steady = (!day || (do_day & COVGPU_DAY_STEADY)) ? 1 : 0;
  k_agent_step<<<agent_grid(st), AGENT_THREADS, 0, S(stream)>>>(*st, t, do_prev, day, 1, steady);
  return launch_status();
}

int64_t covgpu_edge_resident_bytes(const covgpu_state* st) {
  if (!st || st->n <= 0) return 0;
  covgpu_state probe = *st;
  if (probe.edge_tile < RES_THREADS * EDGE_VEC) probe.edge_tile = RES_THREADS * EDGE_VEC;
  return edge_res_smem(&probe);
}

int covgpu_edge_pass(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF) return COVGPU_BADARG;
  if (st->edge_parts < 0 || st->edge_parts > 2) return COVGPU_BADARG;
  rc = configure_edge_pass(st);
  if (rc) return rc;
  return launch_edge_pass(st, t, S(stream), st->edge_parts);
}

int covgpu_lik_targets(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF || !st->lik.factor) return COVGPU_BADARG;
  return launch_lik_targets(st, t, S(stream));
}

int covgpu_infect_claims(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  k_infect_claims<<<grid_for(st->n / 8 + 1, 256, 152 * 4), 256, 0, S(stream)>>>(*st, t);
  return launch_status();
}

int covgpu_infect_list(const covgpu_state* st, int32_t t, const int32_t* inds, const int32_t* sources, int64_t n_inds,
                       int32_t sim, int32_t variant, int32_t layer_tag, int32_t call_tag, uint8_t* infected,
                       void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (n_inds < 0 || sim < 0 || sim >= st->n_sims || variant < 0 || variant >= COVGPU_MAX_VARIANTS) return COVGPU_BADARG;
  if (n_inds == 0) return COVGPU_OK;
  if (!inds) return COVGPU_BADARG;
  k_infect_list<<<grid_for(n_inds, 128), 128, 0, S(stream)>>>(*st, t, inds, sources, n_inds, sim, variant, layer_tag,
                                                               call_tag, infected);
  return launch_status();
}

int covgpu_import_day(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF) return COVGPU_BADARG;
  if (t >= st->import_days) return COVGPU_OK;
  k_import_day<<<IMPORT_BLOCKS, 256, 0, S(stream)>>>(*st, t);
  return launch_status();
}

int covgpu_rescale_check(const covgpu_state* st, int32_t t, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t < 0 || t >= 0xFFFF || !st->hold) return COVGPU_BADARG;
  k_rescale_check<<<1, 128, 0, S(stream)>>>(*st, t);
  return launch_status();
}

int covgpu_layer_lists(const covgpu_state* st, int32_t segment, int32_t t, int64_t agent_begin, int64_t n_agents,
                       int32_t* counts, const int64_t* offsets, int32_t* partners, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (segment < 0 || segment >= st->n_segments || t < 0 || t >= 0xFFFF || agent_begin < 0 || n_agents < 0 ||
      (offsets ? !partners : !counts))
    return COVGPU_BADARG;
  if (n_agents == 0) return COVGPU_OK;
  k_layer_lists<<<grid_for(n_agents, 256), 256, 0, S(stream)>>>(*st, segment, t, agent_begin, n_agents, counts,
                                                                 offsets, partners);
  return launch_status();
}

int covgpu_run_days(const covgpu_state* st, int32_t t0, int32_t t1, int32_t open_prev, int32_t close_last,
                    int32_t use_graph, void* stream) {
  int rc = check_state(st);
  if (rc) return rc;
  if (t0 < 0 || t1 < t0 || t1 >= 0xFFFF) return COVGPU_BADARG;
  open_prev = (open_prev && t0 > 0) ? 1 : 0;
  rc = configure_edge_pass(st);  // function attributes: outside any capture
  if (rc) return rc;
  cudaStream_t s = S(stream);
  if (!use_graph) return enqueue_days(st, t0, t1, open_prev, close_last, s);
  GraphEntry* hit = nullptr;
  for (auto& g : g_graphs)
    if (g.used && g.t0 == t0 && g.t1 == t1 && g.close_last == close_last && g.open_prev == open_prev &&
        memcmp(&g.st, st, sizeof(covgpu_state)) == 0) { hit = &g; break; }
  if (!hit) {  // first run of this state and range: direct launches, remembered
    GraphEntry& g = g_graphs[g_graph_next];
    g_graph_next = (g_graph_next + 1) % N_GRAPHS;
    if (g.used && g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    g.st = *st; g.t0 = t0; g.t1 = t1; g.open_prev = open_prev; g.close_last = close_last; g.used = true;
    return enqueue_days(st, t0, t1, open_prev, close_last, s);
  }
  if (!hit->exec) {  // second run: capture
    if (!g_capture_stream && cudaStreamCreateWithFlags(&g_capture_stream, cudaStreamNonBlocking) != cudaSuccess)
      return COVGPU_CUDA_ERROR;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(g_capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return COVGPU_CUDA_ERROR;
    const int erc = enqueue_days(st, t0, t1, open_prev, close_last, g_capture_stream);
    if (cudaStreamEndCapture(g_capture_stream, &graph) != cudaSuccess || erc != COVGPU_OK) {
      if (graph) cudaGraphDestroy(graph);
      return COVGPU_CUDA_ERROR;
    }
    cudaGraphExec_t exec = nullptr;
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) { cudaGraphDestroy(graph); return COVGPU_CUDA_ERROR; }
    cudaGraphDestroy(graph);
    hit->exec = exec;
  }
  return cudaGraphLaunch(hit->exec, s) == cudaSuccess ? COVGPU_OK : COVGPU_CUDA_ERROR;
}

}  // extern "C"
