/*
 * covgpu.h -- C ABI of the GB300 (sm_103a) implementation of Covasim 3.1.7's
 * per-day step hot path.
 *
 * Every entry point takes device pointers, sizes and a cudaStream_t (passed
 * as void*), enqueues work on that stream, never synchronises unless stated,
 * never frees caller memory and returns an int status (COVGPU_*); no entry
 * point traps or asserts on the device. Data-dependent failures found on the
 * device (buffer overflow) are reported in a device status word that the
 * caller reads back when convenient.
 *
 * Reference interfaces replaced (paths inside the Covasim source tree):
 *   covgpu_viral_load        covasim/utils.py:38-79   compute_viral_load
 *   covgpu_trans_sus         covasim/utils.py:81-90   compute_trans_sus
 *   covgpu_infections        covasim/utils.py:92-128  compute_infections
 *   covgpu_agent_step        covasim/people.py:164-186 update_states_pre (+ the checks at
 *                            people.py:211-312,368-374), covasim/immunity.py:303-350
 *                            check_immunity, immunity.py:205-213 update_nab and the
 *                            per-day counts of covasim/sim.py:651-674
 *   covgpu_edge_pass         covasim/sim.py:601-649: viral load + compute_trans_sus +
 *                            compute_infections over every variant and layer, with the
 *                            dynamic-layer resampling of covasim/base.py:1849-1876
 *   covgpu_infect_claims     covasim/people.py:435-586 infect (+ immunity.py:138-202
 *                            update_peak_nab) for the day's transmissions
 *   covgpu_infect_list       covasim/people.py:435-586 infect for an explicit index list
 *                            (seed infections, sim.py:505-532; variant importations,
 *                            immunity.py:117-130)
 *   covgpu_import_day        covasim/sim.py:582-587 the day's Poisson importations
 *   covgpu_layer_lists       covasim/base.py:1849-1876 Layer.update: a dynamic layer's day-t
 *                            edges, as per-agent lists
 *   covgpu_check             covasim/people.py:222-312,368-374 People.check_infectious ...
 *                            check_death, check_exit_iso, one at a time
 *   covgpu_check_immunity    covasim/immunity.py:303-350 check_immunity
 *   covgpu_update_nab        covasim/immunity.py:205-213 update_nab
 *   covgpu_update_peak_nab   covasim/immunity.py:138-202 update_peak_nab
 */
#ifndef COVGPU_H
#define COVGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define COVGPU_OK          0
#define COVGPU_OVERFLOW    1   /* a fixed-capacity device buffer was too small */
#define COVGPU_TIMEOUT     2   /* a bounded device wait gave up                */
#define COVGPU_BADARG      3   /* rejected on the host before any launch       */
#define COVGPU_CUDA_ERROR  4   /* a CUDA runtime call failed                   */

/* ---- limits ------------------------------------------------------------ */
#define COVGPU_MAX_VARIANTS 8
#define COVGPU_MAX_LAYERS   16
#define COVGPU_N_DATES      19
#define COVGPU_N_DURS       5
#define COVGPU_N_DRAWS      10  /* draws consumed by one infection (see covgpu_infect_*) */

/* ---- packed per-agent state word (bit i of flags) ---------------------- */
/* bits 0..15 are defaults.py:59-76 in order: susceptible, naive, exposed,
 * infectious, symptomatic, severe, critical, tested, diagnosed, recovered,
 * known_dead, dead, known_contact, quarantined, isolated, vaccinated;
 * bits 16..23 exposed_by_variant[v]; bits 24..31 infectious_by_variant[v]. */
#define COVGPU_NO_VARIANT 0xFFu  /* byte value of an undefined variant field */

/* date block rows (index into dates[COVGPU_N_DATES][n]) */
enum {
  COVGPU_DATE_SUSCEPTIBLE = 0, COVGPU_DATE_NAIVE, COVGPU_DATE_EXPOSED, COVGPU_DATE_INFECTIOUS,
  COVGPU_DATE_SYMPTOMATIC, COVGPU_DATE_SEVERE, COVGPU_DATE_CRITICAL, COVGPU_DATE_TESTED,
  COVGPU_DATE_DIAGNOSED, COVGPU_DATE_RECOVERED, COVGPU_DATE_KNOWN_DEAD, COVGPU_DATE_DEAD,
  COVGPU_DATE_KNOWN_CONTACT, COVGPU_DATE_QUARANTINED, COVGPU_DATE_ISOLATED,
  COVGPU_DATE_VACCINATED, COVGPU_DATE_POS_TEST, COVGPU_DATE_END_QUARANTINE,
  COVGPU_DATE_END_ISOLATION
};
enum { COVGPU_DUR_EXP2INF = 0, COVGPU_DUR_INF2SYM, COVGPU_DUR_SYM2SEV, COVGPU_DUR_SEV2CRIT,
       COVGPU_DUR_DISEASE };

/* duration distributions (utils.py:156-236 sample(), one standard normal per draw) */
enum { COVGPU_DIST_LOGNORMAL_INT = 0, COVGPU_DIST_LOGNORMAL, COVGPU_DIST_NORMAL,
       COVGPU_DIST_NORMAL_INT, COVGPU_DIST_NORMAL_POS, COVGPU_DIST_ZERO };
/* order of the nine duration parameters in covgpu_sim_params.dur */
enum { COVGPU_D_EXP2INF = 0, COVGPU_D_INF2SYM, COVGPU_D_SYM2SEV, COVGPU_D_SEV2CRIT,
       COVGPU_D_ASYM2REC, COVGPU_D_MILD2REC, COVGPU_D_SEV2REC, COVGPU_D_CRIT2REC,
       COVGPU_D_CRIT2DIE, COVGPU_N_DUR_PARS };

/* per-sim-day integer results: the 15 flows of defaults.py:167-183, then the
 * 13 stocks of defaults.py:145-159, then the severe/critical counts seen by
 * infect() that day (sim.py:579-580) */
#define COVGPU_N_RES_INT 30
#define COVGPU_RES_SEVERE_NOW 28
#define COVGPU_RES_CRITICAL_NOW 29
/* per-sim-day-variant integer results: 4 variant flows (defaults.py:185-190),
 * then the 2 by-variant stocks (defaults.py:160-163) */
#define COVGPU_N_RES_VAR 6
/* per-sim-day float sums, as signed 64-bit fixed point (integer atomics make
 * them independent of block order, so every run gives the same bits): sum of
 * NAbs of the living (sim.py:672) scaled by 2^24, sums of sus_imm and of
 * symp_imm over [nv, n] (sim.py:673-674) scaled by 2^32; the host divides */
#define COVGPU_N_RES_F 3
#define COVGPU_FX_NAB_BITS 24
#define COVGPU_FX_IMM_BITS 32

/* ---- device-side descriptors ------------------------------------------- */
typedef struct covgpu_dur_par { int32_t code; int32_t _pad; double a; double b; } covgpu_dur_par;

/* quar_policy of test_prob (interventions.py:682-710): who counts as a
 * quarantined tester on day t */
#define COVGPU_QP_START 1    /* date_quarantined == t - 1   */
#define COVGPU_QP_END 2      /* date_end_quarantine == t + 1 */
#define COVGPU_QP_DAILY 4    /* quarantined                 */
#define COVGPU_QP_OFFSETS 8  /* date_quarantined == t - 1 - q for every bit q of quar_offsets */

/* One sim's test_prob (interventions.py:858-981) and contact_tracing
 * (interventions.py:984-1145). Days are inclusive ranges; an empty range
 * (start > end) switches the intervention off. Probabilities p are passed as
 * thresholds ceil(p * 2^53): a Philox uniform u = (2k + 1) / 2^53 satisfies
 * u < p exactly when 2k + 1 < threshold, which is float64's u < p. */
typedef struct covgpu_testing {
  int32_t test_start, test_end;
  int32_t quar_policy;            /* COVGPU_QP_* bits                                 */
  uint32_t quar_offsets;
  uint64_t thr_symp, thr_asymp, thr_symp_quar, thr_asymp_quar;
  uint64_t thr_sensitivity;       /* test_sensitivity                                 */
  uint64_t thr_not_lost;          /* 1 - loss_prob                                    */
  int32_t test_delay;
  int32_t trace_start, trace_end;
  int32_t presumptive;            /* trace the exposed tested today, not the diagnosed */
  double trace_time[COVGPU_MAX_LAYERS];        /* days from diagnosis to notification */
  uint64_t thr_trace[COVGPU_MAX_LAYERS];       /* per-layer trace_probs; 0: not traced */
  int32_t trace_start_off[COVGPU_MAX_LAYERS];  /* int(trace_time): quarantine start offset */
  int32_t trace_period[COVGPU_MAX_LAYERS];     /* int(quar_period - trace_time)        */
  /* test_prob's subtarget (interventions.py:150-187, 970-972): per local agent the
   * threshold of its fixed test probability, COVGPU_NO_SUBTARGET for none (NULL: no
   * subtarget); applied after the symptom and quarantine probabilities, before the
   * diagnosed are set to 0 */
  const uint64_t* sub_thr;
  /* test_prob's influenza-like illness (interventions.py:941-947): the agents of day
   * test_start + d are ili_inds[ili_off[d] .. ili_off[d + 1]) (local indices), for
   * d < ili_days; ili_mark [n_agents] is the last day an agent was marked (written by
   * the test pass's first kernel; NULL: no ILI). A marked agent without COVID
   * symptoms tests with the symptomatic probability. */
  const int64_t* ili_off;
  const int32_t* ili_inds;
  int32_t* ili_mark;
  int32_t ili_days;
  int32_t _pad_ili;
  /* test_prob's swab delay (interventions.py:930-938; NULL swab_pdf: none): swab_pdf
   * [swab_len] the delay distribution's density at 0, 1, ... days (computed on the
   * host); swab_bins [swab_len + 1] the day's symptomatic agents by whole days since
   * symptom onset, and their total (zeroed and filled on the device before the test
   * pass); symp_prob the float64 symptomatic probability */
  const double* swab_pdf;
  int32_t* swab_bins;
  double symp_prob;
  int32_t swab_len;
  int32_t _pad_swab;
  /* contact_tracing's capacity (interventions.py:1074-1078; NULL cap_list: none): of
   * the day's cases, int(capacity / scale) are traced, scale the sim's rescale_vec[t]
   * (cap_scale without dynamic rescaling): those with the smallest keys, the x word
   * of Philox (agent, 2, t, TAG_TEST) above the agent's index. cap_list [n_agents]
   * and *cap_count hold the day's cases (local indices; filled by the test pass). */
  double capacity;
  double cap_scale;
  int32_t* cap_list;
  uint32_t* cap_count;
} covgpu_testing;
#define COVGPU_NO_SUBTARGET 0xFFFFFFFFFFFFFFFFull

/* One sim's parameter block (device memory, one entry per sim). */
typedef struct covgpu_sim_params {
  int64_t agent_off;          /* first global agent index (multiple of 32)          */
  int32_t n_agents;
  int32_t n_variants;
  int32_t n_layers;
  int32_t npts;               /* days + 1                                           */
  uint32_t key0, key1;        /* Philox key (64-bit seed)                           */
  int32_t use_waning;
  int32_t nab_kin_len;
  int64_t n_beds_hosp;        /* -1: unconstrained                                  */
  int64_t n_beds_icu;
  float frac_time, load_ratio, high_cap, asymp_factor;
  float trans_redux, nab_boost, no_hosp_factor, no_icu_factor;
  float rel_symp[COVGPU_MAX_VARIANTS], rel_severe[COVGPU_MAX_VARIANTS];
  float rel_crit[COVGPU_MAX_VARIANTS], rel_death[COVGPU_MAX_VARIANTS];
  float immunity[COVGPU_MAX_VARIANTS * COVGPU_MAX_VARIANTS]; /* [variant][recovered_variant] */
  double rel_imm_asymp, rel_imm_mild, rel_imm_severe, nab_norm; /* nab_norm = 1 + alpha_inf_diff */
  /* calc_VE parameters (immunity.py:216-247) as float pairs (hi, lo): alpha and
   * beta of the sus, symp and sev axes, and ln of each immunity-matrix entry */
  float ve_alpha[3][2], ve_beta[3][2];
  float ln_immunity[COVGPU_MAX_VARIANTS * COVGPU_MAX_VARIANTS][2];
  covgpu_dur_par dur[COVGPU_N_DUR_PARS];
  covgpu_dur_par nab_init;
  const float* nab_kin;           /* [nab_kin_len][2] nab_kin as float pairs (hi, lo) */
  const float* beta_tab;          /* [npts][n_variants] float32 beta per day/variant */
  const float* beta_layer_tab;    /* [npts][n_layers]                                */
  const float* vx_imm;            /* [n_vaccines][n_variants] or NULL                */
  const float* vx_ln_imm;         /* [n_vaccines][n_variants][2] ln(vx_imm) pairs    */
  int32_t n_vaccines;
  int32_t _pad2;
  int64_t* res_int;               /* [npts][COVGPU_N_RES_INT]                        */
  int64_t* res_var;               /* [npts][COVGPU_N_RES_VAR][n_variants]            */
  int64_t* res_fx;                /* [npts][COVGPU_N_RES_F] fixed-point sums         */
  covgpu_testing testing;
  int32_t seg_of_layer[COVGPU_MAX_LAYERS]; /* layer -> segment index (-1: no edges)   */
  /* dynamic rescaling (sim.py:535-556; rescale_vec NULL: off). The day kernels
   * only detect the day it is due; the host performs it (covgpu_state.hold) */
  double pop_scale;
  double rescale_threshold;
  const double* rescale_vec;      /* [npts] current scale of each day               */
  int64_t* nonnaive;              /* [3] agents not naive, the last day whose flows
                                     are in that count, the last day checked        */
} covgpu_sim_params;

/* One contact layer of one sim (device memory, one entry per layer segment).
 *
 * A dynamic layer (base.py:1849-1876 Layer.update: every day all n_edges
 * edges redrawn with both endpoints uniform over the sim's agents) stores no
 * edges. Its day-t edges are drawn per agent: the edges of agent a as p1 and
 * as p2 are two lists, each of Binomial(n_edges, 1 / n_agents) entries with
 * uniform partners, keyed by (seed, a, day, layer). The edge pass draws the
 * lists of the day's sources only, the tracing pass those of the traced
 * agents (covgpu_layer_lists writes them out). dyn_cdf holds the count
 * distribution: dyn_cdf[k] = floor(2^64 * P(count <= k)) for k < dyn_k - 1
 * and dyn_cdf[dyn_k - 1] = 2^64 - 1, with dyn_k <= COVGPU_DYN_MAX_LIST. */
#define COVGPU_DYN_MAX_LIST 1024
typedef struct covgpu_layer {
  const int32_t* p1;              /* global agent indices, sorted ascending (static) */
  const int32_t* p2;
  const float* beta;              /* per-edge beta, or NULL: every edge has beta_const */
  int64_t n_edges;
  int64_t tile_begin;             /* first edge-pass tile of this segment (a dynamic
                                     layer has no tiles)                           */
  int32_t sim;
  int32_t layer;                  /* layer index within the sim (0..n_layers-1)      */
  int32_t dynamic;                /* 1: edges redrawn every day (p1/p2 unused)       */
  float beta_const;
  float iso_factor, quar_factor;
  int32_t dyn_k;                  /* dynamic: entries of dyn_cdf                    */
  /* agent index of a stored layer (NULL: none; covgpu_trace_index): the agent
   * a's edges as p1 are [rp1[a], rp1[a+1]), as p2 the edges perm2[rp2[a] ..
   * rp2[a+1]) (a local to the sim). With it the edge pass walks the layer from
   * the day's sources on days its sim has few infectious agents, and the
   * tracing pass visits only the traced agents' edges. */
  const uint32_t* rp1;
  const uint32_t* rp2;
  const uint32_t* perm2;
  const uint64_t* dyn_cdf;        /* dynamic: [dyn_k] count distribution (above)     */
  float dyn_rse_max;              /* dynamic: a bound on rel_sus * quarantine factor *
                                     (1 - sus_imm) over the sim's agents (the largest
                                     rel_sus, times quar_factor when above 1); the
                                     edge pass thins each source's entries by it     */
  int32_t _pad2;
} covgpu_layer;

/* One agent block of the agent kernel: agents [begin, end) of one sim. */
typedef struct covgpu_agent_block { int64_t begin; int64_t end; int32_t sim; int32_t _pad; } covgpu_agent_block;

/* One transmission event recorded by the edge pass. */
typedef struct covgpu_event { uint64_t key; int32_t target; int32_t source; } covgpu_event;

/* One infection-log record (people.py:508-511): local source (-1 for seed
 * infections and importations) and target, day, and layer | variant << 8 | sim << 16. */
typedef struct covgpu_log_rec { int32_t source; int32_t target; int32_t day; int32_t layer_variant; } covgpu_log_rec;

/* Transmission log-likelihood and expected infections of each day, with
 * their sensitivities (all device pointers; factor == NULL switches the
 * likelihood passes off). Every exposed direction source -> target of day t
 * (the candidates of the edge pass) has
 *   p = F[t][layer][variant] * edge beta * rel_trans' * rel_sus'
 * (float-float, ~2^-44 relative, capped at 1; GB300's float64 rate is a small
 * fraction of its float32 rate), with rel_trans' = rel_trans * quar/asymp/iso factors * viral
 * load and rel_sus' = rel_sus * quar factor * (1 - sus_imm) as in
 * compute_trans_sus (utils.py:82-90) but without beta_layer, which F holds
 * together with beta, rel_beta and the variant's rel_beta. Its outcome is
 * the edge pass's own Bernoulli draw. Per sim and day:
 *   ll       = sum over infecting directions of log p + over the others of log(1 - p)
 *   expected = sum over targets of 1 - prod over their directions of (1 - p)
 * and per layer the derivatives with respect to log F[t][layer][*]:
 *   g_ll     = sum of (infecting ? 1 : -p / (1 - p))
 *   g_exp    = sum over targets of prod(1 - p) * sum over the layer's directions of p / (1 - p). */
typedef struct covgpu_lik {
  const float* factor;            /* [n_sims][npts_max][n_layers_max][nv_max][2]:
                                     F as float pairs (hi, lo), hi + lo = F to 2^-48 */
  double* ll;                     /* [n_sims][npts_max]                             */
  double* expected;               /* [n_sims][npts_max]                             */
  double* g_ll;                   /* [n_sims][npts_max][n_layers_max] or NULL       */
  double* g_exp;                  /* [n_sims][npts_max][n_layers_max] or NULL       */
  double* logq;                   /* [n] zero between days (the agent pass of the
                                     likelihood clears what it reads)               */
  double* w;                      /* [n_layers_max][n], zero; needed with g_exp     */
  int32_t npts_max, n_layers_max, nv_max, _pad;
} covgpu_lik;

/* Everything the fused kernels touch. Host struct; the library copies it into
 * kernel parameters. All pointers are device pointers. */
typedef struct covgpu_state {
  int64_t n;                      /* global agents, including 32-alignment padding  */
  int32_t n_sims;
  int32_t n_segments;             /* layer segments over all sims                   */
  int64_t n_tiles;                /* edge-pass tiles over all segments              */
  int64_t n_agent_blocks;
  int32_t edge_tile;              /* edges per edge-pass tile: 1024, 2048, 4096 or
                                     8192 (segments' tile_begin count these tiles)   */
  int32_t edge_resident;          /* 1: one sim's source bitmap resident in shared
                                     memory (one block per SM; a single sim of at
                                     most ~1.1M agents, tiles of 4096 or 8192)     */
  int32_t edge_wave;              /* > 0: the stored layers' pass as one wave of
                                     blocks walking balanced ranges of tiles, at
                                     most this many blocks per SM; 0: one block per
                                     tile. Not with edge_resident.                 */
  int32_t _pad_wave;
  /* per-agent state */
  uint32_t* flags;
  uint32_t* vstate;               /* bytes: exposed, infectious, recovered variant   */
  float* symp_prob; float* severe_prob; float* crit_prob; float* death_prob;
  float* rel_trans; float* rel_sus;
  int32_t* n_infections; int32_t* n_breakthroughs;
  float* peak_nab; float* nab; int32_t* t_nab_event;
  int32_t* vaccine_source;
  float* sus_imm; float* symp_imm; float* sev_imm;   /* [n_variants_max][n]           */
  int32_t imm_stride_variants;    /* rows of the imm blocks (max variants over sims) */
  int32_t edge_parts;             /* what covgpu_edge_pass launches: 0 both passes, 1 the
                                     stored layers' tiles only, 2 the dynamic layers'
                                     sources only (covgpu_run_days runs both)        */
  float* dates;                   /* [COVGPU_N_DATES][n]                             */
  float* durs;                    /* [COVGPU_N_DURS][n]                              */
  /* per-day working buffers */
  float* viral_load;              /* [n]                                             */
  uint32_t* roles;                /* [2][ceil(n/32)]: source bitmap, target bitmap    */
  uint64_t* claim;                /* [n] first-infector claim (day-tagged)           */
  float* src_rec;                 /* [n][4] per source, written by the agent pass for
                                     the edge pass: rel_trans, viral load, vstate bits,
                                     flags bits (the post pass updates the last) */
  covgpu_event* events;           /* [event_capacity]                                */
  int64_t event_capacity;
  unsigned long long* event_count;/* device counter                                  */
  covgpu_log_rec* log;            /* [log_capacity] or NULL                          */
  int64_t log_capacity;
  unsigned long long* log_count;
  int32_t* status;                /* device status word (COVGPU_OVERFLOW ...)        */
  const int32_t* hospicu;         /* optional [2 * n_sims] forced hosp_max / icu_max;
                                     NULL: from the day's severe/critical counts     */
  /* descriptors */
  const covgpu_sim_params* sims;  /* [n_sims]                                        */
  const covgpu_layer* segments;   /* [n_segments]                                    */
  const covgpu_agent_block* agent_blocks; /* [n_agent_blocks]                        */
  /* test mode: per-agent injected draws [n][COVGPU_N_DRAWS] (NULL: Philox) and
   * injected edge uniforms (NULL: Philox), per segment a [n_variants][2][n_edges]
   * table indexed by (source variant, direction, edge) */
  const double* draw_table;
  const double* const* edge_uniforms; /* [n_segments] -> [n_variants][2][n_edges] */
  /* testing and tracing (all NULL / 0 when no sim tests) */
  int32_t has_testing;            /* bit 0: run the testing, tracing and post passes;
                                     bit 1: some sim's test_prob has a swab delay;
                                     bit 2: some sim's contact_tracing a capacity;
                                     bit 3: every stored layer has its agent index
                                     (the tracing scan of the tiles is skipped)      */
  int32_t pending_slots;          /* R: days of scheduled quarantines kept ahead     */
  uint32_t* trace_bits;           /* [ceil(n/32)] agents traced today                */
  uint32_t* contact_bits;         /* [n_contact_layers][ceil(n/32)] contacts found   */
  int32_t n_contact_layers;       /* max layers over sims                            */
  int32_t src_walk;               /* indexed stored layers on quiet days: k > 0 walks a
                                     layer from the day's sources while its sim's
                                     infectious agents x k < its agents; 0 never,
                                     -1 always (the streamed and walked passes give
                                     the same results)                             */
  int32_t* pending_quar;          /* [R][n] end day of a quarantine starting on day
                                     s (slot s mod R), -1: none                      */
  uint32_t* trace_count;          /* [n_sims] agents traced today                    */
  covgpu_lik lik;                 /* likelihood passes after each edge pass (factor
                                     NULL: off)                                      */
  /* daily importations (sim.py:582-587; all NULL / 0 when no sim imports): the
   * agents imported on day t are imports[import_day_off[t] .. import_day_off[t+1]),
   * global agent indices, with the sim of each in import_sims */
  const int64_t* import_day_off;  /* [import_days + 1]                               */
  const int32_t* imports;
  const int32_t* import_sims;
  int32_t import_days;            /* days covered; 0: no importations                */
  int32_t n_dynamic;              /* dynamic layer segments (the edge pass draws their
                                     edges from the day's sources' lists)           */
  /* the first day held back for a host step (a due rescaling, found by the
   * day's rescale check); 0x7FFFFFFF: none. Every day kernel of a held day
   * returns at once, the agent pass of the held day closes the day before it.
   * NULL: no sim rescales dynamically */
  int32_t* hold;
  float* tgt_rec;                 /* [imm_stride_variants][n] per edge-pass target,
                                     written by the agent pass: rel_sus * (1 - sus_imm[v])
                                     with the sign bit set when quarantined (the post
                                     pass updates the sign)                          */
} covgpu_state;

/* ---- standalone kernels: the reference's numba functions ----------------- */

/* compute_viral_load (utils.py:38-79). float32 arithmetic as numba types it. */
int covgpu_viral_load(int32_t t, const float* date_inf, const float* date_rec, const float* date_dead,
                      int64_t n, float frac_time, float load_ratio, float high_cap,
                      float* out_load, void* stream);

/* compute_trans_sus (utils.py:81-90). Booleans as one byte per agent. */
int covgpu_trans_sus(const float* rel_trans, const float* rel_sus, const uint8_t* inf, const uint8_t* sus,
                     float beta_layer, const float* viral_load, const uint8_t* symp, const uint8_t* iso,
                     const uint8_t* quar, float asymp_factor, float iso_factor, float quar_factor,
                     const float* immunity_factors, int64_t n, float* out_rel_trans, float* out_rel_sus,
                     void* stream);

/* compute_infections (utils.py:92-128, non-legacy). Output order is the
 * reference's: direction p1->p2 in edge order, then p2->p1 in edge order.
 * uniforms: [2][n_edges] float64 draws per (direction, edge), or NULL to
 * draw from Philox keyed (seed, day, variant, layer, edge). *out_count
 * (device) receives the number of transmissions; if it exceeds capacity only
 * the first capacity are written and COVGPU_OVERFLOW is stored in *status.
 * An edge whose p1 or p2 is outside [0, n_agents) is skipped and
 * COVGPU_BADARG is stored in *status (status may be NULL).
 * scratch: device memory of covgpu_infections_scratch_bytes(n_edges) bytes. */
int64_t covgpu_infections_scratch_bytes(int64_t n_edges);
int covgpu_infections(float beta, const int32_t* p1, const int32_t* p2, const float* layer_betas,
                      int64_t n_edges, const float* rel_trans, const float* rel_sus, int64_t n_agents,
                      const double* uniforms, uint64_t seed, int32_t day, int32_t variant, int32_t layer,
                      int32_t* out_src, int32_t* out_tgt, int64_t capacity, int64_t* out_count,
                      int32_t* status, void* scratch, int64_t scratch_bytes, void* stream);

/* compute_infections for callers that cannot allocate device memory. (No
 * counterpart in the reference, which has no device memory at all.) Some
 * callers must not call cudaMalloc or any allocating routine: a framework
 * capturing work into a CUDA graph under its own allocator, a plugin host
 * that hands out a fixed memory budget, or a latency-critical thread that
 * cannot afford the device synchronisation an allocation or free may cause.
 * This variant takes no scratch argument: its tile counts and offsets live in
 * a file-scope __device__ array of this library, sized for at most
 * COVGPU_NOALLOC_MAX_EDGES edges (196,608 bytes, held by every GPU that
 * loads the library until the process exits); larger n_edges is rejected
 * with COVGPU_BADARG before any launch. Arguments, outputs and statuses are
 * otherwise those of covgpu_infections, and it allocates nothing. The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress
 * with that device current); make that first call before any stream capture.
 * After a device reset (a new context) the next call looks the address up again.
 * Every call shares the one array and rewrites the part it reads, so calls
 * need no clearing between them, but calls whose kernels overlap on the GPU
 * (different streams, or concurrent host threads) race on it: serialise them. */
#define COVGPU_NOALLOC_MAX_EDGES (1LL << 24)
int covgpu_infections_noalloc(float beta, const int32_t* p1, const int32_t* p2, const float* layer_betas,
                              int64_t n_edges, const float* rel_trans, const float* rel_sus, int64_t n_agents,
                              const double* uniforms, uint64_t seed, int32_t day, int32_t variant, int32_t layer,
                              int32_t* out_src, int32_t* out_tgt, int64_t capacity, int64_t* out_count,
                              int32_t* status, void* stream);

/* ---- synthetic populations on the device --------------------------------
 * The distributions of covasim/population.py and people.py:139-161, each
 * agent / member / cluster one thread, variable-length outputs placed by
 * exclusive scans, draws from Philox keyed by (seed, purpose, layer, index).
 * Every scan needs `scratch` of covgpu_pop_scan_scratch(n) int64 elements and
 * writes n + 1 offsets (offsets[n] = total). Rejection samplers are bounded:
 * an exhausted one stores COVGPU_TIMEOUT in *status. */
int64_t covgpu_pop_scan_scratch(int64_t n);

/* Ages and sexes (population.py:196-210): a bin by weight (bin_cdf: cumulative
 * weights), then uniform in [bin_lo, bin_lo + bin_width); sex Bernoulli(0.5)
 * (sex may be NULL). */
int covgpu_pop_ages(int64_t n, const double* bin_lo, const double* bin_width, const double* bin_cdf, int32_t n_bins,
                    uint64_t seed, float* age, int32_t* sex, void* stream);

/* Agents with age_lo <= age < age_hi, ascending (population.py:353-354):
 * flags [n], pos [n + 1] (pos[n] = number of members), members [n]. */
int covgpu_pop_members(int64_t n, const float* age, float age_lo, float age_hi, int64_t* flags, int64_t* pos,
                       int64_t* scratch, int32_t* members, void* stream);

/* A random layer (population.py:241-284): partners per member
 * round(X / 2) half to even, X ~ Poisson(mean) (dispersion <= 0) or negative
 * binomial(mean, dispersion); counts [n_members], offsets [n_members + 1]. */
int covgpu_pop_random_counts(int64_t n_members, double mean, double dispersion, uint64_t seed, int32_t layer,
                             int64_t* counts, int64_t* offsets, int64_t* scratch, int32_t* status, void* stream);
/* ... then the edges: p1 = the member (ascending), p2 uniform over the members
 * (members NULL: agents 0..n_members-1). */
int covgpu_pop_random_fill(int64_t n_members, const int32_t* members, const int64_t* offsets, uint64_t seed,
                           int32_t layer, int32_t* p1, int32_t* p2, void* stream);

/* Household clusters (population.py:287-329): n_clusters Poisson(mean) sizes
 * and their starts [n_clusters + 1]; the caller checks starts[n_clusters] >= n
 * (else draws more clusters). */
int covgpu_pop_cluster_sizes(int64_t n_clusters, double mean, uint64_t seed, int32_t layer, int64_t* sizes,
                             int64_t* starts, int64_t* scratch, int32_t* status, void* stream);
/* pairs (i, j > i) per agent within its cluster (clusters cut at n): counts
 * [n], offsets [n + 1]; then the edges. */
int covgpu_pop_cluster_counts(int64_t n, int64_t n_clusters, const int64_t* starts, int64_t* counts,
                              int64_t* offsets, int64_t* scratch, void* stream);
int covgpu_pop_cluster_fill(int64_t n, const int64_t* offsets, int32_t* p1, int32_t* p2, void* stream);

/* set_prognoses (people.py:139-161): the age bin (np.digitize over cutoffs)
 * selects symp, severe (x comorbidity), crit, death probabilities and rel_sus
 * from tables [6][n_bins] (float64: those five then trans_ORs); rel_trans =
 * trans_OR * draw, draw negative binomial (trans_dist 0: mean par1,
 * dispersion par2, in units of step) or lognormal (1: mean par1, sd par2). */
int covgpu_pop_prognoses(int64_t n, const float* age, const double* cutoffs, int32_t n_bins, const double* tables,
                         int32_t trans_dist, double par1, double par2, double step, uint64_t seed, float* symp,
                         float* severe, float* crit, float* death, float* rel_sus, float* rel_trans, int32_t* status,
                         void* stream);

/* ---- fused per-day kernels over a batch of sims ------------------------- */

/* One dense pass over every agent of every sim. With do_prev, first closes
 * day t-1 (stock counts, update_nab, NAb sum); with do_day, then runs day t's
 * update_states_pre (all checks, in the reference's order), check_immunity,
 * the flow counts, the viral load of the infectious and the source/target
 * role bitmaps the edge pass reads. Also resets the day's event counter.
 * do_day | COVGPU_DAY_STEADY: the caller has run a full pass (do_day) of this
 * state since anything but this library's day kernels last changed it, so the
 * pass may skip the warps whose agents are all susceptible and naive and
 * nothing else (their records and role bits are current; covgpu_run_days
 * does this on every day of a launch sequence but the first). */
#define COVGPU_DAY_STEADY 2
int covgpu_agent_step(const covgpu_state* st, int32_t t, int32_t do_prev, int32_t do_day, void* stream);

/* Transmission over every layer segment and variant: both directions of each
 * stored edge from one read, the dynamic layers' edges from the day's
 * sources' lists, Bernoulli draws from Philox (or, for stored layers,
 * st->edge_uniforms),
 * events appended to st->events and the first infector of each target
 * claimed with a 64-bit atomicMin on (day, variant, layer, direction, edge).
 * With st->lik.factor set, also the likelihood terms of every candidate
 * direction (covgpu_lik). */
int covgpu_edge_pass(const covgpu_state* st, int32_t t, void* stream);

/* Shared memory the resident-bitmap edge pass needs for this state (one sim;
 * 0: it cannot run here). Set st->edge_resident only when this is nonzero. */
int64_t covgpu_edge_resident_bytes(const covgpu_state* st);

/* The testing and tracing interventions of day t, after the agent pass and
 * any importations, before transmission (sim.py:596-600): test_prob's
 * Bernoulli draws and People.test (interventions.py:921-981,
 * people.py:589-617), contact_tracing's case selection, find_contacts over
 * every layer, binomial_filter and notify (interventions.py:1044-1145,
 * utils.py:131-147), then update_states_post: check_diagnosed, check_quar
 * with the scheduled quarantines, check_enter_iso (people.py:189-196,
 * 315-366). A no-op when st->has_testing is 0. */
int covgpu_test_trace(const covgpu_state* st, int32_t t, void* stream);

/* The per-target half of day t's likelihood (see covgpu_lik): expected
 * infections and their sensitivities from the per-target sums that
 * covgpu_edge_pass accumulates when st->lik.factor is set (it then adds the
 * likelihood terms of every candidate direction to its usual work). Call
 * after covgpu_edge_pass and before covgpu_infect_claims of the same day.
 * BADARG when st->lik.factor is NULL. */
int covgpu_lik_targets(const covgpu_state* st, int32_t t, void* stream);

/* The agent index of one stored layer segment (p1 ascending, global agent
 * indices from agent_off, n_local agents): rp1 and rp2 [n_local + 1], perm2
 * [n_edges], scratch covgpu_trace_index_scratch(n_local) int64 elements. With
 * it, covgpu_edge_pass can walk the layer from the day's sources on quiet days
 * (covgpu_state.src_walk; the same candidates and draws as the streamed pass),
 * and covgpu_test_trace visits only the traced agents' edges of that layer
 * instead of scanning the layer. */
int64_t covgpu_trace_index_scratch(int64_t n_local);
int covgpu_trace_index(const int32_t* p1, const int32_t* p2, int64_t n_edges, int64_t agent_off, int64_t n_local,
                       uint32_t* rp1, uint32_t* rp2, uint32_t* perm2, int64_t* scratch, void* stream);

/* infect() for the winning event of each target. */
int covgpu_infect_claims(const covgpu_state* st, int32_t t, void* stream);

/* infect() for an explicit list of global agent indices (unique), as
 * People.infect(inds, source=..., layer=..., variant=...) does: only the
 * susceptible are infected. sources (or NULL: none) holds each target's
 * source as a local index, recorded in the infection log (people.py:508-511)
 * with layer_tag (>= COVGPU_MAX_LAYERS for non-layer sources); infected (or
 * NULL) receives 1 for each agent actually infected, 0 for the others.
 * call_tag selects the Philox stream (1: seed infections, 2+: importations).
 * Seed infections (call_tag 1) are not counted in the day's flows: the
 * reference seeds before update_states_pre resets them (sim.py:571-577). */
int covgpu_infect_list(const covgpu_state* st, int32_t t, const int32_t* inds, const int32_t* sources, int64_t n_inds,
                       int32_t sim, int32_t variant, int32_t layer_tag, int32_t call_tag, uint8_t* infected,
                       void* stream);

/* The day's importations (sim.py:582-587): infect() with the wild type for the
 * agents st->imports lists for day t (all sims; infection log layer
 * COVGPU_MAX_LAYERS + 1, Philox stream call_tag 2). covgpu_run_days runs it
 * after each day's agent pass; a day beyond st->import_days imports nobody.
 * Entries outside their sim's agents are skipped and set COVGPU_BADARG in the
 * device status word. */
int covgpu_import_day(const covgpu_state* st, int32_t t, void* stream);

/* The rescale check of day t (sim.py:535-547), run before the day's agent pass
 * by covgpu_run_days when st->hold is set: for each sim with rescale_vec, the
 * day's count of agents not naive (nonnaive[0] plus the first infections of
 * the days since nonnaive[1]) and, unless day t was already checked
 * (nonnaive[2] >= t), whether rescale_vec[t] < pop_scale and that count /
 * n_agents > rescale_threshold; if so *st->hold = t (the earliest such day). */
int covgpu_rescale_check(const covgpu_state* st, int32_t t, void* stream);

/* The day-t contact lists of agents [agent_begin, agent_begin + n_agents)
 * (local to the segment's sim) in one dynamic layer segment: the draws the
 * edge pass makes for a source and the tracing pass for a traced agent. With
 * offsets NULL, counts[2 i + d] receives the length of list d (0: the agent
 * as p1, 1: as p2) of agent agent_begin + i; with offsets (the exclusive sum
 * of those counts, 2 n_agents + 1 entries), partners[offsets[2 i + d] + j]
 * receives partner j of that list (local index) and counts is unused. */
int covgpu_layer_lists(const covgpu_state* st, int32_t segment, int32_t t, int64_t agent_begin, int64_t n_agents,
                       int32_t* counts, const int64_t* offsets, int32_t* partners, void* stream);

/* Run days [t0, t1) of every sim: per day agent_step, test_trace (when
 * st->has_testing), edge_pass, lik_targets (when st->lik.factor is set),
 * infect_claims. open_prev: day t0-1 still needs its closing pass (stocks,
 * update_nab), which day t0's agent pass then does first; close_last: end
 * with the closing pass of day t1-1. With use_graph a sequence run again
 * with the same state and arguments is captured into a CUDA graph on its
 * second run and replayed from then on; its first run launches the kernels
 * directly (a run made once does not pay for the capture). */
int covgpu_run_days(const covgpu_state* st, int32_t t0, int32_t t1, int32_t open_prev, int32_t close_last,
                    int32_t use_graph, void* stream);

/* ---- the day path one function at a time --------------------------------
 * For callers that keep the reference's call sequence (update_states_pre's
 * checks one by one, check_immunity, update_nab, update_peak_nab) instead of
 * the fused kernels. Agents are local indices of sim `sim`; each function
 * writes the same state as the fused passes, with the same arithmetic. */

/* which People.check_* covgpu_check runs */
enum { COVGPU_CHECK_INFECTIOUS = 0, COVGPU_CHECK_SYMPTOMATIC, COVGPU_CHECK_SEVERE, COVGPU_CHECK_CRITICAL,
       COVGPU_CHECK_RECOVERY, COVGPU_CHECK_DEATH, COVGPU_CHECK_EXIT_ISO };

/* covasim/people.py:222-312, 368-374 People.check_infectious, check_symptomatic,
 * check_severe, check_critical, check_recovery, check_death, check_exit_iso at
 * day t over the sim's n_agents agents: applies the transition and writes the
 * local indices of the agents it changed to out (in no particular order; at
 * most capacity, else COVGPU_OVERFLOW in the device status word). counts
 * (device, 2 entries, zeroed first): the agents changed, and for check_death
 * those of them diagnosed (the known deaths). filter_exposed: only exposed
 * agents (the reference's is_exp, its snapshot of the exposed flag at the start
 * of update_states_pre, which equals the current flag for every check run in
 * update_states_pre's order); check_exit_iso takes no filter. inds (recovery
 * only, else NULL): recover exactly these n_inds agents, as check_recovery's
 * inds argument does. Indices outside the sim set COVGPU_BADARG in the device
 * status word and are skipped. */
int covgpu_check(const covgpu_state* st, int32_t t, int32_t which, int32_t sim, int32_t filter_exposed,
                 const int32_t* inds, int64_t n_inds, int64_t n_agents, int32_t* out, int64_t capacity,
                 int64_t* counts, void* stream);

/* covasim/immunity.py:303-350 check_immunity(people, variants): sus_imm,
 * symp_imm and sev_imm of every agent of the sim for the variants whose bit is
 * set in variant_mask, at day t. */
int covgpu_check_immunity(const covgpu_state* st, int32_t t, int32_t sim, uint32_t variant_mask, void* stream);

/* covasim/immunity.py:205-213 update_nab(people, inds) at day t: nab += nab_kin[t
 * - t_nab_event] * peak_nab, clamped to [0, peak_nab]. */
int covgpu_update_nab(const covgpu_state* st, int32_t t, int32_t sim, const int32_t* inds, int64_t n_inds,
                      void* stream);

/* covasim/immunity.py:138-202 update_peak_nab(people, inds, nab_pars, symp) at day
 * t: agents with NAbs have peak_nab *= nab_boost; the others get 2^x with x ~
 * nab_init (one standard normal per agent from the Philox stream (seed, agent,
 * day, call_tag), block 3, which infect()'s draws leave unused), times
 * rel_imm_symp of symp_class[i] (0 asymptomatic, 1 mild, 2 severe) and
 * norm_factor when symp_class is given (natural infection), unscaled when it is
 * NULL (vaccination); t_nab_event = t for all. */
int covgpu_update_peak_nab(const covgpu_state* st, int32_t t, int32_t sim, const int32_t* inds, int64_t n_inds,
                           const int8_t* symp_class, covgpu_dur_par nab_init, float nab_boost, double norm_factor,
                           int32_t call_tag, void* stream);

/* Library/ABI version. */
int covgpu_version(void);

/* ABI layout check (no device work): writes up to n values: sizeof of
 * covgpu_sim_params, covgpu_layer, covgpu_agent_block, covgpu_event,
 * covgpu_log_rec, covgpu_state, then the offsets of covgpu_state.sims,
 * covgpu_state.edge_uniforms and covgpu_sim_params.res_fx. Returns the number
 * of values available. */
int covgpu_abi_layout(int64_t* out, int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* COVGPU_H */
