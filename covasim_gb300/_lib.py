"""Loader and ctypes mirror of the covgpu C ABI (include/covgpu.h).

The shared library is required: there is no CPU fallback. Importing this
module does not need a GPU; calling a kernel does.
"""
import ctypes as C
import os

from . import build as _build

MAX_VARIANTS = 8
MAX_LAYERS = 16
# infection-log layer tags beyond the contact layers (people.py:508-511 records the
# infect() call's ``layer``): seed infections, importations, layer=None, then any
# other label passed to People.infect (registered per batch)
LOG_SEED, LOG_IMPORT, LOG_NONE, LOG_EXTRA = MAX_LAYERS, MAX_LAYERS + 1, MAX_LAYERS + 2, MAX_LAYERS + 3
N_DATES = 19
N_DURS = 5
N_DRAWS = 10
N_RES_INT = 30
RES_SEVERE_NOW = 28
RES_CRITICAL_NOW = 29
N_RES_VAR = 6
N_RES_F = 3
FX_NAB_BITS = 24
FX_IMM_BITS = 32
NO_VARIANT = 0xFF
NOALLOC_MAX_EDGES = 1 << 24   # covgpu_infections_noalloc limit (COVGPU_NOALLOC_MAX_EDGES)
NO_SUBTARGET = 0xFFFFFFFFFFFFFFFF  # covgpu_testing.sub_thr: no subtarget (COVGPU_NO_SUBTARGET)
EDGE_TILE = '2048w'       # default edge pass: 2048-edge tiles, the stored layers' pass as one wave of blocks
DYN_MAX_LIST = 1024       # longest contact list of an agent in a dynamic layer (COVGPU_DYN_MAX_LIST)
EDGE_TILES = (1024, 2048, 4096, 8192)   # tile sizes the library supports (covgpu_state.edge_tile)
DAY_STEADY = 2  # COVGPU_DAY_STEADY, a flag of covgpu_agent_step's do_day
EDGE_WAVE_MAX = 32  # covgpu_state.edge_wave for 'as many blocks per SM as fit' (the kernel's occupancy caps it)
AGENT_BLOCK = 256         # agents per agent-pass block (covgpu.cu AGENT_THREADS)
AGENT_ALIGN = 32          # each sim's first agent is a multiple of this

OK, OVERFLOW, TIMEOUT, BADARG, CUDA_ERROR = 0, 1, 2, 3, 4
# covgpu_check: which People.check_* runs (COVGPU_CHECK_*)
CHECK_INFECTIOUS, CHECK_SYMPTOMATIC, CHECK_SEVERE, CHECK_CRITICAL, CHECK_RECOVERY, CHECK_DEATH, CHECK_EXIT_ISO = range(7)
STATUS_NAMES = {OK: 'OK', OVERFLOW: 'OVERFLOW', TIMEOUT: 'TIMEOUT', BADARG: 'BADARG', CUDA_ERROR: 'CUDA_ERROR'}

DIST_CODES = {'lognormal_int': 0, 'lognorm_int': 0, 'lognormal': 1, 'lognorm': 1, 'normal': 2, 'norm': 2,
              'normal_int': 3, 'normal_pos': 4}
DIST_ZERO = 5
DUR_ORDER = ['exp2inf', 'inf2sym', 'sym2sev', 'sev2crit', 'asym2rec', 'mild2rec', 'sev2rec', 'crit2rec', 'crit2die']


class CovgpuError(RuntimeError):
    """A covgpu entry point returned a non-OK status."""

    def __init__(self, fn, rc):
        super().__init__(f'{fn} failed with status {STATUS_NAMES.get(rc, rc)}')
        self.rc = rc


class DurPar(C.Structure):
    _fields_ = [('code', C.c_int32), ('_pad', C.c_int32), ('a', C.c_double), ('b', C.c_double)]


QP_START, QP_END, QP_DAILY, QP_OFFSETS = 1, 2, 4, 8   # COVGPU_QP_* quarantine testing policies


class Testing(C.Structure):
    _fields_ = [
        ('test_start', C.c_int32), ('test_end', C.c_int32), ('quar_policy', C.c_int32), ('quar_offsets', C.c_uint32),
        ('thr_symp', C.c_uint64), ('thr_asymp', C.c_uint64), ('thr_symp_quar', C.c_uint64),
        ('thr_asymp_quar', C.c_uint64), ('thr_sensitivity', C.c_uint64), ('thr_not_lost', C.c_uint64),
        ('test_delay', C.c_int32), ('trace_start', C.c_int32), ('trace_end', C.c_int32), ('presumptive', C.c_int32),
        ('trace_time', C.c_double * MAX_LAYERS), ('thr_trace', C.c_uint64 * MAX_LAYERS),
        ('trace_start_off', C.c_int32 * MAX_LAYERS), ('trace_period', C.c_int32 * MAX_LAYERS),
        ('sub_thr', C.c_void_p), ('ili_off', C.c_void_p), ('ili_inds', C.c_void_p), ('ili_mark', C.c_void_p),
        ('ili_days', C.c_int32), ('_pad_ili', C.c_int32),
        ('swab_pdf', C.c_void_p), ('swab_bins', C.c_void_p), ('symp_prob', C.c_double), ('swab_len', C.c_int32),
        ('_pad_swab', C.c_int32),
        ('capacity', C.c_double), ('cap_scale', C.c_double), ('cap_list', C.c_void_p), ('cap_count', C.c_void_p),
    ]


class SimParams(C.Structure):
    _fields_ = [
        ('agent_off', C.c_int64), ('n_agents', C.c_int32), ('n_variants', C.c_int32),
        ('n_layers', C.c_int32), ('npts', C.c_int32), ('key0', C.c_uint32), ('key1', C.c_uint32),
        ('use_waning', C.c_int32), ('nab_kin_len', C.c_int32),
        ('n_beds_hosp', C.c_int64), ('n_beds_icu', C.c_int64),
        ('frac_time', C.c_float), ('load_ratio', C.c_float), ('high_cap', C.c_float), ('asymp_factor', C.c_float),
        ('trans_redux', C.c_float), ('nab_boost', C.c_float), ('no_hosp_factor', C.c_float),
        ('no_icu_factor', C.c_float),
        ('rel_symp', C.c_float * MAX_VARIANTS), ('rel_severe', C.c_float * MAX_VARIANTS),
        ('rel_crit', C.c_float * MAX_VARIANTS), ('rel_death', C.c_float * MAX_VARIANTS),
        ('immunity', C.c_float * (MAX_VARIANTS * MAX_VARIANTS)),
        ('rel_imm_asymp', C.c_double), ('rel_imm_mild', C.c_double), ('rel_imm_severe', C.c_double),
        ('nab_norm', C.c_double),
        ('ve_alpha', (C.c_float * 2) * 3), ('ve_beta', (C.c_float * 2) * 3),
        ('ln_immunity', (C.c_float * 2) * (MAX_VARIANTS * MAX_VARIANTS)),
        ('dur', DurPar * len(DUR_ORDER)), ('nab_init', DurPar),
        ('nab_kin', C.c_void_p), ('beta_tab', C.c_void_p), ('beta_layer_tab', C.c_void_p), ('vx_imm', C.c_void_p),
        ('vx_ln_imm', C.c_void_p),
        ('n_vaccines', C.c_int32), ('_pad2', C.c_int32),
        ('res_int', C.c_void_p), ('res_var', C.c_void_p), ('res_fx', C.c_void_p),
        ('testing', Testing), ('seg_of_layer', C.c_int32 * MAX_LAYERS),
        ('pop_scale', C.c_double), ('rescale_threshold', C.c_double), ('rescale_vec', C.c_void_p),
        ('nonnaive', C.c_void_p),
    ]


class Layer(C.Structure):
    _fields_ = [('p1', C.c_void_p), ('p2', C.c_void_p), ('beta', C.c_void_p), ('n_edges', C.c_int64),
                ('tile_begin', C.c_int64), ('sim', C.c_int32), ('layer', C.c_int32), ('dynamic', C.c_int32),
                ('beta_const', C.c_float), ('iso_factor', C.c_float), ('quar_factor', C.c_float),
                ('dyn_k', C.c_int32), ('rp1', C.c_void_p), ('rp2', C.c_void_p), ('perm2', C.c_void_p),
                ('dyn_cdf', C.c_void_p), ('dyn_rse_max', C.c_float), ('_pad2', C.c_int32)]


class AgentBlock(C.Structure):
    _fields_ = [('begin', C.c_int64), ('end', C.c_int64), ('sim', C.c_int32), ('_pad', C.c_int32)]


class Lik(C.Structure):
    _fields_ = [('factor', C.c_void_p), ('ll', C.c_void_p), ('expected', C.c_void_p), ('g_ll', C.c_void_p),
                ('g_exp', C.c_void_p), ('logq', C.c_void_p), ('w', C.c_void_p), ('npts_max', C.c_int32),
                ('n_layers_max', C.c_int32), ('nv_max', C.c_int32), ('_pad', C.c_int32)]


class State(C.Structure):
    _fields_ = [
        ('n', C.c_int64), ('n_sims', C.c_int32), ('n_segments', C.c_int32), ('n_tiles', C.c_int64),
        ('n_agent_blocks', C.c_int64), ('edge_tile', C.c_int32), ('edge_resident', C.c_int32),
        ('edge_wave', C.c_int32), ('_pad_wave', C.c_int32),
        ('flags', C.c_void_p), ('vstate', C.c_void_p),
        ('symp_prob', C.c_void_p), ('severe_prob', C.c_void_p), ('crit_prob', C.c_void_p), ('death_prob', C.c_void_p),
        ('rel_trans', C.c_void_p), ('rel_sus', C.c_void_p),
        ('n_infections', C.c_void_p), ('n_breakthroughs', C.c_void_p),
        ('peak_nab', C.c_void_p), ('nab', C.c_void_p), ('t_nab_event', C.c_void_p),
        ('vaccine_source', C.c_void_p),
        ('sus_imm', C.c_void_p), ('symp_imm', C.c_void_p), ('sev_imm', C.c_void_p),
        ('imm_stride_variants', C.c_int32), ('edge_parts', C.c_int32),
        ('dates', C.c_void_p), ('durs', C.c_void_p),
        ('viral_load', C.c_void_p), ('roles', C.c_void_p), ('claim', C.c_void_p),
        ('src_rec', C.c_void_p),
        ('events', C.c_void_p), ('event_capacity', C.c_int64), ('event_count', C.c_void_p),
        ('log', C.c_void_p), ('log_capacity', C.c_int64), ('log_count', C.c_void_p),
        ('status', C.c_void_p), ('hospicu', C.c_void_p),
        ('sims', C.c_void_p), ('segments', C.c_void_p), ('agent_blocks', C.c_void_p),
        ('draw_table', C.c_void_p), ('edge_uniforms', C.c_void_p),
        ('has_testing', C.c_int32), ('pending_slots', C.c_int32), ('trace_bits', C.c_void_p),
        ('contact_bits', C.c_void_p), ('n_contact_layers', C.c_int32), ('src_walk', C.c_int32),
        ('pending_quar', C.c_void_p), ('trace_count', C.c_void_p),
        ('lik', Lik),
        ('import_day_off', C.c_void_p), ('imports', C.c_void_p), ('import_sims', C.c_void_p),
        ('import_days', C.c_int32), ('n_dynamic', C.c_int32),
        ('hold', C.c_void_p), ('tgt_rec', C.c_void_p),
    ]


_lib = None


def lib():
    """The loaded covgpu library (built in-tree on first use if missing)."""
    global _lib
    if _lib is None:
        path = _build.LIB_PATH
        if not os.path.exists(path):
            _build.build()
        L = C.CDLL(path)
        vp, i32, i64, f32, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_uint64
        sp = C.POINTER(State)
        L.covgpu_version.restype = C.c_int
        L.covgpu_abi_layout.argtypes = [C.POINTER(C.c_int64), i32]
        L.covgpu_abi_layout.restype = C.c_int
        L.covgpu_viral_load.argtypes = [i32, vp, vp, vp, i64, f32, f32, f32, vp, vp]
        L.covgpu_trans_sus.argtypes = [vp, vp, vp, vp, f32, vp, vp, vp, vp, f32, f32, f32, vp, i64, vp, vp, vp]
        L.covgpu_infections_scratch_bytes.argtypes = [i64]
        L.covgpu_infections_scratch_bytes.restype = i64
        L.covgpu_infections.argtypes = [f32, vp, vp, vp, i64, vp, vp, i64, vp, u64, i32, i32, i32, vp, vp, i64, vp,
                                        vp, vp, i64, vp]
        L.covgpu_infections_noalloc.argtypes = [f32, vp, vp, vp, i64, vp, vp, i64, vp, u64, i32, i32, i32, vp, vp,
                                                i64, vp, vp, vp]
        L.covgpu_infections_noalloc.restype = C.c_int
        L.covgpu_agent_step.argtypes = [sp, i32, i32, i32, vp]
        L.covgpu_edge_pass.argtypes = [sp, i32, vp]
        L.covgpu_infect_claims.argtypes = [sp, i32, vp]
        L.covgpu_test_trace.argtypes = [sp, i32, vp]
        L.covgpu_lik_targets.argtypes = [sp, i32, vp]
        L.covgpu_infect_list.argtypes = [sp, i32, vp, vp, i64, i32, i32, i32, i32, vp, vp]
        L.covgpu_check.argtypes = [sp, i32, i32, i32, i32, vp, i64, i64, vp, i64, vp, vp]
        L.covgpu_check_immunity.argtypes = [sp, i32, i32, C.c_uint32, vp]
        L.covgpu_update_nab.argtypes = [sp, i32, i32, vp, i64, vp]
        L.covgpu_update_peak_nab.argtypes = [sp, i32, i32, vp, i64, vp, DurPar, f32, C.c_double, i32, vp]
        L.covgpu_import_day.argtypes = [sp, i32, vp]
        L.covgpu_rescale_check.argtypes = [sp, i32, vp]
        L.covgpu_layer_lists.argtypes = [sp, i32, i32, i64, i64, vp, vp, vp, vp]
        L.covgpu_run_days.argtypes = [sp, i32, i32, i32, i32, i32, vp]
        L.covgpu_edge_resident_bytes.argtypes = [sp]
        L.covgpu_edge_resident_bytes.restype = i64
        L.covgpu_trace_index_scratch.argtypes = [i64]
        L.covgpu_trace_index_scratch.restype = i64
        L.covgpu_trace_index.argtypes = [vp, vp, i64, i64, i64, vp, vp, vp, vp, vp]
        L.covgpu_trace_index.restype = C.c_int
        L.covgpu_pop_scan_scratch.argtypes = [i64]
        L.covgpu_pop_scan_scratch.restype = i64
        f64 = C.c_double
        L.covgpu_pop_ages.argtypes = [i64, vp, vp, vp, i32, u64, vp, vp, vp]
        L.covgpu_pop_members.argtypes = [i64, vp, f32, f32, vp, vp, vp, vp, vp]
        L.covgpu_pop_random_counts.argtypes = [i64, f64, f64, u64, i32, vp, vp, vp, vp, vp]
        L.covgpu_pop_random_fill.argtypes = [i64, vp, vp, u64, i32, vp, vp, vp]
        L.covgpu_pop_cluster_sizes.argtypes = [i64, f64, u64, i32, vp, vp, vp, vp, vp]
        L.covgpu_pop_cluster_counts.argtypes = [i64, i64, vp, vp, vp, vp, vp]
        L.covgpu_pop_cluster_fill.argtypes = [i64, vp, vp, vp, vp]
        L.covgpu_pop_prognoses.argtypes = [i64, vp, vp, i32, vp, i32, f64, f64, f64, u64, vp, vp, vp, vp, vp, vp, vp,
                                           vp]
        for name in POP_FUNCS:
            getattr(L, name).restype = C.c_int
        for name in ('covgpu_viral_load', 'covgpu_trans_sus', 'covgpu_infections', 'covgpu_agent_step',
                     'covgpu_edge_pass', 'covgpu_infect_claims', 'covgpu_infect_list', 'covgpu_layer_lists',
                     'covgpu_run_days', 'covgpu_test_trace', 'covgpu_lik_targets', 'covgpu_import_day',
                     'covgpu_rescale_check', 'covgpu_check', 'covgpu_check_immunity', 'covgpu_update_nab',
                     'covgpu_update_peak_nab'):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def check(fn, rc):
    if rc != OK:
        raise CovgpuError(fn, rc)


def call(name, *args):
    rc = getattr(lib(), name)(*args)
    check(name, rc)
    return rc


def abi_layout():
    """(library values, ctypes values) of the ABI layout check."""
    out = (C.c_int64 * 32)()
    m = lib().covgpu_abi_layout(out, 32)
    mine = [C.sizeof(SimParams), C.sizeof(Layer), C.sizeof(AgentBlock), 16, 16, C.sizeof(State),
            State.sims.offset, State.edge_uniforms.offset, SimParams.res_fx.offset, C.sizeof(Testing),
            SimParams.testing.offset, State.pending_quar.offset, State.trace_count.offset, C.sizeof(Lik),
            State.lik.offset, State.import_day_off.offset, SimParams.pop_scale.offset, State.hold.offset]
    return list(out[:m]), mine


POP_FUNCS = ['covgpu_pop_ages', 'covgpu_pop_members', 'covgpu_pop_random_counts', 'covgpu_pop_random_fill',
             'covgpu_pop_cluster_sizes', 'covgpu_pop_cluster_counts', 'covgpu_pop_cluster_fill', 'covgpu_pop_prognoses']

EXPORTED = ['covgpu_version', 'covgpu_abi_layout', 'covgpu_viral_load', 'covgpu_trans_sus', 'covgpu_infections_scratch_bytes',
            'covgpu_infections', 'covgpu_infections_noalloc', 'covgpu_agent_step', 'covgpu_edge_pass', 'covgpu_infect_claims',
            'covgpu_infect_list', 'covgpu_import_day', 'covgpu_rescale_check', 'covgpu_layer_lists', 'covgpu_run_days', 'covgpu_test_trace',
            'covgpu_lik_targets', 'covgpu_trace_index_scratch', 'covgpu_trace_index', 'covgpu_edge_resident_bytes',
            'covgpu_check', 'covgpu_check_immunity', 'covgpu_update_nab', 'covgpu_update_peak_nab',
            'covgpu_pop_scan_scratch'] + POP_FUNCS
