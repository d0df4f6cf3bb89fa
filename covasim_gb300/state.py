"""Device-resident agent state for a batch of sims, and the fused-kernel calls.

Layout in HBM (``n`` = total agents, each sim starting at a multiple of 32):

* ``flags``   uint32[n]   the 16 boolean states (bit i = defaults.STATES[i]),
                          exposed_by_variant in bits 16-23, infectious_by_variant in 24-31
* ``vstate``  uint32[n]   exposed / infectious / recovered variant, one byte each (0xFF = NaN)
* per-person float32[n]: symp/severe/crit/death prob, rel_trans, rel_sus, peak_nab, nab
* int32[n]: n_infections, n_breakthroughs, t_nab_event, vaccine_source
* ``sus_imm``/``symp_imm``/``sev_imm`` float32[nv_max, n]
* ``dates`` float32[19, n], ``durs`` float32[5, n] (NaN = undefined)
* per-day working buffers: viral_load float32[n], roles uint32[2, n/32] (source
  bitmap, then target bitmap), claim uint64[n], event list, infection log
* contact layers: one (p1, p2[, beta]) segment per (sim, layer), int32 global agent
  indices sorted by p1; dynamic layers store no edges (redrawn from Philox each day)

A single simulation is a batch of one; ``covasim_gb300.Sim`` and
``covasim_gb300.BatchSim`` both drive this class.
"""
import ctypes as C
from decimal import Decimal, getcontext

import numpy as np
import torch

from . import _lib as L
from . import defaults as cvd
from . import torch_ops  # noqa: F401  (registers torch.ops.covgpu.*)

F32, I32, I64, F64 = torch.float32, torch.int32, torch.int64, torch.float64
getcontext().prec = 50

STATE_BIT = cvd.STATE_BIT
SUS_NAIVE = (1 << STATE_BIT['susceptible']) | (1 << STATE_BIT['naive'])
VSTATE_NONE = 0x00FFFFFF


def _align(x, a):
    return (x + a - 1) // a * a


def _upload(x, device):
    """A host array (numpy or CPU tensor) on the device through pinned memory, the
    copy asynchronous on the current stream: a new state's small tables then cost
    no synchronisation with the uploads and index builds queued before them (the
    pinned staging block is not reused before its copy has run)."""
    t = torch.from_numpy(x) if isinstance(x, np.ndarray) else x
    return t.pin_memory().to(device, non_blocking=True)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def ff_split(x):
    """A float64 value as a float32 pair (hi, lo), hi + lo = x to ~2^-48."""
    x = float(x)
    hi = np.float32(x)
    return float(hi), float(np.float32(x - float(hi)))


def ff_log(x):
    """ln(x) of a positive value as a float32 pair, from the decimal module (platform independent)."""
    d = Decimal(float(x)).ln()
    hi = np.float32(float(d))
    lo = np.float32(float(d - Decimal(float(hi))))
    return float(hi), float(lo)


def dur_par(dist):
    """Pack one duration distribution (utils.py:156-236 sample()) as (code, a, b)."""
    name = dist['dist']
    if name not in L.DIST_CODES:
        raise NotImplementedError(f'duration distribution "{name}" is not supported on the GPU path')
    code = L.DIST_CODES[name]
    p1, p2 = dist['par1'], dist['par2']
    if code in (0, 1):
        if not p1 > 0:
            return L.DurPar(L.DIST_ZERO, 0, 0.0, 0.0)
        mean = np.log(p1 ** 2 / np.sqrt(p2 ** 2 + p1 ** 2))   # utils.py:224
        sigma = np.sqrt(np.log(p2 ** 2 / p1 ** 2 + 1))         # utils.py:225
        return L.DurPar(code, 0, float(mean), float(sigma))
    return L.DurPar(code, 0, float(p1), float(p2))


class SimSpec:
    """Everything the device needs to know about one sim.

    Args:
        pars: full parameter dict (prognoses applied; nab_kin and immunity set if waning)
        person: per-person host arrays: symp_prob, severe_prob, crit_prob, death_prob, rel_trans, rel_sus
        layers: list of dicts(key, p1, p2, beta, dynamic) in layer order
        beta_sched: float64 [npts] overall beta per day (change_beta applied)
        beta_layer_sched: float64 [npts, n_layers] per-layer beta per day
        testing: test_prob / contact_tracing settings (``interventions.device_testing``) or None
    """

    def __init__(self, pars, person, layers, beta_sched=None, beta_layer_sched=None, testing=None):
        self.testing = testing  # dict from the test_prob / contact_tracing interventions, or None
        self.pars = pars
        self.person = person
        self.layers = layers
        self.n = int(pars['pop_size'])
        self.npts = int(pars['n_days']) + 1
        self.nv = int(pars['n_variants'])
        if self.nv > L.MAX_VARIANTS:
            raise ValueError(f'at most {L.MAX_VARIANTS} variants are supported')
        if len(layers) > L.MAX_LAYERS:
            raise ValueError(f'at most {L.MAX_LAYERS} layers are supported')
        keys = [ly['key'] for ly in layers]
        self.beta_sched = (np.full(self.npts, float(pars['beta'])) if beta_sched is None
                           else np.asarray(beta_sched, dtype=np.float64))
        if beta_layer_sched is None:
            beta_layer_sched = np.array([[float(pars['beta_layer'][k]) for k in keys]] * self.npts)
        self.beta_layer_sched = np.asarray(beta_layer_sched, dtype=np.float64).reshape(self.npts, len(keys))

    def beta_table(self):
        """sim.py:626: float32(beta * rel_beta * variant rel_beta) per day and variant."""
        p = self.pars
        tab = np.zeros((self.npts, self.nv), dtype=np.float32)
        for v in range(self.nv):
            label = p['variant_map'][v]
            rb = p['variant_pars'][label]['rel_beta']
            tab[:, v] = [np.float32(b * p['rel_beta'] * rb) for b in self.beta_sched]
        return tab


IMPORT_TAG = 0x1B1B
RESCALE_TAG = 0x5C5C
HOLD_NONE = 0x7FFFFFFF


def _max_of(x):
    """The largest value of a host array or device tensor (0 when empty)."""
    if torch.is_tensor(x):
        return float(x.max().item()) if x.numel() else 0.0
    x = np.asarray(x)
    return float(x.max()) if x.size else 0.0


def rse_bound(rel_sus_max, quar_factor):
    """The thinning bound of a dynamic layer: a float32 value at least
    rel_sus * (quarantined ? quar_factor : 1) * (1 - sus_imm) as the edge pass
    forms it in float32 for any agent (sus_imm in [0, 1]), i.e. the largest
    rel_sus, or its float32 product with quar_factor when that is larger."""
    rs = np.float32(rel_sus_max)
    return float(max(rs, np.float32(rs * np.float32(quar_factor))))


def dynamic_count_table(n_edges, n_agents):
    """The length distribution of one agent's contact list in a dynamic layer.

    Layer.update (base.py:1849-1876) redraws all n_edges edges of the layer with
    both endpoints uniform over the n_agents agents, so the edges of one agent as
    p1 (and, separately, as p2) number Binomial(n_edges, 1 / n_agents). Returns
    uint64 thresholds: entry k = floor(2^64 * P(count <= k)), the last entry
    2^64 - 1 (at the first k whose upper tail is below 2^-64, at most
    L.DYN_MAX_LIST entries). 50-digit decimal arithmetic, identical on every
    platform."""
    E, n = int(n_edges), int(n_agents)
    top = (1 << 64) - 1
    one = Decimal(1)
    if n == 1:
        if E >= L.DYN_MAX_LIST:
            raise ValueError('dynamic layer: contact lists longer than the supported maximum')
        return np.array([0] * E + [top], dtype=np.uint64)
    p = one / Decimal(n)
    q = one - p
    term = (Decimal(E) * q.ln()).exp()  # P(count = 0)
    tail_limit = Decimal(2) ** -64
    acc = Decimal(0)
    table = []
    for k in range(L.DYN_MAX_LIST):
        acc += term
        if one - acc < tail_limit or k == E:
            table.append(top)
            return np.array(table, dtype=np.uint64)
        table.append(min(int(acc * (1 << 64)), top))
        term = term * Decimal(E - k) / Decimal(k + 1) * p / q
    if one - acc > Decimal(2) ** -40:
        raise ValueError('dynamic layer: contact lists longer than the supported maximum (too many contacts '
                         'per agent)')
    table[-1] = top
    return np.array(table, dtype=np.uint64)


def daily_importations(seed, rate, n, npts, start=0):
    """The agents imported on days ``start`` .. ``npts - 1`` of a run (sim.py:582-587):
    a list of sorted arrays of distinct local indices. Day t's count is
    Poisson(rate[t]) (cvu.poisson, utils.py:379-390, with the rate rounded to the
    float32 of its numba signature; ``rate`` a number or one per day, n_imports
    over the day's scale) and its agents a uniform choice without replacement
    among all ``n`` (cvu.choose, utils.py:430-443), both from a PCG64 stream keyed
    by (seed, 0x1B1B, t). Neither depends on the sim's state, so a run's
    importations are drawn before it starts (and redrawn from the day of a
    rescaling on). A count above ``n`` raises ValueError, as the reference's
    choice does."""
    rates = np.broadcast_to(np.asarray(rate, dtype=np.float64), (int(npts),))
    out = []
    for t in range(int(start), int(npts)):
        rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, IMPORT_TAG, t]))
        k = int(rng.poisson(float(np.float32(rates[t]))))
        if k > n:
            raise ValueError(f'day {t}: {k} importations drawn for a population of {n}: cannot take a larger '
                             'sample than population when replace=False')
        out.append(np.sort(rng.choice(int(n), size=k, replace=False)).astype(np.int64) if k
                   else np.zeros(0, dtype=np.int64))
    return out


def prob_threshold(p):
    """ceil(p * 2^53) as an exact integer: the device's test 2k + 1 < threshold on
    the 52 random bits k of a uniform (2k + 1) / 2^53 is float64's u < p."""
    p = float(p)
    if not p > 0.0:
        return 0
    if p >= 1.0:
        return (1 << 53) + 1
    num, den = p.as_integer_ratio()
    return -((-num << 53) // den)


def testing_record(spec):
    """covgpu_testing of one sim (both interventions off when ``spec.testing`` is None)."""
    r = L.Testing()
    r.test_start, r.test_end, r.trace_start, r.trace_end = 1, 0, 1, 0
    T = spec.testing
    if not T:
        return r
    keys = [ly['key'] for ly in spec.layers]
    if T.get('test') is not None:
        tp = T['test']
        r.test_start, r.test_end = tp['start_day'], tp['end_day']
        r.quar_policy, r.quar_offsets = tp['quar_policy'], tp['quar_offsets']
        r.thr_symp, r.thr_asymp = prob_threshold(tp['symp_prob']), prob_threshold(tp['asymp_prob'])
        r.thr_symp_quar, r.thr_asymp_quar = prob_threshold(tp['symp_quar_prob']), prob_threshold(tp['asymp_quar_prob'])
        r.thr_sensitivity = prob_threshold(tp['sensitivity'])
        r.thr_not_lost = prob_threshold(1.0 - tp['loss_prob'])  # people.py:611 n_binomial(1.0 - loss_prob, ...)
        r.test_delay = tp['test_delay']
    if T.get('trace') is not None:
        ct = T['trace']
        r.trace_start, r.trace_end = ct['start_day'], ct['end_day']
        r.presumptive = int(ct['presumptive'])
        for li, k in enumerate(keys):
            prob, tt = ct['trace_probs'].get(k, 0.0), float(ct['trace_time'].get(k, 0.0))
            r.thr_trace[li] = 0 if prob == 0 else prob_threshold(prob)  # interventions.py:1103 skips prob == 0
            r.trace_time[li] = tt
            r.trace_start_off[li] = int(tt)                        # people.py:635 int(t + trace_time)
            r.trace_period[li] = int(ct['quar_period'] - tt)       # people.py:636 int(quar_period - trace_time)
    return r


ILI_TAG = 0x111E


def ili_agents(seed, t, n, n_ili):
    """The n_ili distinct agents with influenza-like symptoms on day t (test_prob's
    ili_prev, interventions.py:941-947), from a PCG64 stream keyed by (seed, 0x111E,
    t): they do not depend on the sim's state, so they are drawn on the host."""
    rng = np.random.default_rng([int(seed) & 0xFFFFFFFFFFFFFFFF, ILI_TAG, int(t)])
    return np.sort(rng.choice(int(n), int(n_ili), replace=False)).astype(np.int32)


# Default of covgpu_state.src_walk for a state with a redrawn layer: the stored
# layers are walked from the day's sources while fewer than 1/128 of a sim's agents
# are infectious, and streamed otherwise (results are the same either way). The
# walk then runs in the redrawn layers' launch, beside their draws: on the 1M-agent
# hybrid run, 18.45 -> 18.0 ms per run (thresholds 1/64 to 1/512 within 0.1 ms of
# each other). Without a redrawn layer the walk is a launch of its own after the
# tile pass, which costs about 12 us a day before any source is walked, and the
# stored layers are streamed (0), unless the state holds at least SRC_WALK_MIN_EDGES
# stored edges: then the day's stream is long enough for the walk to pay even as a
# launch of its own (256 random-population sims, 320M edges, 120 days: 262 -> 238 ms
# per batched run walking below 1/64 infectious).
SRC_WALK = 128
SRC_WALK_BIG = 64
SRC_WALK_MIN_EDGES = 50_000_000


def parse_edge_tile(choice):
    """An edge-pass label ('4096', 4096, '8192r', '1024w', '1024w4') as
    set_edge_tile's keyword arguments."""
    text = str(choice)
    if text.endswith('r'):
        return dict(tile=int(text[:-1]), resident=True)
    if 'w' in text:
        tile, cap = text.split('w', 1)
        return dict(tile=int(tile), wave=int(cap) if cap else True)
    return dict(tile=int(text))


class BatchState:
    """Agent and layer arrays of one or more sims in device memory."""

    def __init__(self, specs, device='cuda', event_capacity=None, log_capacity=None, log=True,
                 edge_tile=L.EDGE_TILE):
        et = parse_edge_tile(edge_tile)
        if et['tile'] not in L.EDGE_TILES or et.get('resident'):
            raise ValueError(f'edge tile must be one of {L.EDGE_TILES}, optionally with the one-wave suffix w')
        self.edge_tile = et['tile']
        self.edge_resident = False
        self.edge_wave = L.EDGE_WAVE_MAX if et.get('wave') is True else int(et.get('wave', 0))
        if any(ly.get('dynamic') for sp in specs for ly in sp.layers):
            self.src_walk = SRC_WALK
        else:
            stored = sum(len(ly['p1']) for sp in specs for ly in sp.layers)
            self.src_walk = SRC_WALK_BIG if stored >= SRC_WALK_MIN_EDGES else 0
        self._index_pending = []  # stored segments whose agent index is built on demand
        self._index_tensors = []
        if not torch.cuda.is_available():
            raise RuntimeError('covasim_gb300 needs a CUDA device: the GPU path has no CPU fallback')
        self.lib = L.lib()
        self.device = torch.device(device)
        self.specs = list(specs)
        S = len(self.specs)
        offs, n = [], 0
        for sp in self.specs:
            offs.append(n)
            n = _align(n + sp.n, L.AGENT_ALIGN)
        self.offsets = offs
        self.n = max(n, L.AGENT_ALIGN)
        self.nv_max = max(sp.nv for sp in self.specs)
        dev = self.device
        n = self.n
        t = {}
        t['flags'] = torch.zeros(n, dtype=I32, device=dev)
        t['vstate'] = torch.full((n,), VSTATE_NONE, dtype=I32, device=dev)
        for k in ('symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus', 'peak_nab', 'nab',
                  'viral_load'):
            t[k] = torch.zeros(n, dtype=F32, device=dev)
        for k in ('n_infections', 'n_breakthroughs', 't_nab_event', 'vaccine_source'):
            t[k] = torch.zeros(n, dtype=I32, device=dev)
        for k in ('sus_imm', 'symp_imm', 'sev_imm'):
            t[k] = torch.zeros((self.nv_max, n), dtype=F32, device=dev)
        t['dates'] = torch.full((L.N_DATES, n), float('nan'), dtype=F32, device=dev)
        t['durs'] = torch.full((L.N_DURS, n), float('nan'), dtype=F32, device=dev)
        t['roles'] = torch.zeros(2 * ((n + 31) // 32), dtype=I32, device=dev)
        t['claim'] = torch.full((n,), -1, dtype=I64, device=dev)
        t['src_rec'] = torch.zeros((n, 4), dtype=F32, device=dev)  # the edge pass's record of each source
        t['tgt_rec'] = torch.zeros((self.nv_max, n), dtype=F32, device=dev)  # and of each target
        n_real = sum(sp.n for sp in self.specs)
        self.event_capacity = int(event_capacity or (2 * n_real + 65536))
        t['events'] = torch.zeros((self.event_capacity, 4), dtype=I32, device=dev)
        t['event_count'] = torch.zeros(1, dtype=I64, device=dev)
        self.log_enabled = log
        self.log_capacity = int(log_capacity or (3 * n_real + 65536)) if log else 0
        t['log'] = torch.zeros((max(self.log_capacity, 1), 4), dtype=I32, device=dev)
        t['log_count'] = torch.zeros(1, dtype=I64, device=dev)
        t['status'] = torch.zeros(1, dtype=I32, device=dev)
        # testing and tracing (interventions.py:858-1145): bitmaps, scheduled quarantines
        self.testing_recs = [testing_record(sp) for sp in self.specs]
        self.has_testing = any(sp.testing for sp in self.specs)
        self.has_swab = any((sp.testing or {}).get('test') and sp.testing['test'].get('swab_pdf') is not None
                            for sp in self.specs)
        self.has_capacity = any((sp.testing or {}).get('trace') and sp.testing['trace'].get('capacity') is not None
                                for sp in self.specs)
        self.pending_slots = 1
        self.n_contact_layers = max(len(sp.layers) for sp in self.specs) or 1
        if self.has_testing:
            for r, sp in zip(self.testing_recs, self.specs):
                offs_used = [r.trace_start_off[li] for li in range(len(sp.layers)) if r.thr_trace[li]]
                if min(offs_used, default=0) < 0:
                    raise ValueError('contact_tracing trace_time must not be negative')
                self.pending_slots = max(self.pending_slots, max(offs_used, default=0) + 1)
            words = (n + 31) // 32
            t['trace_bits'] = torch.zeros(words, dtype=I32, device=dev)
            t['contact_bits'] = torch.zeros(self.n_contact_layers * words, dtype=I32, device=dev)
            t['pending_quar'] = torch.full((self.pending_slots, n), -1, dtype=I32, device=dev)
            t['trace_count'] = torch.zeros(S, dtype=I32, device=dev)
            self.testing_tensors = self._testing_extras(dev)
        self.t = t

        # per-sim tables, concatenated
        self.res_int = torch.zeros(sum(sp.npts for sp in self.specs) * L.N_RES_INT, dtype=I64, device=dev)
        self.res_var = torch.zeros(sum(sp.npts * L.N_RES_VAR * sp.nv for sp in self.specs), dtype=I64, device=dev)
        self.res_fx = torch.zeros(sum(sp.npts for sp in self.specs) * L.N_RES_F, dtype=I64, device=dev)
        beta_tabs, bl_tabs, kins = [], [], []
        for sp in self.specs:
            beta_tabs.append(sp.beta_table().ravel())
            bl_tabs.append(sp.beta_layer_sched.astype(np.float32).ravel())
            kin = np.asarray(sp.pars.get('nab_kin') if sp.pars.get('nab_kin') is not None else np.zeros(1),
                             dtype=np.float64)
            hi = kin.astype(np.float32)
            lo = (kin - hi.astype(np.float64)).astype(np.float32)
            kins.append(np.stack([hi, lo], axis=1).ravel())   # float pairs: hi + lo = nab_kin to ~2^-48
        self.beta_tab = _upload(np.concatenate(beta_tabs), dev)
        self.beta_layer_tab = _upload(np.concatenate(bl_tabs) if bl_tabs else np.zeros(1, np.float32), dev)
        self.nab_kin = _upload(np.concatenate(kins), dev)  # float32 pairs

        self._build_rescale()
        self._build_imports()
        self._init_people()
        self._build_layers()
        self._build_sims(beta_tabs, bl_tabs, kins)
        self._build_agent_blocks()
        self.draw_table = None
        self.edge_uniform_tensors = None
        self.hospicu = None
        self.lik = None
        self.lik_active = False
        self._refresh_state()

    # ------------------------------------------------------------------ building
    def _testing_extras(self, dev):
        """Device tables of test_prob's subtargets (a threshold per agent) and
        influenza-like illness (the day's agents, drawn on the host, and the mark
        array the device writes), set into each sim's testing record."""
        keep = []
        for r, sp in zip(self.testing_recs, self.specs):
            ct = (sp.testing or {}).get('trace')
            if ct and ct.get('capacity') is not None:
                cap_list = torch.zeros(max(sp.n, 1), dtype=I32, device=dev)
                cap_count = torch.zeros(1, dtype=I32, device=dev)
                p = sp.pars  # the day's scale without dynamic rescaling, as _build_rescale sets it
                r.capacity = float(ct['capacity'])
                r.cap_scale = 1.0 if bool(p.get('rescale', True)) else float(p.get('pop_scale') or 1)
                r.cap_list, r.cap_count = cap_list.data_ptr(), cap_count.data_ptr()
                keep += [cap_list, cap_count]
            tp = (sp.testing or {}).get('test')
            if not tp:
                continue
            if tp.get('subtarget') is not None:
                inds, vals = tp['subtarget']
                thr = np.full(sp.n, L.NO_SUBTARGET, dtype=np.uint64)
                thr[inds] = np.array([prob_threshold(v) for v in vals], dtype=np.uint64)
                tt = torch.from_numpy(thr.view(np.int64)).to(dev)
                r.sub_thr = tt.data_ptr()
                keep.append(tt)
            if tp.get('ili_prev') is not None:
                daily = np.asarray(tp['ili_prev'], dtype=np.float64)
                start = int(tp['start_day'])
                days = max(0, min(len(daily), sp.npts - start))
                seed = int(sp.pars['rand_seed'])
                lists = [ili_agents(seed, start + d, sp.n, int(daily[d] * sp.n)) for d in range(days)]
                off = np.zeros(days + 1, dtype=np.int64)
                off[1:] = np.cumsum([len(x) for x in lists])
                inds = np.concatenate(lists) if lists else np.zeros(0, dtype=np.int32)
                t_off = torch.from_numpy(off).to(dev)
                t_inds = torch.from_numpy(np.ascontiguousarray(inds, dtype=np.int32) if len(inds)
                                          else np.zeros(1, dtype=np.int32)).to(dev)
                t_mark = torch.full((max(sp.n, 1),), -1, dtype=I32, device=dev)
                r.ili_off, r.ili_inds, r.ili_mark, r.ili_days = (t_off.data_ptr(), t_inds.data_ptr(),
                                                                  t_mark.data_ptr(), days)
                keep += [t_off, t_inds, t_mark]
            if tp.get('swab_pdf') is not None:
                pdf = torch.from_numpy(np.ascontiguousarray(tp['swab_pdf'], dtype=np.float64)).to(dev)
                bins = torch.zeros(len(tp['swab_pdf']) + 1, dtype=I32, device=dev)
                r.swab_pdf, r.swab_bins, r.swab_len = pdf.data_ptr(), bins.data_ptr(), len(tp['swab_pdf'])
                r.symp_prob = float(tp['symp_prob'])
                keep += [pdf, bins]
        return keep

    def _build_imports(self):
        """Every sim's daily importations as one device table ordered by day, then
        sim (``covgpu_state.imports``), with the per-day counts kept on the host for
        the ``n_imports`` result."""
        self.import_sched = []
        for sp, vec in zip(self.specs, self.rescale_vecs):
            rate = sp.pars.get('n_imports') or 0
            self.import_sched.append(daily_importations(sp.pars['rand_seed'], rate / vec, sp.n, sp.npts) if rate
                                     else None)
        self.import_variant = [np.zeros(sp.npts) for sp in self.specs]  # variant.apply's, added as they happen
        self.log_labels = []  # infect() layer labels other than the layers, seeds, importations and None
        self._upload_imports()

    def _upload_imports(self):
        days = max(sp.npts for sp in self.specs)
        per_day = [[] for _ in range(days)]
        self.import_daily = []
        for k, (sp, off, sched) in enumerate(zip(self.specs, self.offsets, self.import_sched)):
            counts = np.zeros(sp.npts)
            for t, inds in enumerate(sched or []):
                if len(inds):
                    per_day[t].append((inds + off, k))
                    counts[t] = len(inds)
            self.import_daily.append(counts)
        day_off = np.zeros(days + 1, dtype=np.int64)
        for t in range(days):
            day_off[t + 1] = day_off[t] + sum(len(g) for g, _ in per_day[t])
        self.import_days = days if day_off[-1] else 0
        self.import_tabs = None
        if self.import_days:
            inds = np.concatenate([g for d in per_day for g, _ in d]).astype(np.int32)
            sims = np.concatenate([np.full(len(g), k, dtype=np.int32) for d in per_day for g, k in d])
            self.import_tabs = {'day_off': torch.from_numpy(day_off).to(self.device),
                                'inds': torch.from_numpy(inds).to(self.device),
                                'sims': torch.from_numpy(sims).to(self.device)}

    def _build_rescale(self):
        """The scale of each day of each sim (sim.py:342-346: 1 to start with when
        rescaling dynamically, else pop_scale) and, when some sim rescales
        dynamically (sim.py:535-556), the device word that holds a run back on
        the day a rescaling is due and the counters of the day check."""
        self.rescale_vecs, self.rescaling = [], []
        for sp in self.specs:
            p = sp.pars
            pop_scale = float(p.get('pop_scale') or 1)
            dynamic = bool(p.get('rescale', True))
            self.rescale_vecs.append((1.0 if dynamic else pop_scale) * np.ones(sp.npts))
            self.rescaling.append(dynamic and pop_scale > 1)
        self.hold = self.rescale_dev = self.nonnaive = None
        self._rescaled_day = -1
        if any(self.rescaling):
            dev = self.device
            self.hold = torch.full((1,), HOLD_NONE, dtype=I32, device=dev)
            self.rescale_dev = [torch.from_numpy(v.copy()).to(dev) for v in self.rescale_vecs]
            self.nonnaive = torch.tensor([[0, -1, -1]] * len(self.specs), dtype=I64, device=dev)

    def _reset_rescale(self):
        if self.hold is None:
            return
        for k, sp in enumerate(self.specs):
            if self.rescaling[k]:
                self.rescale_vecs[k][:] = 1.0
                self.rescale_dev[k].fill_(1.0)
        self.hold.fill_(HOLD_NONE)
        self.nonnaive.copy_(torch.tensor([[0, -1, -1]] * len(self.specs), dtype=I64))
        self._rescaled_day = -1
        if any(sched is not None for sched in self.import_sched):
            self._build_imports()

    def count_nonnaive(self, sim):
        """Start the day check's count of agents not naive (after seeding)."""
        if self.hold is None or not self.rescaling[sim]:
            return
        naive = (self.t['flags'][self.sl(sim)] >> STATE_BIT['naive']) & 1
        m = int(self.specs[sim].n - int(naive.sum().item()))
        self.nonnaive[sim] = torch.tensor([m, -1, -1], dtype=I64)

    def held_day(self):
        """The day a run was held back on (a due rescaling), or None."""
        if self.hold is None:
            return None
        h = int(self.hold.item())
        return None if h == HOLD_NONE else h

    def rescale_day(self, t):
        """sim.py:535-556 at the start of day t, for every sim that rescales
        dynamically: when the agents not naive exceed rescale_threshold of the
        population and the scale has room to grow, scale up by at least
        rescale_factor and make that share of them naive again (agents drawn from
        a PCG64 stream keyed by (seed, 0x5C5C, t)); importations are redrawn from
        day t on. Clears the hold; the day check's counters restart from here."""
        if self.hold is None or t <= self._rescaled_day:
            return
        for k, sp in enumerate(self.specs):
            if not self.rescaling[k] or t >= sp.npts:
                continue
            p, vec = sp.pars, self.rescale_vecs[k]
            naive = (self.t['flags'][self.sl(k)] >> STATE_BIT['naive']) & 1
            not_naive = torch.nonzero(naive == 0).squeeze(1)
            m = int(not_naive.numel())
            pop_scale, current = float(p['pop_scale']), vec[t]
            ratio = m / sp.n
            if current < pop_scale and ratio > p['rescale_threshold']:
                scaling = min(max(ratio / p['rescale_threshold'], p['rescale_factor']), pop_scale / current)
                vec[t:] *= scaling
                n_new = int(round(m * (1.0 - 1.0 / scaling)))
                rng = np.random.Generator(np.random.PCG64([int(p['rand_seed']) & 0xFFFFFFFFFFFFFFFF, RESCALE_TAG, t]))
                choices = torch.from_numpy(rng.choice(m, size=n_new, replace=False)).to(self.device)
                self.make_naive(not_naive[choices], sim=k)
                m -= n_new
                self.rescale_dev[k].copy_(torch.from_numpy(vec))
                if self.import_sched[k] is not None:
                    self.import_sched[k][t:] = daily_importations(p['rand_seed'], p['n_imports'] / vec, sp.n,
                                                                  sp.npts, start=t)
                    self._upload_imports()
                    self._refresh_state()
            self.nonnaive[k] = torch.tensor([m, t - 1, t], dtype=I64)
        self.hold.fill_(HOLD_NONE)
        self._rescaled_day = t

    def make_naive(self, inds, sim=0):
        """people.py:378-412 make_naive (vaccination kept) for local indices (a
        device tensor): states back to susceptible and naive, variant fields
        undefined, immunity, NAb and vaccine fields of the unvaccinated zeroed,
        every date but date_vaccinated and every duration undefined."""
        t = self.t
        g = inds.to(device=self.device, dtype=I64) + self.offsets[sim]
        vacc_bit = 1 << STATE_BIT['vaccinated']
        f = t['flags'][g]
        t['flags'][g] = (f & vacc_bit) | SUS_NAIVE
        t['vstate'][g] = (t['vstate'][g] & ~VSTATE_NONE) | VSTATE_NONE
        nvx = g[(f & vacc_bit) == 0]
        for k in ('sus_imm', 'symp_imm', 'sev_imm'):
            t[k][:, nvx] = 0
        for k in ('peak_nab', 'nab', 't_nab_event', 'vaccine_source'):
            t[k][nvx] = 0
        rows = [r for r, key in enumerate(cvd.DATES) if key != 'date_vaccinated']
        t['dates'][torch.tensor(rows, device=self.device).unsqueeze(1), g.unsqueeze(0)] = float('nan')
        t['durs'][:, g] = float('nan')

    def note_imports(self, sim, t, n):
        """Count variant importations (immunity.py:129) in the sim's ``n_imports``."""
        self.import_variant[sim][t] += n

    def _init_people(self):
        t = self.t
        for sp, off in zip(self.specs, self.offsets):
            t['flags'][off:off + sp.n] = SUS_NAIVE
            for k in ('symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus'):
                x = sp.person[k]
                src = x if torch.is_tensor(x) else torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32))
                t[k][off:off + sp.n].copy_(src, non_blocking=True)

    def _build_layers(self):
        self.segments = []   # (ctypes Layer, tensors kept alive)
        self.layer_tensors = []
        self.segment_index = {}  # (sim, layer) -> segment index
        checks, deferred = [], []  # device checks of torch layer inputs; their index builds
        for s, (sp, off) in enumerate(zip(self.specs, self.offsets)):
            for li, ly in enumerate(sp.layers):
                p1 = ly['p1'] if torch.is_tensor(ly['p1']) else np.asarray(ly['p1'], dtype=np.int64)
                n_edges = len(p1)
                if n_edges == 0:
                    continue
                rec = L.Layer()
                rec.n_edges = n_edges
                rec.sim = s
                rec.layer = li
                rec.iso_factor = np.float32(sp.pars['iso_factor'][ly['key']])
                rec.quar_factor = np.float32(sp.pars['quar_factor'][ly['key']])
                keep = []
                if ly.get('dynamic'):
                    rec.dynamic = 1
                    rec.beta_const = 1.0
                    cdf = _upload(dynamic_count_table(n_edges, sp.n).view(np.int64), self.device)
                    rec.dyn_cdf, rec.dyn_k = cdf.data_ptr(), len(cdf)
                    rec.dyn_rse_max = rse_bound(_max_of(sp.person['rel_sus']), rec.quar_factor)
                    keep.append(cdf)
                elif torch.is_tensor(ly['p1']):
                    # torch inputs (e.g. pinned host memory): uploaded as they are, checked on the
                    # device; the checks of every layer are read back together below, before
                    # anything indexes with them
                    tp1 = ly['p1'].to(self.device, torch.int32, non_blocking=True)
                    tp2 = ly['p2'].to(self.device, torch.int32, non_blocking=True)
                    lo1, hi1 = torch.aminmax(tp1)
                    lo2, hi2 = torch.aminmax(tp2)
                    unsorted = (tp1[1:] < tp1[:-1]).any() if n_edges > 1 else torch.zeros((), dtype=torch.bool,
                                                                                          device=self.device)
                    checks.append((ly['key'], sp.n, torch.stack([unsorted.to(torch.int64), torch.minimum(lo1, lo2).to(
                        torch.int64), torch.maximum(hi1, hi2).to(torch.int64)])))
                    if off:  # out of place: .to() returns the caller's tensor when it is already on the device
                        tp1 = tp1 + off
                        tp2 = tp2 + off
                    rec.p1, rec.p2 = tp1.data_ptr(), tp2.data_ptr()
                    keep += [tp1, tp2]
                    deferred.append((rec, sp, off, n_edges, keep))
                    b = ly.get('beta')
                    if b is None or bool((b == b[0]).all()):
                        rec.beta = None
                        rec.beta_const = 1.0 if b is None else float(b[0])
                    else:
                        tb = b.to(self.device, torch.float32, non_blocking=True)
                        rec.beta = tb.data_ptr()
                        keep.append(tb)
                else:
                    p2 = np.asarray(ly['p2'], dtype=np.int64)
                    beta = np.asarray(ly.get('beta', np.ones(n_edges)), dtype=np.float32)
                    if len(p1) > 1 and np.any(p1[1:] < p1[:-1]):
                        order = np.argsort(p1, kind='stable')
                        p1, p2, beta = p1[order], p2[order], beta[order]
                    if p1.min() < 0 or p1.max() >= sp.n or p2.min() < 0 or p2.max() >= sp.n:
                        raise ValueError(f'layer {ly["key"]}: agent index out of range')
                    tp1 = torch.from_numpy((p1 + off).astype(np.int32)).to(self.device)
                    tp2 = torch.from_numpy((p2 + off).astype(np.int32)).to(self.device)
                    if tp1.data_ptr() % 16 or tp2.data_ptr() % 16:
                        raise RuntimeError('edge arrays must be 16-byte aligned')
                    rec.p1, rec.p2 = tp1.data_ptr(), tp2.data_ptr()
                    keep += [tp1, tp2]
                    keep += self._trace_index(rec, sp, off, n_edges)
                    if np.all(beta == beta[0]):
                        rec.beta = None
                        rec.beta_const = float(beta[0])
                    else:
                        tb = torch.from_numpy(beta).to(self.device)
                        rec.beta = tb.data_ptr()
                        keep.append(tb)
                self.segment_index[(s, li)] = len(self.segments)
                self.segments.append(rec)
                self.layer_tensors.append(keep)
        if checks:  # one read-back for all torch layers
            got = torch.stack([c[2] for c in checks]).cpu().tolist()
            for (key, n, _), (unsorted, lo, hi) in zip(checks, got):
                if unsorted:
                    raise ValueError(f'layer {key}: p1 must be sorted')
                if lo < 0 or hi >= n:
                    raise ValueError(f'layer {key}: agent index out of range')
        for rec, sp, off, n_edges, keep in deferred:
            keep += self._trace_index(rec, sp, off, n_edges)
        self._tile_segments()

    def _trace_index(self, rec, sp, off, n_edges):
        """Agent index of a stored layer (covgpu_trace_index), built now when the sim
        traces (tracing visits the traced agents' edges through it), else when the
        walk from the sources is switched on (set_src_walk)."""
        if n_edges < 1 or n_edges > 0xFFFFFFFF:
            return []
        T = sp.testing
        if not (T and T.get('trace') is not None) and not self.src_walk:
            self._index_pending.append((rec, sp, off, n_edges))
            return []
        return self._build_index(rec, sp, off, n_edges)

    def _build_index(self, rec, sp, off, n_edges):
        dev, n = self.device, sp.n
        rp1 = torch.empty(n + 1, dtype=I32, device=dev)
        rp2 = torch.empty(n + 1, dtype=I32, device=dev)
        perm2 = torch.empty(n_edges, dtype=I32, device=dev)
        scratch = torch.empty(int(self.lib.covgpu_trace_index_scratch(n)), dtype=I64, device=dev)
        L.call('covgpu_trace_index', rec.p1, rec.p2, int(n_edges), int(off), int(n), rp1.data_ptr(), rp2.data_ptr(),
               perm2.data_ptr(), scratch.data_ptr(), _stream())
        rec.rp1, rec.rp2, rec.perm2 = rp1.data_ptr(), rp2.data_ptr(), perm2.data_ptr()
        self._index_scratch = scratch  # kept until the build has run on the stream
        return [rp1, rp2, perm2]

    def _tile_segments(self):
        """Each segment's first tile and the tile count for the current edge tile size
        (a dynamic layer has no tiles: the edge pass draws its edges from the day's sources)."""
        tiles = 0
        for rec in self.segments:
            rec.tile_begin = tiles
            if not rec.dynamic:
                tiles += (rec.n_edges + self.edge_tile - 1) // self.edge_tile
        self.n_tiles = tiles
        self.n_dynamic = sum(1 for rec in self.segments if rec.dynamic)
        arr = (L.Layer * max(len(self.segments), 1))(*self.segments)
        self.seg_dev = _upload(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8), self.device)

    def set_edge_tile(self, tile, resident=False, wave=0):
        """Edges per edge-pass tile (one of L.EDGE_TILES), whether the source bitmap
        is resident in shared memory (one sim only), and whether the stored layers'
        pass runs as one wave of blocks walking balanced ranges of tiles (wave: at
        most that many blocks per SM; True: as many as fit); the autotuner's knobs."""
        if int(tile) not in L.EDGE_TILES:
            raise ValueError(f'edge tile must be one of {L.EDGE_TILES}')
        if resident and wave:
            raise ValueError('the resident-bitmap edge pass has its own grid (one block per SM)')
        self.edge_tile = int(tile)
        self.edge_resident = False
        self.edge_wave = L.EDGE_WAVE_MAX if wave is True else int(wave)
        if self.edge_wave < 0:
            raise ValueError('wave: blocks per SM, at least 1 (0: one block per tile)')
        self._tile_segments()
        self._refresh_state()
        if resident:
            if int(tile) < 4096 or not self.resident_possible():
                raise ValueError('the resident-bitmap edge pass needs one sim of at most ~1.1M agents and tiles '
                                 'of 4096 or 8192 edges')
            self.edge_resident = True
            self._refresh_state()

    def resident_possible(self):
        return int(self.lib.covgpu_edge_resident_bytes(self.cstate_ptr)) > 0

    def set_src_walk(self, k):
        """Quiet-day walk of the stored layers (covgpu_state.src_walk): k > 0 walks
        a layer from the day's sources while its sim's infectious agents x k are
        fewer than its agents, 0 never, -1 always (building the layers' agent index
        first). Results do not depend on it."""
        self.src_walk = int(k)
        if self.src_walk and self._index_pending:
            for rec, sp, off, n_edges in self._index_pending:
                self._index_tensors += self._build_index(rec, sp, off, n_edges)
            self._index_pending = []
            self._tile_segments()  # the segment table with the indices
        self._refresh_state()

    @property
    def edge_tile_label(self):
        """The edge-pass configuration as one value: the tile size, suffixed 'r'
        when the source bitmap is resident in shared memory ('4096r'), 'w' when the
        stored layers' pass runs as one wave ('1024w'; '1024w4': at most four blocks
        per SM)."""
        if self.edge_resident:
            return f'{self.edge_tile}r'
        if self.edge_wave:
            return f'{self.edge_tile}w' + ('' if self.edge_wave == L.EDGE_WAVE_MAX else str(self.edge_wave))
        return self.edge_tile

    def apply_edge_tile(self, choice):
        """Set the edge pass from a user choice: None (the default tile), 'auto'
        (autotuned on this state), a tile size, or a label such as '8192r'."""
        if choice is None:
            return
        if choice == 'auto':
            from .autotune import tune_edge_tile
            tune_edge_tile(self)
            return
        self.set_edge_tile(**parse_edge_tile(choice))

    def _build_sims(self, beta_tabs, bl_tabs, kins):
        recs = []
        ri = rv = rf = bt = bl = kn = 0
        self.res_slices = []
        for s, (sp, off) in enumerate(zip(self.specs, self.offsets)):
            p = sp.pars
            r = L.SimParams()
            r.agent_off = off
            r.n_agents = sp.n
            r.n_variants = sp.nv
            r.n_layers = len(sp.layers)
            r.npts = sp.npts
            r.pop_scale = float(p.get('pop_scale') or 1)
            r.rescale_threshold = float(p.get('rescale_threshold') or 0)
            if self.hold is not None and self.rescaling[s]:
                r.rescale_vec = self.rescale_dev[s].data_ptr()
                r.nonnaive = self.nonnaive[s].data_ptr()
            seed = int(p['rand_seed']) & 0xFFFFFFFFFFFFFFFF
            r.key0, r.key1 = seed & 0xFFFFFFFF, seed >> 32
            r.use_waning = int(bool(p['use_waning']))
            r.nab_kin_len = len(kins[s]) // 2
            r.n_beds_hosp = -1 if p['n_beds_hosp'] is None else int(p['n_beds_hosp'])
            r.n_beds_icu = -1 if p['n_beds_icu'] is None else int(p['n_beds_icu'])
            vd = p['viral_dist']
            r.frac_time, r.load_ratio, r.high_cap = (np.float32(vd['frac_time']), np.float32(vd['load_ratio']),
                                                     np.float32(vd['high_cap']))
            r.asymp_factor = np.float32(p['asymp_factor'])
            r.trans_redux = np.float32(p['trans_redux'])
            r.nab_boost = np.float32(p['nab_boost'])
            r.no_hosp_factor = np.float32(p['no_hosp_factor'])
            r.no_icu_factor = np.float32(p['no_icu_factor'])
            for v in range(sp.nv):  # people.py:475-480
                label = p['variant_map'][v]
                vals = {}
                for k in ('rel_symp_prob', 'rel_severe_prob', 'rel_crit_prob', 'rel_death_prob'):
                    x = p[k]
                    if v:
                        x *= p['variant_pars'][label][k]
                    vals[k] = np.float32(x)
                r.rel_symp[v], r.rel_severe[v] = vals['rel_symp_prob'], vals['rel_severe_prob']
                r.rel_crit[v], r.rel_death[v] = vals['rel_crit_prob'], vals['rel_death_prob']
            imm = p.get('immunity')
            if imm is not None:
                imm = np.asarray(imm, dtype=np.float32)
                for a in range(sp.nv):
                    for b in range(sp.nv):
                        r.immunity[a * L.MAX_VARIANTS + b] = imm[a, b]
            ris = p['rel_imm_symp']
            r.rel_imm_asymp, r.rel_imm_mild, r.rel_imm_severe = float(ris['asymp']), float(ris['mild']), float(ris['severe'])
            ne = p['nab_eff']
            r.nab_norm = 1 + ne['alpha_inf_diff']
            for j, (a, b) in enumerate([('alpha_inf', 'beta_inf'), ('alpha_symp_inf', 'beta_symp_inf'),
                                        ('alpha_sev_symp', 'beta_sev_symp')]):
                r.ve_alpha[j][0], r.ve_alpha[j][1] = ff_split(ne[a])   # exp(alpha) * eff^beta = e^(alpha + beta ln eff)
                r.ve_beta[j][0], r.ve_beta[j][1] = ff_split(ne[b])
            if imm is not None:
                for a in range(sp.nv):
                    for b in range(sp.nv):
                        x = float(imm[a, b])
                        if x > 0:
                            r.ln_immunity[a * L.MAX_VARIANTS + b][0], r.ln_immunity[a * L.MAX_VARIANTS + b][1] = ff_log(x)
            for j, key in enumerate(L.DUR_ORDER):
                r.dur[j] = dur_par(p['dur'][key])
            nab_init = p['nab_init']
            r.nab_init = dur_par(nab_init) if nab_init is not None else L.DurPar(L.DIST_ZERO, 0, 0.0, 0.0)
            r.nab_kin = self.nab_kin.data_ptr() + 4 * kn
            r.beta_tab = self.beta_tab.data_ptr() + 4 * bt
            r.beta_layer_tab = self.beta_layer_tab.data_ptr() + 4 * bl
            r.vx_imm = None
            r.n_vaccines = 0
            r.res_int = self.res_int.data_ptr() + 8 * ri
            r.res_var = self.res_var.data_ptr() + 8 * rv
            r.res_fx = self.res_fx.data_ptr() + 8 * rf
            r.testing = self.testing_recs[s]
            for li in range(L.MAX_LAYERS):
                r.seg_of_layer[li] = self.segment_index.get((s, li), -1)
            self.res_slices.append((ri, rv, rf))
            ri += sp.npts * L.N_RES_INT
            rv += sp.npts * L.N_RES_VAR * sp.nv
            rf += sp.npts * L.N_RES_F
            bt += len(beta_tabs[s])
            bl += len(bl_tabs[s])
            kn += len(kins[s])
            recs.append(r)
        arr = (L.SimParams * len(recs))(*recs)
        self.sim_recs = recs
        self.sims_dev = _upload(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8), self.device)

    def _build_agent_blocks(self):
        dt = np.dtype([('begin', '<i8'), ('end', '<i8'), ('sim', '<i4'), ('_pad', '<i4')])
        parts = []
        for s, (sp, off) in enumerate(zip(self.specs, self.offsets)):
            nb = (sp.n + L.AGENT_BLOCK - 1) // L.AGENT_BLOCK
            b = np.zeros(nb, dtype=dt)
            b['begin'] = off + np.arange(nb, dtype=np.int64) * L.AGENT_BLOCK
            b['end'] = np.minimum(b['begin'] + L.AGENT_BLOCK, off + sp.n)
            b['sim'] = s
            parts.append(b)
        blocks = np.concatenate(parts)
        self.n_agent_blocks = len(blocks)
        self.blocks_dev = _upload(blocks.view(np.uint8).copy(), self.device)

    def _refresh_state(self):
        t = self.t
        st = L.State()
        st.n = self.n
        st.n_sims = len(self.specs)
        st.n_segments = len(self.segments)
        st.n_tiles = self.n_tiles
        st.n_dynamic = self.n_dynamic
        st.src_walk = int(self.src_walk)
        st.n_agent_blocks = self.n_agent_blocks
        st.edge_tile = self.edge_tile
        st.edge_resident = int(self.edge_resident)
        st.edge_wave = int(self.edge_wave)
        for k in ('flags', 'vstate', 'symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus',
                  'n_infections', 'n_breakthroughs', 'peak_nab', 'nab', 't_nab_event', 'vaccine_source', 'sus_imm',
                  'symp_imm', 'sev_imm', 'dates', 'durs', 'viral_load', 'roles', 'claim', 'src_rec', 'tgt_rec',
                  'events', 'event_count',
                  'log_count', 'status'):
            setattr(st, k, t[k].data_ptr())
        st.imm_stride_variants = self.nv_max
        st.event_capacity = self.event_capacity
        st.log = t['log'].data_ptr() if self.log_enabled else None
        st.log_capacity = self.log_capacity
        st.hospicu = self.hospicu.data_ptr() if self.hospicu is not None else None
        st.sims = self.sims_dev.data_ptr()
        st.segments = self.seg_dev.data_ptr() if self.segments else None
        st.agent_blocks = self.blocks_dev.data_ptr()
        st.draw_table = self.draw_table.data_ptr() if self.draw_table is not None else None
        st.has_testing = 0
        if self.has_testing:  # bit 0 and its refinements
            st.has_testing = (1 | (2 if self.has_swab else 0) | (4 if self.has_capacity else 0) |
                              (8 if all(rec.dynamic or rec.rp1 for rec in self.segments) else 0))
        st.pending_slots = self.pending_slots
        st.n_contact_layers = self.n_contact_layers
        if self.has_testing:
            for k in ('trace_bits', 'contact_bits', 'pending_quar', 'trace_count'):
                setattr(st, k, t[k].data_ptr())
        st.hold = self.hold.data_ptr() if self.hold is not None else None
        st.import_days = self.import_days
        if self.import_tabs is not None:
            st.import_day_off = self.import_tabs['day_off'].data_ptr()
            st.imports = self.import_tabs['inds'].data_ptr()
            st.import_sims = self.import_tabs['sims'].data_ptr()
        if self.edge_uniform_tensors is not None:
            ptrs = np.array([u.data_ptr() for u in self.edge_uniform_tensors], dtype=np.uint64)
            self._eu_ptrs = torch.from_numpy(ptrs.view(np.int64)).to(self.device)
            st.edge_uniforms = self._eu_ptrs.data_ptr()
        else:
            st.edge_uniforms = None
        if self.lik is not None and self.lik_active:
            k = self.lik
            st.lik.factor = k['factor'].data_ptr()
            st.lik.ll = k['ll'].data_ptr()
            st.lik.expected = k['expected'].data_ptr()
            st.lik.g_ll = k['g_ll'].data_ptr() if k['grad'] else None
            st.lik.g_exp = k['g_exp'].data_ptr() if k['grad'] else None
            st.lik.logq = k['logq'].data_ptr()
            st.lik.w = k['w'].data_ptr()
            st.lik.npts_max, st.lik.n_layers_max, st.lik.nv_max = k['dims']
        self.cstate = st
        self.cstate_ptr = C.pointer(self.cstate)

    # ------------------------------------------------------------------ test hooks
    def set_draw_table(self, table):
        """Inject per-agent infection draws [n, N_DRAWS] (global index); None returns to Philox."""
        self.draw_table = None if table is None else torch.as_tensor(table, dtype=F64, device=self.device).contiguous()
        self._refresh_state()

    def set_edge_uniforms(self, per_segment):
        """Inject edge uniforms: list (one per segment) of float64 [n_variants, 2, n_edges] indexed by
        (source variant, direction, edge); None returns to Philox."""
        if per_segment is None:
            self.edge_uniform_tensors = None
        else:
            self.edge_uniform_tensors = [torch.as_tensor(u, dtype=F64, device=self.device).contiguous()
                                         for u in per_segment]
        self._refresh_state()

    def set_hospicu(self, flags):
        """Force hosp_max/icu_max per sim ([n_sims, 2] ints); None: from the day's counts."""
        self.hospicu = None if flags is None else torch.as_tensor(np.asarray(flags, dtype=np.int32).ravel(),
                                                                  device=self.device)
        self._refresh_state()

    # ------------------------------------------------------------------ likelihood
    def enable_lik(self, grad=False):
        """Allocate the likelihood buffers (covgpu_lik) and switch the passes on.
        With ``grad`` the per-layer sensitivities are accumulated too."""
        if self.lik is None:
            S = len(self.specs)
            T = max(sp.npts for sp in self.specs)
            Lm = max(len(sp.layers) for sp in self.specs) or 1
            V = self.nv_max
            dev = self.device
            f64 = torch.float64
            self.lik = dict(dims=(T, Lm, V), grad=False,
                            factor=torch.zeros((S, T, Lm, V, 2), dtype=torch.float32, device=dev),
                            ll=torch.zeros((S, T), dtype=f64, device=dev),
                            expected=torch.zeros((S, T), dtype=f64, device=dev),
                            g_ll=torch.zeros((S, T, Lm), dtype=f64, device=dev),
                            g_exp=torch.zeros((S, T, Lm), dtype=f64, device=dev),
                            logq=torch.zeros(self.n, dtype=f64, device=dev),
                            w=torch.zeros((Lm, self.n), dtype=f64, device=dev))
        self.lik['grad'] = bool(grad)
        self.lik_active = True
        self._refresh_state()

    def disable_lik(self):
        """Switch the likelihood passes off (the buffers are kept for the next enable_lik)."""
        self.lik_active = False
        self._refresh_state()

    def set_lik_factor(self, factor, sim=0):
        """F[t][layer][variant] of one sim (float64, see covgpu_lik), stored as
        float pairs (hi, lo)."""
        f = np.asarray(factor, dtype=np.float64)
        hi = f.astype(np.float32)
        lo = (f - hi.astype(np.float64)).astype(np.float32)
        pair = torch.from_numpy(np.stack([hi, lo], axis=-1))
        T, Lm, V = f.shape
        self.lik['factor'][sim].zero_()
        self.lik['factor'][sim, :T, :Lm, :V].copy_(pair)

    def zero_lik(self):
        for k in ('ll', 'expected', 'g_ll', 'g_exp', 'logq', 'w'):
            self.lik[k].zero_()

    def lik_targets(self, t):
        """Per-target half of day t's likelihood (after edge_pass, before infect_claims)."""
        torch.ops.covgpu.lik_targets(self._sa, int(t), self.t['status'])

    def set_beta_tables(self, beta_sched, beta_layer_sched, sim=0):
        """Overwrite one sim's per-day beta tables in place (float64 schedules,
        rounded as at initialisation); captured graphs read the new values."""
        spec = self.specs[sim]
        spec.beta_sched = np.asarray(beta_sched, dtype=np.float64)
        spec.beta_layer_sched = np.asarray(beta_layer_sched, dtype=np.float64).reshape(spec.npts, len(spec.layers))
        bt = torch.from_numpy(spec.beta_table().ravel())
        bl = torch.from_numpy(spec.beta_layer_sched.astype(np.float32).ravel())
        b0 = sum(s.npts * s.nv for s in self.specs[:sim])
        l0 = sum(s.npts * len(s.layers) for s in self.specs[:sim])
        self.beta_tab[b0:b0 + bt.numel()].copy_(bt)
        self.beta_layer_tab[l0:l0 + bl.numel()].copy_(bl)

    # ------------------------------------------------------------------ kernels (torch.ops.covgpu.*)
    @property
    def _sa(self):
        """The ops' state argument: the address of the current covgpu_state descriptor."""
        return torch_ops.state_arg(self.cstate)

    def agent_step(self, t, do_prev=True, do_day=True, steady=False):
        """One agent pass (covgpu_agent_step); steady: a full pass of day t - 1 or
        earlier has run since the state was last changed outside the day kernels
        (as in a launch sequence), so warps of susceptible naive agents are skipped."""
        torch.ops.covgpu.agent_step(self._sa, int(t), bool(do_prev), bool(do_day), bool(steady), self.t['status'])

    def edge_pass(self, t, parts=0):
        """Day t's transmission: parts 0 both passes, 1 the stored layers only, 2 the
        dynamic layers only (the two are independent; a run launches both)."""
        if parts:
            self.cstate.edge_parts = int(parts)
        try:
            torch.ops.covgpu.edge_pass(self._sa, int(t), self.t['status'])
        finally:
            self.cstate.edge_parts = 0

    def infect_claims(self, t):
        torch.ops.covgpu.infect_claims(self._sa, int(t), self.t['status'])

    def test_trace(self, t):
        """Day t's testing, tracing and update_states_post (no-op without testing)."""
        torch.ops.covgpu.test_trace(self._sa, int(t), self.t['status'])

    def make_nonnaive(self, inds, sim=0):
        """people.py:414-431 make_nonnaive on agents still in their initial state:
        susceptible and naive cleared (local indices)."""
        inds = np.unique(np.asarray(inds, dtype=np.int64))
        if len(inds) == 0:
            return
        if inds.min() < 0 or inds.max() >= self.specs[sim].n:
            raise IndexError('agent index out of range')
        g = torch.from_numpy(inds + self.offsets[sim]).to(self.device)
        keep = ~((1 << STATE_BIT['susceptible']) | (1 << STATE_BIT['naive']))
        self.t['flags'][g] &= keep

    def import_day(self, t):
        """Day t's importations of every sim (sim.py:582-587; no-op without them)."""
        torch.ops.covgpu.import_day(self._sa, int(t), self.t['status'])

    def infect_list(self, t, inds, sim=0, variant=0, layer_tag=L.LOG_SEED, call_tag=1, sources=None,
                    want_infected=False):
        """Infect explicit agents of one sim (local indices; deduplicated and sorted
        here, the first occurrence's source kept, as people.py:465-468 does). With
        want_infected, returns (inds, mask of the agents actually infected) as
        device tensors; the susceptible alone are infected (people.py:470-474)."""
        inds, first = np.unique(np.asarray(inds, dtype=np.int64), return_index=True)
        if len(inds) == 0:
            return (inds, np.zeros(0, bool)) if want_infected else None
        if inds.min() < 0 or inds.max() >= self.specs[sim].n:
            raise IndexError('agent index out of range')
        g = _upload((inds + self.offsets[sim]).astype(np.int32), self.device)
        src = None
        if sources is not None:
            src = _upload(np.asarray(sources, dtype=np.int32)[first], self.device)
        infected = torch.empty(len(inds), dtype=torch.uint8, device=self.device) if want_infected else None
        self._keep_inds = (g, src)
        torch.ops.covgpu.infect_list(self._sa, int(t), g, src, int(sim), int(variant), int(layer_tag), int(call_tag),
                                     infected, self.t['status'])
        return (inds, infected) if want_infected else None

    def run_days(self, t0, t1, open_prev=False, close_last=True, use_graph=True):
        torch.ops.covgpu.run_days(self._sa, int(t0), int(t1), bool(open_prev), bool(close_last), bool(use_graph),
                                  self.t['status'])

    # ------------------------------------------------------------------ single functions of the day path
    def check(self, t, which, sim=0, filter_exposed=True, inds=None):
        """One of People.check_infectious ... check_death, check_exit_iso
        (people.py:222-312, 368-374; which: L.CHECK_*) at day t: applies it and
        returns (sorted local indices of the agents changed, known deaths)."""
        n = self.specs[sim].n
        ti = None
        if inds is not None:
            ti = torch.as_tensor(np.asarray(inds, dtype=np.int32)).to(self.device)
        out = torch.empty(max(n if ti is None else ti.numel(), 1), dtype=I32, device=self.device)
        counts = torch.zeros(2, dtype=I64, device=self.device)
        torch.ops.covgpu.check(self._sa, int(t), int(which), int(sim), bool(filter_exposed), ti, n, out, counts,
                               self.t['status'])
        c = counts.cpu().tolist()
        return torch.sort(out[:c[0]]).values, c[1]

    def check_immunity(self, t, sim=0, variants=None):
        """check_immunity (immunity.py:303-350) for the given variants (all if None)."""
        nv = self.specs[sim].nv
        mask = (1 << nv) - 1 if variants is None else sum(1 << int(v) for v in variants)
        torch.ops.covgpu.check_immunity(self._sa, int(t), int(sim), int(mask), self.t['status'])

    def update_nab(self, t, inds, sim=0):
        """update_nab (immunity.py:205-213) for local agents inds."""
        ti = torch.as_tensor(np.asarray(inds, dtype=np.int32)).to(self.device)
        if ti.numel():
            torch.ops.covgpu.update_nab(self._sa, int(t), int(sim), ti, self.t['status'])

    def update_peak_nab(self, t, inds, nab_init, nab_boost, norm_factor=1.0, symp_class=None, sim=0, call_tag=2):
        """update_peak_nab (immunity.py:138-202) for local agents inds: nab_init a
        distribution dict, symp_class per agent (0/1/2) or None for vaccine NAbs."""
        ti = torch.as_tensor(np.asarray(inds, dtype=np.int32)).to(self.device)
        if not ti.numel():
            return
        sc = None if symp_class is None else torch.as_tensor(np.asarray(symp_class, dtype=np.int8)).to(self.device)
        d = dur_par(nab_init)
        torch.ops.covgpu.update_peak_nab(self._sa, int(t), int(sim), ti, sc, int(d.code), float(d.a), float(d.b),
                                         float(nab_boost), float(norm_factor), int(call_tag), self.t['status'])

    def layer_lists(self, sim, layer, t, agents=None):
        """The day-t contact lists of a dynamic layer (covgpu_layer_lists): for the
        local agents ``agents`` (a range start, count pair, or None for all of the
        sim's agents) returns (counts [m, 2], offsets [2m + 1], partners) as device
        tensors; partners[offsets[2i + d]:offsets[2i + d + 1]] are the local
        partners of list d (0: the agent as p1, 1: as p2) of agent i."""
        seg = self.segment_index[(sim, layer)]
        if not self.segments[seg].dynamic:
            raise ValueError('layer_lists: the layer is not dynamic')
        begin, m = (0, self.specs[sim].n) if agents is None else (int(agents[0]), int(agents[1]))
        counts = torch.empty(2 * m, dtype=I32, device=self.device)
        torch.ops.covgpu.layer_lists(self._sa, int(seg), int(t), begin, m, counts, None, None, self.t['status'])
        offsets = torch.zeros(2 * m + 1, dtype=I64, device=self.device)
        torch.cumsum(counts.to(I64), 0, out=offsets[1:])
        partners = torch.empty(max(int(offsets[-1].item()), 1), dtype=I32, device=self.device)
        torch.ops.covgpu.layer_lists(self._sa, int(seg), int(t), begin, m, counts, offsets, partners,
                                     self.t['status'])
        return counts.view(m, 2), offsets, partners[:int(offsets[-1].item())]

    # ------------------------------------------------------------------ snapshots
    MUTABLE = ('flags', 'vstate', 'rel_trans', 'n_infections', 'n_breakthroughs', 'peak_nab', 'nab', 't_nab_event',
               'sus_imm', 'symp_imm', 'sev_imm', 'dates', 'durs', 'vaccine_source')

    def snapshot(self):
        """Device copy of every array a run modifies (restore() rewinds to it)."""
        keys = self.MUTABLE + (('pending_quar',) if self.has_testing else ())
        return {k: self.t[k].clone() for k in keys}

    def restore(self, snap):
        """Rewind to a snapshot: agent arrays, results, claims, counters and status."""
        for k, v in snap.items():
            self.t[k].copy_(v)
        self.res_int.zero_()
        self.res_var.zero_()
        self.res_fx.zero_()
        self.t['claim'].fill_(-1)
        self.t['roles'].zero_()
        self.t['viral_load'].zero_()
        self.t['event_count'].zero_()
        self.t['log_count'].zero_()
        self.t['status'].zero_()
        for a in self.import_variant:
            a[:] = 0
        self._reset_rescale()
        if self.has_testing:
            for k in ('trace_bits', 'contact_bits', 'trace_count'):
                self.t[k].zero_()
        self._refresh_state()

    def checkpoint(self, into=None):
        """Device copy of the state at a day boundary (with the results so far),
        for ``rewind``: recomputing from it reproduces the run exactly. ``into``:
        an earlier checkpoint of this state whose buffers are overwritten (no
        allocation)."""
        keys = self.MUTABLE + (('pending_quar',) if self.has_testing else ()) + ('log_count',)
        if into is not None:
            for k in keys:
                into[k].copy_(self.t[k])
            for dst, src in zip(into['_res'], (self.res_int, self.res_var, self.res_fx)):
                dst.copy_(src)
            for a, b in zip(into['_imp'], self.import_variant):
                a[:] = b
            return into
        ck = {k: self.t[k].clone() for k in keys}
        ck['_res'] = (self.res_int.clone(), self.res_var.clone(), self.res_fx.clone())
        ck['_imp'] = [a.copy() for a in self.import_variant]
        return ck

    def rewind(self, ck):
        """Return to a checkpoint (day-local buffers cleared, claims reset)."""
        for k, v in ck.items():
            if k not in ('_res', '_imp'):
                self.t[k].copy_(v)
        for a, b in zip(self.import_variant, ck['_imp']):
            a[:] = b
        for dst, src in zip((self.res_int, self.res_var, self.res_fx), ck['_res']):
            dst.copy_(src)
        self.t['claim'].fill_(-1)
        self.t['event_count'].zero_()
        self.t['status'].zero_()
        if self.has_testing:
            for k in ('trace_bits', 'contact_bits', 'trace_count'):
                self.t[k].zero_()

    def status(self):
        return int(self.t['status'].item())

    def clear_status(self):
        self.t['status'].zero_()

    # ------------------------------------------------------------------ accessors
    def sl(self, sim):
        off = self.offsets[sim]
        return slice(off, off + self.specs[sim].n)

    def flag(self, key, sim=0):
        bit = STATE_BIT[key]
        return ((self.t['flags'][self.sl(sim)] >> bit) & 1).bool()

    def by_variant(self, key, sim=0):
        shift = cvd.EXPOSED_BY_VARIANT_SHIFT if key == 'exposed_by_variant' else cvd.INFECTIOUS_BY_VARIANT_SHIFT
        f = self.t['flags'][self.sl(sim)]
        return torch.stack([((f >> (shift + v)) & 1).bool() for v in range(self.specs[sim].nv)])

    def variant_field(self, key, sim=0):
        shift = 8 * cvd.VARIANT_STATES.index(key)
        b = (self.t['vstate'][self.sl(sim)] >> shift) & 0xFF
        out = b.to(F32)
        out[b == L.NO_VARIANT] = float('nan')
        return out

    def get(self, key, sim=0):
        """One of the reference's People keys for one sim, as a torch tensor on the device."""
        s = self.sl(sim)
        if key in STATE_BIT:
            return self.flag(key, sim)
        if key in cvd.BY_VARIANT_STATES:
            return self.by_variant(key, sim)
        if key in cvd.VARIANT_STATES:
            return self.variant_field(key, sim)
        if key in cvd.DATES:
            return self.t['dates'][cvd.DATES.index(key), s]
        if key in cvd.DURS:
            return self.t['durs'][cvd.DURS.index(key), s]
        if key in cvd.IMM_STATES:
            return self.t[key][:self.specs[sim].nv, s]
        if key in self.t:
            return self.t[key][s]
        if key == 'uid':
            return torch.arange(self.specs[sim].n, dtype=I32, device=self.device)
        if key == 'doses':
            return torch.zeros(self.specs[sim].n, dtype=I32, device=self.device)
        raise KeyError(f'Key "{key}" is not a valid attribute of people')

    def set(self, key, values, sim=0):
        """Write one of the reference's People keys for one sim (host or device values)."""
        s = self.sl(sim)
        if key in STATE_BIT:
            bit = 1 << STATE_BIT[key]
            v = torch.as_tensor(np.asarray(values, dtype=bool) if not torch.is_tensor(values) else values,
                                device=self.device).to(torch.int32)
            f = self.t['flags'][s]
            f.copy_((f & ~bit) | (v * bit))
        elif key in cvd.BY_VARIANT_STATES:
            # bit 31 does not fit a signed int32 scalar: edit the words as uint32 on the host
            shift = cvd.EXPOSED_BY_VARIANT_SHIFT if key == 'exposed_by_variant' else cvd.INFECTIOUS_BY_VARIANT_SHIFT
            vals = np.asarray(values.cpu().numpy() if torch.is_tensor(values) else values, dtype=bool)
            f = self.t['flags'][s].cpu().numpy().view(np.uint32).copy()
            for v in range(vals.shape[0]):
                bit = np.uint32(1 << (shift + v))
                f = np.where(vals[v], f | bit, f & ~bit).astype(np.uint32)
            self.t['flags'][s].copy_(torch.from_numpy(f.view(np.int32)))
        elif key in cvd.VARIANT_STATES:
            shift = 8 * cvd.VARIANT_STATES.index(key)
            x = np.asarray(values, dtype=np.float64)
            b = np.where(np.isnan(x), L.NO_VARIANT, np.nan_to_num(x)).astype(np.int32)
            bt = torch.from_numpy(b).to(self.device)
            vs = self.t['vstate'][s]
            vs.copy_((vs & ~(0xFF << shift)) | (bt << shift))
        elif key in cvd.DATES:
            self.t['dates'][cvd.DATES.index(key), s].copy_(torch.as_tensor(np.asarray(values, np.float32)))
        elif key in cvd.DURS:
            self.t['durs'][cvd.DURS.index(key), s].copy_(torch.as_tensor(np.asarray(values, np.float32)))
        elif key in cvd.IMM_STATES:
            self.t[key][:self.specs[sim].nv, s].copy_(torch.as_tensor(np.asarray(values, np.float32)))
        elif key in self.t and key not in ('roles', 'claim', 'src_rec', 'events', 'log', 'status'):
            dst = self.t[key][s]
            dst.copy_(torch.as_tensor(np.asarray(values), dtype=dst.dtype))
            if key == 'rel_sus':  # the dynamic layers' thinning bound follows the largest rel_sus
                rs = _max_of(dst)
                for (k, _), seg in self.segment_index.items():
                    rec = self.segments[seg]
                    if k == sim and rec.dynamic:
                        rec.dyn_rse_max = rse_bound(rs, rec.quar_factor)
                self._tile_segments()
                self._refresh_state()
        else:
            raise KeyError(f'Key "{key}" cannot be set')

    def results(self, sim=0):
        """Per-day results of one sim as float64 numpy arrays, keyed like sim.results."""
        sp = self.specs[sim]
        ri, rv, rf = self.res_slices[sim]
        npts, nv = sp.npts, sp.nv
        ints = self.res_int[ri:ri + npts * L.N_RES_INT].view(npts, L.N_RES_INT).cpu().numpy().astype(np.float64)
        var = self.res_var[rv:rv + npts * L.N_RES_VAR * nv].view(npts, L.N_RES_VAR, nv).cpu().numpy().astype(np.float64)
        fx = self.res_fx[rf:rf + npts * L.N_RES_F].view(npts, L.N_RES_F).cpu().numpy()
        out = {}
        for k, key in enumerate(cvd.RES_INT_KEYS):
            out[key] = ints[:, k]
        out['n_imports'] = self.import_daily[sim] + self.import_variant[sim]
        out['_severe_now'] = ints[:, L.RES_SEVERE_NOW]
        out['_critical_now'] = ints[:, L.RES_CRITICAL_NOW]
        for k, key in enumerate(cvd.RES_VAR_KEYS):
            out[key] = var[:, k, :].T.copy()
        n_alive = sp.n - out['n_dead']
        with np.errstate(invalid='ignore', divide='ignore'):  # nobody alive: NaN, as sim.py:672 gives
            out['pop_nabs'] = np.ldexp(fx[:, 0].astype(np.float64), -L.FX_NAB_BITS) / n_alive
        denom = nv * sp.n
        out['pop_protection'] = np.ldexp(fx[:, 1].astype(np.float64), -L.FX_IMM_BITS) / denom
        out['pop_symp_protection'] = np.ldexp(fx[:, 2].astype(np.float64), -L.FX_IMM_BITS) / denom
        return out

    def infection_log_tensor(self, sim):
        """Device tensor [n, 5] int64 of sim's records (source, target, date, layer
        index, variant) in the order of ``infection_log``: two stable sorts
        (by target, then by day, variant and layer), as ``np.lexsort`` orders them."""
        dev = self.t['log'].device
        if not self.log_enabled:
            return torch.zeros((0, 5), dtype=torch.int64, device=dev)
        n = min(int(self.t['log_count'].item()), self.log_capacity)
        rec = self.t['log'][:n].long()
        packed = rec[:, 3]
        rec = rec[(packed >> 16) == sim]
        out = torch.stack([rec[:, 0], rec[:, 1], rec[:, 2], rec[:, 3] & 0xFF, (rec[:, 3] >> 8) & 0xFF], dim=1)
        out = out[torch.sort(out[:, 1], stable=True).indices]
        key = (out[:, 2] << 32) | (out[:, 4] << 16) | out[:, 3]
        return out[torch.sort(key, stable=True).indices]

    def infection_log(self, sim=None):
        """Infection-log records (source, target, date, layer index, variant), sorted like the reference's."""
        if not self.log_enabled:
            return np.zeros((0, 5), dtype=np.int64)
        n = min(int(self.t['log_count'].item()), self.log_capacity)
        rec = self.t['log'][:n].cpu().numpy().astype(np.int64)
        out = np.stack([rec[:, 0], rec[:, 1], rec[:, 2], rec[:, 3] & 0xFF, (rec[:, 3] >> 8) & 0xFF,
                        rec[:, 3] >> 16], axis=1)
        if sim is not None:
            out = out[out[:, 5] == sim]
        # the reference appends per infect() call: by day, variant, layer, then target
        order = np.lexsort((out[:, 1], out[:, 3], out[:, 4], out[:, 2], out[:, 5]))
        return out[order, :5]
