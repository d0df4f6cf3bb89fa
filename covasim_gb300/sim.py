"""``Sim``: the reference's cv.Sim interface with the day loop on the GPU.

``Sim(pars).run()`` builds the population on the host, uploads it once, and
runs every day on the device: the fused agent pass, the all-layer edge pass
and infect. With no host-side interventions the whole run is one CUDA graph
launch (``use_graph=True``). Follows covasim/sim.py:94-125 (initialize),
505-532 (seed infections), 558-685 (step), 688-761 (run), 764-870 (finalize).

Random numbers come from counter-based Philox streams keyed by the sim's seed,
so results are reproducible bit for bit, in any batch position, and agree
with the CPU oracle run in its Philox mode.
"""
import copy
import datetime as dt
import time

import numpy as np
import torch

from . import _lib as L
from . import defaults as cvd
from . import parameters as cvpar
from . import population as cvpop
from . import immunity as cvimm
from . import interventions as cvi
from . import analysis as cva
from .people import People, Layer, Contacts
from .state import SimSpec, BatchState

__all__ = ['Sim', 'Result', 'AlreadyRunError', 'choose_seed_infections', 'choose_nonnaive', 'init_infections',
           'build_spec']

SEED_INFECTION_TAG = 0x5EED
POPULATION_TAG = 0x9090
PROGNOSIS_TAG = 0x7070
CALL_SEED, CALL_IMPORT = 1, 2


class AlreadyRunError(RuntimeError):
    """sim.py:1550: the sim was asked to run past its end or to rerun."""


# ----------------------------------------------------------------------------- reporting
def yield_series(res):
    """sim.py:853-869 on result arrays: (test_yield, rel_test_yield)."""
    npts = len(res['new_tests'])
    ty = np.zeros(npts)
    rty = np.zeros(npts)
    inds = np.nonzero(res['new_tests'])[0]
    ty[inds] = res['new_diagnoses'][inds] / res['new_tests'][inds]
    inds = np.nonzero(res['n_infectious'])[0]
    denom = res['n_infectious'][inds] / (res['n_alive'][inds] - res['cum_diagnoses'][inds])
    rty[inds] = ty[inds] / denom
    return ty, rty


def doubling_series(cum, window=3, max_doubling_time=30):
    """sim.py:872-895."""
    cum = np.asarray(cum, dtype=float)
    now, prev = cum[window:], cum[:-window]
    use = (prev > 0) & (now > prev)
    out = np.full(len(cum), np.nan)
    out[window:][use] = np.minimum(window * np.log(2) / np.log(now[use] / prev[use]), max_doubling_time)
    return out


def mean_infectious_duration(d_rec, d_dead, d_inf):
    """sim.py:920-932: mean of the outcome dates minus mean of the infectious dates,
    over the agents with a recovery date then those with a death date (numpy
    arrays or device tensors; sums in float64)."""
    if torch.is_tensor(d_rec):  # masked sums on the device, one read-back
        m_rec, m_dead = ~torch.isnan(d_rec), ~torch.isnan(d_dead)
        zero = d_rec.new_zeros(())
        sums = torch.stack([m_rec.sum().double() + m_dead.sum().double(),
                            torch.where(m_rec, d_rec, zero).double().sum() +
                            torch.where(m_dead, d_dead, zero).double().sum(),
                            torch.where(m_rec, d_inf, zero).double().sum() +
                            torch.where(m_dead, d_inf, zero).double().sum()])
        n_out, s_out, s_inf = sums.tolist()
        if not n_out:
            return 0.0
    else:
        m_rec, m_dead = ~np.isnan(d_rec), ~np.isnan(d_dead)
        n_out = int(m_rec.sum() + m_dead.sum())
        if not n_out:
            return 0.0
        s_out = float(d_rec[m_rec].astype(np.float64).sum() + d_dead[m_dead].astype(np.float64).sum())
        s_inf = float(d_inf[m_rec].astype(np.float64).sum() + d_inf[m_dead].astype(np.float64).sum())
    return s_out / n_out - s_inf / n_out


def r_eff_daily(mean_inf, new_infections, n_imports, n_infectious, dur, smoothing=2):
    """sim.py:934-951: mean infectious duration x new infections / infectious, smoothed."""
    npts = len(new_infections)
    new_inf = np.asarray(new_infections, dtype=float) - np.asarray(n_imports, dtype=float)
    n_inf = np.asarray(n_infectious, dtype=float)
    raw = mean_inf * np.divide(new_inf, n_inf, out=np.zeros(npts), where=n_inf > 0)
    if len(raw) < 3:
        return raw
    initial = int(min(len(raw), dur['exp2inf']['par1'] + dur['asym2rec']['par1']))
    for ind in range(initial):
        raw[ind] = raw[ind:initial].mean()
    values = _smooth(raw, smoothing)
    values[:smoothing] = raw[:smoothing]
    values[-smoothing:] = raw[-smoothing:]
    return values


def r_eff_window(npts, day_arrays, log_sources, window=7):
    """sim.py:954-992: infections caused by the sources of each day (the day of
    becoming infectious, or of recovery/death), averaged over ``window`` days."""
    window = int(window)
    n = len(day_arrays[0])
    sources = np.zeros(npts)
    source_day = np.full(n, -1, dtype=np.int64)
    for t in range(npts):  # the last matching day wins, as in the reference's mapping
        for d in day_arrays:
            inds = np.nonzero(d == t)[0]
            sources[t] += len(inds)
            source_day[inds] = t
    src = np.asarray(log_sources, dtype=np.int64)
    src = src[src >= 0]
    sd = source_day[src]
    targets = np.bincount(sd[sd >= 0], minlength=npts).astype(float)[:npts]
    r = np.divide(targets, sources, out=np.full(npts, np.nan), where=sources > 0)
    num = np.nancumsum(r * sources)
    num[window:] = num[window:] - num[:-window]
    den = np.cumsum(sources)
    den[window:] = den[window:] - den[:-window]
    return np.divide(num, den, out=np.full(npts, np.nan), where=den > 0)


def gen_time(sources, targets, date_exposed, date_symptomatic):
    """sim.py:1004-1040 over the transmission records with a source."""
    sources = np.asarray(sources, dtype=np.int64)
    keep = sources >= 0
    src, tgt = sources[keep], np.asarray(targets, dtype=np.int64)[keep]
    i1 = (date_exposed[tgt] - date_exposed[src]).astype(np.float64)
    ok = np.isfinite(date_symptomatic[src]) & np.isfinite(date_symptomatic[tgt])
    i2 = (date_symptomatic[tgt][ok] - date_symptomatic[src][ok]).astype(np.float64)
    return {'true': np.mean(i1), 'true_std': np.std(i1), 'clinical': np.mean(i2), 'clinical_std': np.std(i2)}


def _smooth(data, repeats):
    """Smoothing used by compute_r_eff: ``repeats`` convolutions with the kernel
    [1/4, 1/2, 1/4] (same length). The reference calls ``sc.smooth`` of sciris
    (pinned 1.0.2, not in the reference tree); this is that published algorithm."""
    out = np.array(data, dtype=float)
    kernel = np.array([0.25, 0.5, 0.25])
    for _ in range(int(repeats)):
        out = np.convolve(out, kernel, mode='same')
    return out


class Result:
    """A per-day result series (covasim/base.py:117-193), array-like."""

    def __init__(self, name=None, npts=None, scale=True, values=None, n_variants=0):
        self.name = name
        self.scale = scale
        if values is None:
            shape = (n_variants, npts) if n_variants else (npts,)
            values = np.zeros(shape, dtype=cvd.result_float)
        self.values = np.asarray(values, dtype=cvd.result_float)

    def __getitem__(self, k):
        return self.values[k]

    def __setitem__(self, k, v):
        self.values[k] = v

    def __len__(self):
        return len(self.values)

    def __array__(self, dtype=None, copy=None):
        return self.values if dtype is None else self.values.astype(dtype)

    def __repr__(self):
        return f'Result({self.name}): {self.values!r}'

    @property
    def low(self):
        return getattr(self, '_low', None)


def choose_seed_infections(seed, n, k):
    """The agents infected on day 0 (sim.py:528-530): k distinct agents from a
    PCG64 stream keyed by the sim's seed."""
    rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, SEED_INFECTION_TAG]))
    return np.sort(rng.choice(int(n), size=int(k), replace=False)).astype(np.int64)


NONNAIVE_TAG = 0x4A4A


def choose_nonnaive(seed, n, frac_susceptible):
    """The agents made non-naive on day 0 when frac_susceptible < 1 (sim.py:519-522):
    round((1 - frac_susceptible) * n) distinct agents from a PCG64 stream keyed by
    (seed, 0x4A4A)."""
    k = int(np.round((1 - frac_susceptible) * n))
    rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, NONNAIVE_TAG]))
    return np.sort(rng.choice(int(n), size=k, replace=False)).astype(np.int64)


def variant_import_count(v, scale, rng):
    """immunity.py:121-124: a variant's importations on one of its days, n_imports
    over the day's scale (if the variant rescales) rounded at random (sciris'
    randround: floor(x + u); a whole number stays as it is and draws nothing)."""
    x = v.n_imports / (scale if getattr(v, 'rescale', True) else 1.0)
    return int(x) if x == int(x) else int(np.floor(x + rng.random()))


def init_infections(state, k, pars):
    """sim.py:505-532 for sim ``k`` of a batch on day 0: the non-susceptible
    fraction made non-naive (people.py:414-431), then the seed infections."""
    if pars['frac_susceptible'] < 1:
        state.make_nonnaive(choose_nonnaive(pars['rand_seed'], pars['pop_size'], pars['frac_susceptible']), sim=k)
    if pars['pop_infected']:
        inds = choose_seed_infections(pars['rand_seed'], pars['pop_size'], pars['pop_infected'])
        state.infect_list(0, inds, sim=k, variant=0, layer_tag=L.LOG_SEED, call_tag=CALL_SEED)
    state.count_nonnaive(k)


def _layers_from_popdict(pars, popdict):
    layers = []
    for lkey in pars['beta_layer'].keys():
        c = popdict['contacts'].get(lkey, dict(p1=np.zeros(0, np.int32), p2=np.zeros(0, np.int32)))
        if torch.is_tensor(c['p1']):  # device or pinned-host tensors: passed through (p1 must be sorted)
            layers.append(dict(key=lkey, p1=c['p1'], p2=c['p2'], beta=c.get('beta'),
                               dynamic=bool(pars['dynam_layer'].get(lkey, 0))))
            continue
        p1 = np.asarray(c['p1'], dtype=np.int32)
        p2 = np.asarray(c['p2'], dtype=np.int32)
        beta = np.asarray(c.get('beta', np.ones(len(p1))), dtype=np.float32)
        dyn = bool(pars['dynam_layer'].get(lkey, 0))
        if not dyn and len(p1) > 1 and np.any(p1[1:] < p1[:-1]):
            order = np.argsort(p1, kind='stable')
            p1, p2, beta = p1[order], p2[order], beta[order]
        layers.append(dict(key=lkey, p1=p1, p2=p2, beta=beta, dynamic=dyn))
    return layers


def build_spec(pars, popdict=None, person=None, interventions=None, gpu_population=False):
    """Population + prognoses + per-day tables of one sim -> (SimSpec, popdict, person).
    With ``gpu_population`` a missing population is built on the device."""
    seed = int(pars['rand_seed'])
    npts = int(pars['n_days']) + 1
    if popdict is None:
        if gpu_population:
            popdict = cvpop.make_randpop_device(pars, seed)
        else:
            popdict = cvpop.make_randpop(pars, rng=np.random.default_rng([seed, POPULATION_TAG]))
    if person is None:
        if gpu_population and popdict.get('_age_device') is not None:
            person = cvpop.set_prognoses_device(popdict['_age_device'], pars, seed)
        else:
            person = cvpop.set_prognoses(np.asarray(popdict['age']), pars,
                                         np.random.default_rng([seed, PROGNOSIS_TAG]))
    layers = _layers_from_popdict(pars, popdict)
    keys = [ly['key'] for ly in layers]
    betas = {'overall': pars['beta'], **{k: pars['beta_layer'][k] for k in keys}}
    beta_sched = np.zeros(npts)
    bl_sched = np.zeros((npts, len(keys)))
    for t in range(npts):
        for iv in interventions or []:
            if hasattr(iv, 'apply_day'):
                iv.apply_day(t, betas)
        beta_sched[t] = betas['overall']
        bl_sched[t] = [betas[k] for k in keys]
    testing = cvi.device_testing(interventions)
    return SimSpec(pars, person, layers, beta_sched, bl_sched, testing=testing), popdict, person


class Sim:
    """A Covasim simulation whose per-day step runs on the GPU.

    Args:
        pars (dict): parameters (see ``covasim_gb300.make_pars``); keyword
            arguments are merged in
        popdict (dict): optional population (uid, age, sex, contacts)
        use_graph (bool): capture the day loop in a CUDA graph
        edge_tile (int, str or 'auto'): edges per edge-pass tile (1024, 2048, 4096
            or 8192), suffixed 'w' ('2048w', the default) to run the stored layers'
            pass as one wave of blocks walking balanced ranges of tiles, or 'r'
            ('8192r') to keep the source bitmap resident in shared memory; 'auto'
            times whole runs with each at initialize (``covasim_gb300.autotune``,
            cached per workload)
        gpu_population (bool): build the population (ages, layers, prognoses) on
            the device instead of the host (same distributions, Philox draws)
        datafile (str, dict or DataTable): data to compare with (``cv.load_data``),
            used by ``compute_fit`` and ``Calibration``
    """

    def __init__(self, pars=None, label=None, popdict=None, use_graph=True, person=None, edge_tile=None,
                 gpu_population=False, datafile=None, data=None, **kwargs):
        self.label = label
        self.gpu_population = gpu_population  # build a missing population on the device
        self.edge_tile = edge_tile  # edges per edge-pass block; 'auto': autotuned at initialize
        self.pars = cvpar.make_pars()
        self.update_pars(pars, **kwargs)
        self.popdict = popdict
        if person is not None:
            self._person = person
        self.use_graph = use_graph
        self.people = None
        self.state = None
        self.t = None
        self.results = {}
        self.initialized = False
        self.complete = False
        self.results_ready = False
        self._event_capacity = None
        self._log_capacity = None
        self.datafile = datafile if datafile is not None else data
        self.data = None
        if self.datafile is not None:
            self.load_data(self.datafile)

    # ------------------------------------------------------------------ pars
    def __getitem__(self, key):
        return self.pars[key]

    def __setitem__(self, key, value):
        self.pars[key] = value

    def update_pars(self, pars=None, **kwargs):
        """sim.py:259-281."""
        pars = {**(pars or {}), **kwargs}
        if not pars:
            return
        for k1, k2 in dict(n_agents='pop_size', init_infected='pop_infected').items():
            if k1 in pars:
                pars[k2] = pars.pop(k1)
        if pars.get('pop_type'):
            cvpar.reset_layer_pars(pars, force=False)
        if pars.get('prog_by_age'):  # base.py:278-279: a truthy prog_by_age resets the prognoses
            pars['prognoses'] = cvpar.get_prognoses(by_age=pars['prog_by_age'])
        unknown = [k for k in pars if k not in self.pars]
        if unknown:
            raise KeyError(f'Key(s) {unknown} not found; available keys are {list(self.pars.keys())}')
        self.pars.update(pars)

    @property
    def npts(self):
        return int(self['n_days']) + 1

    @property
    def tvec(self):
        return np.arange(self.npts)

    def layer_keys(self):
        return list(self['beta_layer'].keys())

    # ------------------------------------------------------------------ dates and data (base.py:341-421)
    @property
    def datevec(self):
        """The date of each day of the sim."""
        start = cva.to_date(self['start_day'])
        return np.array([start + dt.timedelta(days=int(d)) for d in self.tvec], dtype=object)

    def day(self, day, *args):
        """Days since start_day of a date ('YYYY-MM-DD' or a date object); integers pass through."""
        days = [day] + list(args)
        out = [cva.to_day(d, self['start_day']) for d in days]
        return out[0] if len(out) == 1 else out

    def date(self, ind, *args, dateformat=None, as_date=False):
        """The date (a 'YYYY-MM-DD' string, or a date with ``as_date``) of sim day(s)."""
        inds = list(ind) if isinstance(ind, (list, tuple, np.ndarray)) else [ind] + list(args)
        start = cva.to_date(self['start_day'])
        out = []
        for i in inds:
            d = start + dt.timedelta(days=int(i)) if isinstance(i, (int, np.integer)) else cva.to_date(i)
            out.append(d if as_date else d.strftime(dateformat or '%Y-%m-%d'))
        return out[0] if len(out) == 1 and not isinstance(ind, (list, tuple, np.ndarray)) else out

    def load_data(self, datafile=None, verbose=False, **kwargs):
        """Attach data (misc.py:33-91) for ``compute_fit`` / ``Calibration``."""
        self.datafile = datafile
        self.data = cva.load_data(datafile, verbose=verbose, start_day=self['start_day'], **kwargs)
        return self.data

    def result_keys(self, which='main'):
        """Names of the per-day results (base.py:424-440)."""
        if which not in ('main', 'variant', 'all'):
            raise ValueError(f'Choice "{which}" not available; choices are main, variant, all')
        keys = []
        if which in ('main', 'all'):
            keys += [k for k, v in self.results.items() if isinstance(v, Result)]
        if which in ('variant', 'all') and 'variant' in self.results:
            keys += [k for k, v in self.results['variant'].items() if isinstance(v, Result)]
        return keys

    def compute_fit(self, *args, **kwargs):
        """The fit to the sim's data (sim.py:1086-1104); stored as ``sim.fit``."""
        self.fit = cva.Fit(self, *args, **kwargs)
        return self.fit

    def make_transtree(self, *args, output=True, **kwargs):
        """The transmission tree (sim.py:1107-1124), built on the device from the infection log."""
        tt = cva.TransTree(self, *args, **kwargs)
        if output:
            return tt
        self.results['transtree'] = tt
        return None

    def copy(self):
        """An unrun copy: its own parameters, the same population and data."""
        new = Sim(pars=None, label=self.label, popdict=self.popdict, use_graph=self.use_graph,
                  person=getattr(self, '_person', None), edge_tile=self.edge_tile,
                  gpu_population=self.gpu_population)
        new.pars = copy.deepcopy(self.pars)
        new.datafile, new.data = self.datafile, self.data
        return new

    # ------------------------------------------------------------------ initialize
    def validate_pars(self):
        p = self.pars
        p['pop_size'] = int(p['pop_size'])
        p['pop_infected'] = int(p['pop_infected'])
        if p.get('scaled_pop') is not None:  # sim.py:208-214
            if p['pop_scale'] in (None, 1, 1.0):
                p['pop_scale'] = p['scaled_pop'] / p['pop_size']
            else:
                p['pop_size'] = int(p['scaled_pop'] / p['pop_scale'])
        if p['pop_scale'] is None:
            p['pop_scale'] = 1
        if not 0 <= p['frac_susceptible'] <= 1:
            raise ValueError(f'frac_susceptible must be between 0 and 1, not {p["frac_susceptible"]}')
        if p['pop_infected'] > p['pop_size']:
            raise ValueError('pop_infected is larger than pop_size')
        for lp in cvpar.LAYER_PARS:
            if np.isscalar(p[lp]):
                p[lp] = {k: p[lp] for k in self.layer_keys()}

    def init_variants(self):
        """sim.py:477-495."""
        for v in self['variants']:
            if not isinstance(v, cvimm.variant):
                raise TypeError(f'Variant {v} is not a cv.variant object; please create using cv.variant()')
            if not v.initialized:
                v.initialize(self.pars)
        self['n_variants'] = len(self['variant_pars'])

    def init_interventions(self):
        self._host_interventions = []
        for iv in self['interventions']:
            if isinstance(iv, cvi.Intervention):
                iv.initialize(self)
                if not (hasattr(iv, 'apply_day') or hasattr(iv, 'device_testing')):
                    raise NotImplementedError(f'intervention {type(iv).__name__} is not supported on the GPU path yet')
            elif callable(iv):
                raise NotImplementedError('function interventions are not supported on the GPU path yet')

    def initialize(self, reset=False, **kwargs):
        """sim.py:94-125."""
        self.t = 0
        self.validate_pars()
        self.init_variants()
        if self['prognoses'] is None:
            self['prognoses'] = cvpar.get_prognoses(self['prog_by_age'])
        cvimm.init_immunity(self.pars, self.npts)
        self.init_results()
        self.init_interventions()
        spec, popdict, person = build_spec(self.pars, self.popdict, getattr(self, '_person', None),
                                           self['interventions'], gpu_population=self.gpu_population)
        self.popdict = popdict
        self._person = person
        self.spec = spec
        self.state = BatchState([spec], event_capacity=self._event_capacity, log_capacity=self._log_capacity)
        self.state.apply_edge_tile(self.edge_tile)
        contacts = Contacts()
        for ly in spec.layers:
            if torch.is_tensor(ly['p1']):
                contacts[ly['key']] = ly
            else:
                contacts[ly['key']] = Layer(ly['p1'], ly['p2'], ly['beta'], label=ly['key'])
        self.people = People(self.state, 0, self.pars, contacts)
        self.people['age'] = popdict['age']
        self.people['sex'] = popdict['sex']
        self._open_day = None     # day whose closing pass (stocks, update_nab) is pending
        self._seeded = False
        self.initialized = True
        self.complete = False
        self.results_ready = False
        return self

    def init_results(self):
        """sim.py:284-351 (the keys the GPU path fills)."""
        npts, nv = self.npts, self['n_variants']
        self.results = {}
        for key in cvd.result_flows:
            self.results[f'cum_{key}'] = Result(f'cum_{key}', npts)
            self.results[f'new_{key}'] = Result(f'new_{key}', npts)
        for key in cvd.result_stocks:
            self.results[f'n_{key}'] = Result(f'n_{key}', npts)
        for key in ('n_imports', 'n_alive', 'n_naive', 'n_preinfectious', 'n_removed', 'prevalence', 'incidence',
                    'frac_vaccinated', 'pop_nabs', 'pop_protection', 'pop_symp_protection', 'r_eff', 'doubling_time',
                    'test_yield', 'rel_test_yield'):
            self.results[key] = Result(key, npts)
        self.results['variant'] = {}
        for key in cvd.result_flows_by_variant:
            self.results['variant'][f'cum_{key}'] = Result(f'cum_{key}', npts, n_variants=nv)
            self.results['variant'][f'new_{key}'] = Result(f'new_{key}', npts, n_variants=nv)
        for key in cvd.result_stocks_by_variant:
            self.results['variant'][f'n_{key}'] = Result(f'n_{key}', npts, n_variants=nv)
        self.results['t'] = self.tvec
        self.results['date'] = self.datevec
        self.results_ready = False

    # ------------------------------------------------------------------ day loop
    def _seed(self):
        """sim.py:505-532: prior immunity and seed infections on day 0."""
        if not self._seeded:
            init_infections(self.state, 0, self.pars)
        self._seeded = True

    def _variant_days(self):
        days = set()
        for v in self['variants']:
            days.update(int(d) for d in np.atleast_1d(v.days))
        return days

    def _apply_variants(self, t):
        """immunity.py:117-130 variant.apply: import n_imports agents chosen among the susceptible."""
        for v in self['variants']:
            if t in np.atleast_1d(v.days):
                sus = np.nonzero(self.people['susceptible'])[0]
                rng = np.random.default_rng([int(self['rand_seed']), 0x1A1A, t, v.index])
                n_imp = variant_import_count(v, self.state.rescale_vecs[0][t], rng)  # more than len(sus): ValueError, as immunity.py:128
                inds = rng.choice(sus, n_imp, replace=False)
                self.state.set_hospicu([[0, 0]])  # variant.apply calls infect() without bed limits
                self.state.infect_list(t, inds, sim=0, variant=v.index, layer_tag=L.LOG_IMPORT,
                                       call_tag=CALL_IMPORT + v.index)
                self.state.set_hospicu(None)
                self.state.note_imports(0, t, n_imp)

    def step(self):
        """One day (sim.py:558-685), then that day's closing pass."""
        if not self.initialized:
            self.initialize()
        if self.complete:
            raise AlreadyRunError('Simulation already complete (call sim.initialize() to re-run)')
        t = self.t
        if t == 0:
            self._seed()
        self.state.rescale_day(t)  # sim.py:575, before update_states_pre
        self.people.__dict__['t'] = t
        self.state.agent_step(t, do_prev=self._open_day is not None, do_day=True)
        self.state.import_day(t)  # sim.py:582-587, then the variants' importations (sim.py:590-592)
        self._apply_variants(t)
        self.state.test_trace(t)  # sim.py:596-600 interventions after importations, then update_states_post
        self.state.edge_pass(t)
        self.state.infect_claims(t)
        self.state.agent_step(t + 1, do_prev=True, do_day=False)
        self._open_day = None
        self.t += 1
        if self.t == self.npts:
            self.complete = True

    def run(self, do_plot=False, until=None, restore_pars=True, reset_seed=True, verbose=None, use_graph=None):
        """sim.py:688-761: run to ``until`` (default: the end) and finalize."""
        if not self.initialized:
            self.initialize()
        until = self.npts if until is None else int(until)
        if until > self.npts:
            raise AlreadyRunError(f'Requested to run until t={until} but the simulation end is t={self.npts}')
        if self.t >= until:
            raise AlreadyRunError(f'Simulation is currently at t={self.t}, requested to run until t={until} '
                                  'which has already been reached')
        if self.complete:
            raise AlreadyRunError('Simulation is already complete (call sim.initialize() to re-run)')
        use_graph = self.use_graph if use_graph is None else use_graph
        T = time.perf_counter()
        host_days = sorted(d for d in self._variant_days() if self.t <= d < until)
        if self.t == 0:
            self._seed()
        while self.t < until:
            if self['timelimit'] and time.perf_counter() - T > self['timelimit']:
                break
            if self['stopping_func'] and self['stopping_func'](self):
                break
            nxt = next((d for d in host_days if d >= self.t), until)
            if nxt > self.t:  # days without host work: one fused launch sequence (or graph)
                self.state.run_days(self.t, nxt, close_last=True, use_graph=use_graph)
                held = self.state.held_day()
                if held is not None and held < nxt:  # a rescaling fell due: do it, go on from that day
                    self.state.rescale_day(held)
                    self.t = held
                    continue
                self.t = nxt
            if self.t < until and self.t == nxt:  # a day with host work
                self.step()
        if self.t >= self.npts:
            self.complete = True
        status = self.state.status()
        if status:
            if status & L.OVERFLOW:
                return self._rerun_bigger(until)
            raise L.CovgpuError('device status', status)
        if self.complete:
            self.finalize()
        return self

    def rewind(self, snap):
        """Return an initialised sim to day 0 from ``state.snapshot()`` taken before
        its first run (device copy, no population rebuild), ready to run again."""
        self.state.restore(snap)
        self.t = 0
        self._seeded = False
        self._open_day = None
        self.complete = False
        self.results_ready = False
        self.init_results()
        return self

    def _rerun_bigger(self, until):
        """A fixed-capacity device buffer overflowed: the run is deterministic, so
        redo it from the start with twice the capacity."""
        self._event_capacity = 2 * self.state.event_capacity
        self._log_capacity = 2 * max(self.state.log_capacity, 1)
        self.initialize()
        return self.run(until=until)

    # ------------------------------------------------------------------ results
    def finalize(self, verbose=None, restore_pars=True):
        """sim.py:764-815 (no rescaling on the GPU path)."""
        if self.results_ready:
            raise AlreadyRunError('Simulation has already been finalized')
        self._fill_results(self.state.results(0), self.state.rescale_vecs[0])
        self.results_ready = True
        self.t -= 1
        self.people.__dict__['t'] = self.t
        self.compute_results()
        self.summary = {k: v.values[-1] for k, v in self.results.items() if isinstance(v, Result)}
        return self

    UNSCALED = ('prevalence', 'incidence', 'r_eff', 'doubling_time', 'test_yield', 'rel_test_yield',
                'frac_vaccinated', 'pop_nabs', 'pop_protection', 'pop_symp_protection', 'prevalence_by_variant',
                'incidence_by_variant')

    def _fill_results(self, res, rescale_vec):
        """sim.py:771-787: the device's per-day counts, scaled by each day's scale
        (the results that count people), their cumulative sums, and the seed
        infections at day 0's scale."""
        self.rescale_vec = np.array(rescale_vec, dtype=np.float64)
        for key, vals in res.items():
            if key.startswith('_'):
                continue
            scale = 1.0 if key in self.UNSCALED else self.rescale_vec
            if key in self.results['variant']:
                self.results['variant'][key].values[:] = vals * scale
            elif key in self.results:
                self.results[key].values[:] = vals * scale
        for key in cvd.result_flows:
            self.results[f'cum_{key}'].values[:] = np.cumsum(self.results[f'new_{key}'].values)
        for key in cvd.result_flows_by_variant:
            self.results['variant'][f'cum_{key}'].values[:] = np.cumsum(self.results['variant'][f'new_{key}'].values,
                                                                        axis=1)
        self.results['cum_infections'].values += self['pop_infected'] * self.rescale_vec[0]
        self.results['variant']['cum_infections_by_variant'].values[0] += self['pop_infected'] * self.rescale_vec[0]

    @property
    def scaled_pop_size(self):
        """base.py:316-321: agents times the scale factor."""
        return self['pop_size'] * self['pop_scale']

    def compute_results(self):
        """sim.py:818-825 (the summary is formed by finalize)."""
        self.compute_states()
        self.compute_yield()
        self.compute_doubling()
        self.compute_r_eff()

    def compute_states(self):
        """sim.py:828-850."""
        res = self.results
        count_recov = 1 - self['use_waning']
        n = self.scaled_pop_size
        res['n_alive'].values[:] = n - res['cum_deaths'].values
        res['n_naive'].values[:] = n - res['cum_deaths'].values - res['n_recovered'].values - res['n_exposed'].values
        res['n_susceptible'].values[:] = res['n_alive'].values - res['n_exposed'].values - count_recov * res['cum_recoveries'].values
        res['n_preinfectious'].values[:] = res['n_exposed'].values - res['n_infectious'].values
        res['n_removed'].values[:] = count_recov * res['cum_recoveries'].values + res['cum_deaths'].values
        with np.errstate(divide='ignore', invalid='ignore'):
            res['prevalence'].values[:] = res['n_exposed'].values / res['n_alive'].values
            res['incidence'].values[:] = res['new_infections'].values / res['n_susceptible'].values
            res['frac_vaccinated'].values[:] = res['n_vaccinated'].values / res['n_alive'].values

    def compute_yield(self):
        """sim.py:853-869: test positivity and its ratio to the prevalence among the undiagnosed."""
        res = self.results
        ty, rty = yield_series({k: res[k].values for k in ('new_tests', 'new_diagnoses', 'n_infectious', 'n_alive',
                                                            'cum_diagnoses')})
        res['test_yield'].values[:] = ty
        res['rel_test_yield'].values[:] = rty

    def compute_doubling(self, window=3, max_doubling_time=30):
        """sim.py:872-895: doubling time of cumulative infections over ``window`` days."""
        self.results['doubling_time'].values[:] = doubling_series(self.results['cum_infections'].values, window,
                                                                  max_doubling_time)
        return self.results['doubling_time'].values

    def compute_r_eff(self, method='daily', smoothing=2, window=7):
        """sim.py:898-1001: effective reproduction number (methods 'daily',
        'infectious', 'outcome'); the date means and day counts come from the
        device arrays."""
        res = self.results
        if method == 'daily':
            g = self.people.gpu
            mean_inf = mean_infectious_duration(g('date_recovered'), g('date_dead'), g('date_infectious'))
            values = r_eff_daily(mean_inf, res['new_infections'].values, res['n_imports'].values,
                                 res['n_infectious'].values, self['dur'], smoothing)
        elif method in ('infectious', 'outcome'):
            keys = ['date_infectious'] if method == 'infectious' else ['date_recovered', 'date_dead']
            log = self.state.infection_log(0)
            values = r_eff_window(self.npts, [self.people[k] for k in keys], log[:, 0], window)
        else:
            raise ValueError(f'Method must be "daily", "infectious", or "outcome", not "{method}"')
        res['r_eff'].values[:] = values
        return res['r_eff'].values

    def compute_gen_time(self):
        """sim.py:1004-1040: mean and sd of the exposure-to-exposure and
        symptom-to-symptom intervals over the transmission log."""
        log = self.state.infection_log(0)
        self.results['gen_time'] = gen_time(log[:, 0], log[:, 1], self.people['date_exposed'],
                                            self.people['date_symptomatic'])
        return self.results['gen_time']

    def raw_results(self):
        """Per-day device results before finalize's post-processing (stocks as counted)."""
        return self.state.results(0)

    def infection_log(self):
        return self.people.infection_log
