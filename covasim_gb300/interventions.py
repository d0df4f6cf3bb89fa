"""Interventions that the GPU day loop consumes as device tables.

``change_beta`` (covasim/interventions.py:530-586) changes the overall beta or a
layer's beta from given days on. On the GPU path its effect is folded into the
per-day beta tables before the run, so the whole day loop can be captured in a
CUDA graph without a host round trip per day.

``test_prob`` (interventions.py:858-981) and ``contact_tracing``
(interventions.py:984-1145) become the sim's testing record: thresholds and
day ranges that the testing, tracing and post passes of the library read
every day, again with no host round trip.
"""
import numbers

import numpy as np

from . import _lib as L

__all__ = ['Intervention', 'change_beta', 'test_prob', 'contact_tracing']


class Intervention:
    """Base class (interventions.py:223-410): ``initialize(sim)`` then ``apply(sim)`` per day.

    Subclasses that only change per-day parameters implement ``apply_day(t, betas)``,
    which the GPU sim folds into its per-day tables; other interventions are
    called on the host between the agent pass and the transmission pass.
    """

    def __init__(self, label=None, show_label=False, do_plot=None, line_args=None):
        self.label = label or self.__class__.__name__
        self.show_label = show_label
        self.do_plot = do_plot if do_plot is not None else True
        self.days = []
        self.initialized = False
        self.finalized = False

    def initialize(self, sim=None):
        self.initialized = True

    def finalize(self, sim=None):
        self.finalized = True

    def apply(self, sim):
        raise NotImplementedError

    def __call__(self, *args, **kwargs):
        if not self.initialized:
            raise RuntimeError(f'Intervention (label={self.label}, {type(self)}) has not been initialized')
        return self.apply(*args, **kwargs)


def _process_days(days):
    if not isinstance(days, (list, tuple, np.ndarray)):
        days = [days]
    return np.sort(np.asarray(days, dtype=int))


def _process_changes(changes, days):
    if not isinstance(changes, (list, tuple, np.ndarray)):
        changes = [changes] * len(days)
    changes = np.asarray(changes, dtype=float)
    if len(changes) != len(days):
        raise ValueError(f'Number of days supplied ({len(days)}) does not match number of changes ({len(changes)})')
    return changes


class change_beta(Intervention):
    """Multiply beta (or layer betas) by ``changes[i]`` from ``days[i]`` on (interventions.py:530-586).

    The multiplier applies to the beta the sim had at initialisation, as in
    the reference.
    """

    def __init__(self, days, changes, layers=None, **kwargs):
        super().__init__(**kwargs)
        self.days = days
        self.changes = changes
        self.layers = layers
        self.orig_betas = None

    def initialize(self, sim):
        super().initialize()
        self.days = _process_days(self.days)
        self.changes = _process_changes(self.changes, self.days)
        layers = self.layers
        self.layers = [layers] if (layers is None or isinstance(layers, str)) else list(layers)
        self.orig_betas = {}
        for lkey in self.layers:
            if lkey is None:
                self.orig_betas['overall'] = sim['beta']
            else:
                self.orig_betas[lkey] = sim['beta_layer'][lkey]

    def apply_day(self, t, betas):
        """Day-t effect on ``betas`` = {'overall': beta, layer key: beta_layer} (in place)."""
        for ind in np.nonzero(self.days == t)[0]:
            for lkey, orig in self.orig_betas.items():
                betas[lkey] = orig * self.changes[ind]

    def apply(self, sim):
        betas = {'overall': sim['beta'], **sim['beta_layer']}
        self.apply_day(sim.t, betas)
        sim['beta'] = betas.pop('overall')
        sim['beta_layer'].update(betas)


def _day(d, default):
    """interventions.py:56-65 preprocess_day for integer days (None keeps the default)."""
    if d is None:
        return default
    if callable(d) or isinstance(d, str):
        raise NotImplementedError('intervention days must be integers on the GPU path')
    return int(d)


class test_prob(Intervention):
    """Test each agent with a probability set by its symptom and quarantine state
    (interventions.py:858-981). Same arguments as the reference: ``swab_delay`` a
    dict of ``dist`` ('uniform' or 'lognormal'), ``par1`` and ``par2`` (get_pdf,
    utils.py:240-268), ``ili_prev`` a number or a daily sequence
    (process_daily_data, interventions.py:111-147), ``subtarget`` a dict of fixed
    ``inds`` and ``vals`` (get_subtargets, interventions.py:150-187; functions of
    the sim are not supported on the GPU path).
    """

    def __init__(self, symp_prob, asymp_prob=0.0, symp_quar_prob=None, asymp_quar_prob=None, quar_policy=None,
                 subtarget=None, ili_prev=None, sensitivity=1.0, loss_prob=0.0, test_delay=0, start_day=0,
                 end_day=None, swab_delay=None, **kwargs):
        super().__init__(**kwargs)
        self.symp_prob = symp_prob
        self.asymp_prob = asymp_prob
        self.symp_quar_prob = symp_quar_prob if symp_quar_prob is not None else symp_prob
        self.asymp_quar_prob = asymp_quar_prob if asymp_quar_prob is not None else asymp_prob
        self.quar_policy = quar_policy if quar_policy else 'start'
        self.subtarget = subtarget
        self.ili_prev = ili_prev
        self.sensitivity = sensitivity
        self.loss_prob = loss_prob
        self.test_delay = test_delay
        self.start_day = start_day
        self.end_day = end_day
        self.swab_delay = swab_delay

    def initialize(self, sim):
        super().initialize()
        self.start_day = _day(self.start_day, 0)
        self.end_day = _day(self.end_day, None)
        self.days = [self.start_day, self.end_day]
        self._subtarget = self._fixed_subtarget(self.subtarget, sim['pop_size'])
        self._ili = self._daily(self.ili_prev, sim.npts)
        self._swab_pdf = self._swab_table(self.swab_delay, sim.npts)

    @staticmethod
    def _swab_table(swab_delay, npts):
        """The density of the delay from symptom onset to swab (get_pdf, utils.py:240-268:
        uniform, or lognormal of the given mean and variance) at 0 .. npts days, or None."""
        d = dict(swab_delay or {})
        dist, par1, par2 = d.get('dist'), d.get('par1'), d.get('par2')
        if dist in ('None', 'none', None):
            return None
        import scipy.stats as sps
        if dist == 'uniform':
            pdf = sps.uniform(loc=par1, scale=par2)
        elif dist == 'lognormal':
            mean = np.log(par1**2 / np.sqrt(par2 + par1**2))
            sigma = np.sqrt(np.log(par2 / par1**2 + 1))
            pdf = sps.lognorm(sigma, loc=-0.5, scale=np.exp(mean))
        else:
            raise NotImplementedError(f'The selected distribution "{dist}" is not implemented; choices are: none, '
                                      'uniform, lognormal')
        return np.asarray(pdf.pdf(np.arange(npts + 1, dtype=np.int32)), dtype=np.float64)

    @staticmethod
    def _fixed_subtarget(st, n):
        """get_subtargets (interventions.py:150-187) for fixed indices and values."""
        if st is None:
            return None
        if callable(st) or (isinstance(st, dict) and (callable(st.get('inds')) or callable(st.get('vals')))):
            raise NotImplementedError('subtargets given as functions of the sim are not supported on the GPU path')
        if not isinstance(st, dict) or 'inds' not in st:
            raise ValueError(f'The subtarget dict must have keys "inds" and "vals", but you supplied {st}')
        inds = np.asarray(st['inds'], dtype=np.int64).ravel()
        vals = st['vals']
        if np.ndim(vals) == 0:
            vals = np.full(len(inds), float(vals))
        else:
            vals = np.asarray(vals, dtype=np.float64).ravel()
            if len(vals) != len(inds):
                raise ValueError(f'Length of subtargeting indices ({len(inds)}) does not match length of values '
                                 f'({len(vals)})')
        if len(inds) and (inds.min() < 0 or inds.max() >= n):
            raise ValueError('subtarget indices must be agents of the sim')
        return inds, vals

    @staticmethod
    def _daily(x, npts):
        """process_daily_data (interventions.py:111-147) for a number or a sequence."""
        if x is None:
            return None
        if isinstance(x, numbers.Number):
            return np.array([float(x)] * npts)
        if isinstance(x, str) or not hasattr(x, '__len__'):
            raise NotImplementedError('ili_prev from data columns or dataframes is not supported on the GPU path')
        return np.asarray(x, dtype=np.float64).ravel()

    @staticmethod
    def _quar_policy(qp):
        """interventions.py:682-710 -> (COVGPU_QP_* bits, offset bits)."""
        named = {'start': L.QP_START, 'end': L.QP_END, 'both': L.QP_START | L.QP_END, 'daily': L.QP_DAILY}
        if qp is None:
            return 0, 0
        if isinstance(qp, str):
            if qp not in named:
                raise ValueError(f'Quarantine policy "{qp}" not recognized')
            return named[qp], 0
        if callable(qp):
            raise NotImplementedError('function quarantine policies are not supported on the GPU path')
        offs = 0
        for q in np.atleast_1d(qp):
            if float(q) != int(q) or not 0 <= int(q) < 32:
                raise NotImplementedError('numeric quarantine policies must be integers in [0, 32)')
            offs |= 1 << int(q)
        return L.QP_OFFSETS, offs

    def device_testing(self):
        qp, offs = self._quar_policy(self.quar_policy)
        if float(self.test_delay) != int(self.test_delay):
            raise NotImplementedError('test_delay must be a whole number of days on the GPU path')
        return dict(start_day=self.start_day, end_day=0xFFFE if self.end_day is None else self.end_day,
                    quar_policy=qp, quar_offsets=offs, symp_prob=float(self.symp_prob),
                    asymp_prob=float(self.asymp_prob), symp_quar_prob=float(self.symp_quar_prob),
                    asymp_quar_prob=float(self.asymp_quar_prob), sensitivity=float(self.sensitivity),
                    loss_prob=float(self.loss_prob), test_delay=int(self.test_delay),
                    subtarget=getattr(self, '_subtarget', None), ili_prev=getattr(self, '_ili', None),
                    swab_pdf=getattr(self, '_swab_pdf', None))

    def apply(self, sim):
        raise NotImplementedError('test_prob runs on the device as part of the day loop')


class contact_tracing(Intervention):
    """Trace the contacts of the diagnosed (interventions.py:984-1145). Same
    arguments as the reference.
    """

    def __init__(self, trace_probs=None, trace_time=None, start_day=0, end_day=None, presumptive=False,
                 quar_period=None, capacity=None, **kwargs):
        super().__init__(**kwargs)
        self.trace_probs = trace_probs
        self.trace_time = trace_time
        self.start_day = start_day
        self.end_day = end_day
        self.presumptive = presumptive
        self.capacity = capacity
        self.quar_period = quar_period

    def initialize(self, sim):
        """interventions.py:1023-1041."""
        super().initialize()
        if self.capacity is not None and not isinstance(self.capacity, numbers.Number):
            raise ValueError('contact_tracing capacity must be a number')
        self.start_day = _day(self.start_day, 0)
        self.end_day = _day(self.end_day, None)
        self.days = [self.start_day, self.end_day]
        if self.trace_probs is None:
            self.trace_probs = 1.0
        if self.trace_time is None:
            self.trace_time = 0.0
        if self.quar_period is None:
            self.quar_period = sim['quar_period']
        keys = sim.layer_keys()
        if isinstance(self.trace_probs, numbers.Number):
            self.trace_probs = {k: self.trace_probs for k in keys}
        if isinstance(self.trace_time, numbers.Number):
            self.trace_time = {k: self.trace_time for k in keys}

    def device_testing(self):
        return dict(start_day=self.start_day, end_day=0xFFFE if self.end_day is None else self.end_day,
                    presumptive=bool(self.presumptive), trace_probs=dict(self.trace_probs),
                    trace_time=dict(self.trace_time), quar_period=self.quar_period,
                    capacity=None if self.capacity is None else float(self.capacity))

    def apply(self, sim):
        raise NotImplementedError('contact_tracing runs on the device as part of the day loop')


def device_testing(interventions):
    """The sim's testing record from its interventions (None without testing)."""
    test = trace = None
    for iv in interventions or []:
        if isinstance(iv, test_prob):
            if test is not None:
                raise NotImplementedError('one test_prob per sim is supported on the GPU path')
            test = iv.device_testing()
        elif isinstance(iv, contact_tracing):
            if trace is not None:
                raise NotImplementedError('one contact_tracing per sim is supported on the GPU path')
            if test is None and any(isinstance(j, test_prob) for j in interventions):
                raise NotImplementedError('contact_tracing must follow test_prob in the interventions list')
            trace = iv.device_testing()
    if test is None and trace is None:
        return None
    return {'test': test, 'trace': trace}
