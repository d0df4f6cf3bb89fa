"""NAb kinetics and cross-immunity tables (host side, O(n_days) and O(nv^2)).

The per-agent NAb and immunity work (check_immunity, update_nab,
update_peak_nab) runs in the CUDA agent and infect kernels; this module
builds the tables they read: ``nab_kin`` (covasim/immunity.py:356-448) and the
cross-immunity matrix (immunity.py:269-300). ``check_immunity``,
``update_nab`` and ``update_peak_nab`` are also drop-ins with the reference's
signatures, each one CUDA kernel over a People object's agents.
"""
import numpy as np

from . import defaults as cvd
from . import parameters as cvpar

__all__ = ['nab_growth_decay', 'nab_decay', 'exp_decay', 'precompute_waning', 'init_immunity', 'variant',
           'check_immunity', 'update_nab', 'update_peak_nab']


# ---------------------------------------------------------------- reference-signature drop-ins
def check_immunity(people, variants=None):
    """immunity.py:303-350: each agent's sus_imm, symp_imm and sev_imm for the
    given variants (all if None) from its NAbs and the larger of its natural
    and vaccine immunity, on the device (calc_VE in float-float arithmetic,
    rounded once, as the reference's float64)."""
    people._state.check_immunity(people.t, sim=people._sim, variants=variants)


def update_nab(people, inds):
    """immunity.py:205-213: nab += nab_kin[t - t_nab_event] * peak_nab for the
    agents inds, clamped to [0, peak_nab], on the device."""
    people._state.update_nab(people.t, np.asarray(inds), sim=people._sim)


def update_peak_nab(people, inds, nab_pars, symp=None):
    """immunity.py:138-202 on the device: agents with NAbs have their peak
    boosted by nab_pars['nab_boost']; the others get 2 ** nab_init, scaled by the
    symptom class's rel_imm_symp and 1 + nab_eff['alpha_inf_diff'] when symp
    (a dict of 'asymp', 'mild' and 'sev' index arrays) is given; t_nab_event = t.
    The initial levels are drawn from the library's Philox streams."""
    inds = np.asarray(inds, dtype=np.int64)
    if not len(inds):
        return
    no_prior = ~(people['nab'][inds] > 0)
    if no_prior.any() and nab_pars.get('nab_init') is None:
        raise ValueError(f'Attempt to administer a vaccine without an initial NAb distribution to '
                         f'{int(no_prior.sum())} unvaccinated people failed.')
    cls, norm = None, 1.0
    if symp is not None:
        cls = np.full(len(inds), -1, dtype=np.int8)
        for c, key in enumerate(('asymp', 'mild', 'sev')):
            cls[np.isin(inds, np.asarray(symp.get(key, []), dtype=np.int64))] = c
        if np.any(cls[no_prior] < 0):
            raise ValueError('update_peak_nab: every agent without NAbs must be in one of symp\'s lists')
        norm = 1 + nab_pars['nab_eff']['alpha_inf_diff']
    init = nab_pars.get('nab_init') or dict(dist='normal', par1=0, par2=1)
    people._state.update_peak_nab(people.t, inds, init, nab_pars['nab_boost'], norm_factor=norm, symp_class=cls,
                                  sim=people._sim)


def nab_growth_decay(length, growth_time, decay_rate1, decay_time1, decay_rate2, decay_time2):
    """immunity.py:406-448: linear growth then exponential decay whose rate falls linearly."""
    if decay_time2 < decay_time1:
        raise ValueError(f'Decay time 2 must be larger than decay time 1, but you supplied {decay_time2} '
                         f'which is smaller than {decay_time1}.')
    length = length + 1
    t1 = np.arange(growth_time, dtype=cvd.default_int)
    t2 = np.arange(length - growth_time, dtype=cvd.default_int)
    y1 = (1 / growth_time) * t1
    rate = np.full(len(t2), fill_value=decay_rate1)
    rate[np.nonzero(t2 > decay_time2)[0]] = decay_rate2
    slowing = (1 / (decay_time2 - decay_time1)) * (decay_rate1 - decay_rate2)
    mid = np.nonzero((t2 > decay_time1) * (t2 <= decay_time2))[0]
    rate[mid] = decay_rate1 - slowing * np.arange(len(mid), dtype=cvd.default_int)
    titre = np.zeros(len(t2))
    # a running sum from index 1, element by element in float64 (as the reference's loop)
    for i in range(1, len(t2)):
        titre[i] = titre[i - 1] + rate[i]
    y2 = np.exp(-titre)
    y = np.concatenate([y1, y2])
    return np.diff(y)[0:length]


def nab_decay(length, decay_rate1, decay_time1, decay_rate2):
    """immunity.py:451-479: exponential decay whose rate itself decays after decay_time1."""
    t = np.arange(length, dtype=cvd.default_int)
    ta = np.nonzero(t <= decay_time1)[0]
    tb = np.nonzero(t > decay_time1)[0]
    y1 = np.exp(-ta * decay_rate1)
    y2 = np.exp(-tb * (decay_rate1 * np.exp(-(tb - decay_time1) * decay_rate2)))
    y = np.diff(np.concatenate([[-np.inf], y1, y2]))[0:length]
    y[0] = 1
    return y


def exp_decay(length, init_val, half_life, delay=None):
    """immunity.py:482-495: exponential decay, optionally after a linear ramp of ``delay`` days."""
    length = length + 1
    decay_rate = np.log(2) / half_life if ~np.isnan(half_life) else 0.
    if delay is not None:
        t = np.arange(length - delay, dtype=cvd.default_int)
        growth = (init_val / delay) * np.ones(delay)
        result = np.concatenate([growth, init_val * np.exp(-decay_rate * t)], axis=None)
    else:
        t = np.arange(length, dtype=cvd.default_int)
        result = init_val * np.exp(-decay_rate * t)
    return np.diff(result)


def precompute_waning(length, pars=None):
    """immunity.py:356-403."""
    pars = dict(pars)
    form = pars.pop('form')
    if form is None or form == 'nab_growth_decay':
        return nab_growth_decay(length, **pars)
    if form == 'nab_decay':
        return nab_decay(length, **pars)
    if form == 'exp_decay':
        if pars['half_life'] is None:
            pars['half_life'] = np.nan
        return exp_decay(length, **pars)
    if callable(form):
        return form(length, **pars)
    raise NotImplementedError(f'The selected functional form "{form}" is not implemented')


def init_immunity(pars, npts, create=False):
    """immunity.py:269-300: cross-immunity matrix and nab_kin for a sim of npts points."""
    if not pars['use_waning']:
        return pars
    nv = pars['n_variants']
    if pars['immunity'] is None or create:
        immunity = np.ones((nv, nv), dtype=cvd.default_float)
        cross = cvpar.get_cross_immunity()
        for i in range(nv):
            li = pars['variant_map'][i]
            for j in range(nv):
                lj = pars['variant_map'][j]
                if li in cross and lj in cross:
                    immunity[j][i] = cross[lj][li]
        pars['immunity'] = immunity
    pars['nab_kin'] = precompute_waning(length=npts, pars=pars['nab_decay'])
    return pars


class variant:
    """A variant introduced on given days (immunity.py:18-130).

    ``variant`` is a known variant name or a dict of variant parameters;
    ``n_imports`` agents chosen among the susceptible are infected with it on
    each of ``days``.
    """

    def __init__(self, variant, days, label=None, n_imports=1, rescale=True):
        self.days = days
        self.n_imports = int(n_imports)
        self.rescale = rescale
        self.index = None
        self.label = None
        self.p = None
        self.parse(variant=variant, label=label)
        self.initialized = False

    def parse(self, variant=None, label=None):
        if isinstance(variant, str):
            choices, mapping = cvpar.get_variant_choices()
            key = variant.lower()
            for txt in ['.', ' ', 'variant', 'voc']:
                key = key.replace(txt, '')
            if key not in mapping:
                raise NotImplementedError(f'The selected variant "{variant}" is not implemented; choices are: {choices}')
            label = mapping[key]
            pars = dict(cvpar.get_variant_pars(variant=label))
        elif isinstance(variant, dict):
            defaults = cvpar.get_variant_pars(default=True)
            pars = dict(variant)
            label = pars.pop('label', label) or 'custom'
            invalid = [k for k in pars if k not in defaults]
            if invalid:
                raise KeyError(f'Could not parse variant keys "{invalid}"; valid keys are: "{cvd.variant_pars}"')
            for k in defaults:
                pars.setdefault(k, defaults[k])
        else:
            raise ValueError(f'Could not understand {type(variant)}, please specify as a dict or a predefined variant')
        self.label = label
        self.p = pars

    def initialize(self, pars):
        """immunity.py:106-114 against a parameter dict."""
        days = self.days if isinstance(self.days, (list, tuple, np.ndarray)) else [self.days]
        self.days = np.sort(np.asarray(days, dtype=int))
        pars['variant_pars'][self.label] = self.p
        self.index = list(pars['variant_pars'].keys()).index(self.label)
        pars['variant_map'][self.index] = self.label
        self.initialized = True
