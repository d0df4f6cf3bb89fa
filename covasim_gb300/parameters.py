"""Simulation parameters for the GPU path.

The parameter names and default values are those of Covasim 3.1.7
(covasim/parameters.py): the kernels consume them through a per-sim parameter
block, so the values must be the reference's. Tables kept alike on purpose:
``make_pars`` defaults (parameters.py:15-151), layer defaults
(parameters.py:158-227), age prognoses (parameters.py:230-294), variant
parameters (parameters.py:376-420) and cross-immunity (parameters.py:422-470).
"""
import copy

import numpy as np

from . import defaults as cvd

__all__ = ['make_pars', 'reset_layer_pars', 'get_prognoses', 'get_variant_pars',
           'get_cross_immunity', 'get_variant_choices', 'relative_prognoses', 'absolute_prognoses']

LAYER_PARS = ['beta_layer', 'contacts', 'dynam_layer', 'iso_factor', 'quar_factor']


def make_pars(set_prognoses=False, prog_by_age=True, **kwargs):
    """Default parameters (parameters.py:15-151)."""
    pars = {}
    pars['pop_size'] = 20e3
    pars['pop_infected'] = 20
    pars['pop_type'] = 'random'
    pars['location'] = None
    pars['start_day'] = '2020-03-01'
    pars['end_day'] = None
    pars['n_days'] = 60
    pars['rand_seed'] = 1
    pars['verbose'] = 0
    pars['pop_scale'] = 1
    pars['scaled_pop'] = None
    pars['rescale'] = True
    pars['rescale_threshold'] = 0.05
    pars['rescale_factor'] = 1.2
    pars['frac_susceptible'] = 1.0
    pars['contacts'] = None
    pars['dynam_layer'] = None
    pars['beta_layer'] = None
    pars['beta_dist'] = dict(dist='neg_binomial', par1=1.0, par2=0.45, step=0.01)
    pars['viral_dist'] = dict(frac_time=0.3, load_ratio=2, high_cap=4)
    pars['beta'] = 0.016
    pars['asymp_factor'] = 1.0
    pars['n_imports'] = 0
    pars['n_variants'] = 1
    pars['use_waning'] = True
    pars['nab_init'] = dict(dist='normal', par1=0, par2=2)
    pars['nab_decay'] = dict(form='nab_growth_decay', growth_time=21, decay_rate1=np.log(2) / 50,
                             decay_time1=150, decay_rate2=np.log(2) / 250, decay_time2=365)
    pars['nab_kin'] = None
    pars['nab_boost'] = 1.5
    pars['nab_eff'] = dict(alpha_inf=1.08, alpha_inf_diff=1.812, beta_inf=0.967, alpha_symp_inf=-0.739,
                           beta_symp_inf=0.038, alpha_sev_symp=-0.014, beta_sev_symp=0.079)
    pars['rel_imm_symp'] = dict(asymp=0.85, mild=1, severe=1.5)
    pars['immunity'] = None
    pars['trans_redux'] = 0.59
    pars['rel_beta'] = 1.0
    pars['dur'] = {
        'exp2inf': dict(dist='lognormal_int', par1=4.5, par2=1.5),
        'inf2sym': dict(dist='lognormal_int', par1=1.1, par2=0.9),
        'sym2sev': dict(dist='lognormal_int', par1=6.6, par2=4.9),
        'sev2crit': dict(dist='lognormal_int', par1=1.5, par2=2.0),
        'asym2rec': dict(dist='lognormal_int', par1=8.0, par2=2.0),
        'mild2rec': dict(dist='lognormal_int', par1=8.0, par2=2.0),
        'sev2rec': dict(dist='lognormal_int', par1=18.1, par2=6.3),
        'crit2rec': dict(dist='lognormal_int', par1=18.1, par2=6.3),
        'crit2die': dict(dist='lognormal_int', par1=10.7, par2=4.8),
    }
    pars['rel_symp_prob'] = 1.0
    pars['rel_severe_prob'] = 1.0
    pars['rel_crit_prob'] = 1.0
    pars['rel_death_prob'] = 1.0
    pars['prog_by_age'] = prog_by_age
    pars['prognoses'] = None
    pars['iso_factor'] = None
    pars['quar_factor'] = None
    pars['quar_period'] = 14
    pars['interventions'] = []
    pars['analyzers'] = []
    pars['timelimit'] = None
    pars['stopping_func'] = None
    pars['n_beds_hosp'] = None
    pars['n_beds_icu'] = None
    pars['no_hosp_factor'] = 2.0
    pars['no_icu_factor'] = 2.0
    pars['vaccine_pars'] = {}
    pars['vaccine_map'] = {}
    pars['variants'] = []
    pars['variant_map'] = {0: 'wild'}
    pars['variant_pars'] = dict(wild={})
    for key in cvd.variant_pars:
        if key in pars:
            pars['variant_pars']['wild'][key] = pars[key]
    pars.update(kwargs)
    reset_layer_pars(pars)
    if set_prognoses:
        pars['prognoses'] = get_prognoses(pars['prog_by_age'])
    return pars


def _layer_defaults(pop_type):
    random = dict(beta_layer=dict(a=1.0), contacts=dict(a=20), dynam_layer=dict(a=0),
                  iso_factor=dict(a=0.2), quar_factor=dict(a=0.3))
    hybrid = dict(beta_layer=dict(h=3.0, s=0.6, w=0.6, c=0.3),
                  contacts=dict(h=2.0, s=20, w=16, c=20),
                  dynam_layer=dict(h=0, s=0, w=0, c=0),
                  iso_factor=dict(h=0.3, s=0.1, w=0.1, c=0.1),
                  quar_factor=dict(h=0.6, s=0.2, w=0.2, c=0.2))
    table = {'random': random, 'hybrid': hybrid}
    if pop_type == 'synthpops':
        sp = copy.deepcopy(hybrid)
        for key, val in dict(beta_layer=1.5, contacts=10, dynam_layer=0, iso_factor=0.2, quar_factor=0.3).items():
            sp[key]['l'] = val
        table['synthpops'] = sp
    return random, table


def reset_layer_pars(pars, layer_keys=None, force=False):
    """Layer-specific parameters (parameters.py:158-227)."""
    random, table = _layer_defaults(pars['pop_type'])
    try:
        defaults = table[pars['pop_type']]
    except KeyError as E:
        raise ValueError(f'Cannot load defaults for population type "{pars["pop_type"]}": '
                         'must be hybrid, random, or synthpops') from E
    default_keys = list(defaults['beta_layer'].keys())
    for pkey in LAYER_PARS:
        default_val = random[pkey]['a']
        if force:
            par_dict = defaults[pkey]
        else:
            par_dict = dict(defaults[pkey])
            user = pars.get(pkey, None)
            if user:
                par_dict.update(user)
        if layer_keys:
            keys = list(layer_keys)
        else:
            keys = list(dict.fromkeys(default_keys + list(par_dict.keys())))
        pars[pkey] = {lkey: par_dict.get(lkey, default_val) for lkey in keys}
    return


def get_prognoses(by_age=True):
    """Prognosis probabilities by age, made conditional (parameters.py:230-294)."""
    if not by_age:
        prognoses = dict(
            age_cutoffs=np.array([0]),
            sus_ORs=np.array([1.00]),
            trans_ORs=np.array([1.00]),
            symp_probs=np.array([0.75]),
            comorbidities=np.array([1.00]),
            severe_probs=np.array([0.10]),
            crit_probs=np.array([0.04]),
            death_probs=np.array([0.01]),
        )
    else:
        prognoses = dict(
            age_cutoffs=np.array([0, 10, 20, 30, 40, 50, 60, 70, 80, 90]),
            sus_ORs=np.array([0.34, 0.67, 1.00, 1.00, 1.00, 1.00, 1.24, 1.47, 1.47, 1.47]),
            trans_ORs=np.array([1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00]),
            comorbidities=np.array([1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00]),
            symp_probs=np.array([0.50, 0.55, 0.60, 0.65, 0.70, 0.75, 0.80, 0.85, 0.90, 0.90]),
            severe_probs=np.array([0.00050, 0.00165, 0.00720, 0.02080, 0.03430, 0.07650, 0.13280,
                                   0.20655, 0.24570, 0.24570]),
            crit_probs=np.array([0.00003, 0.00008, 0.00036, 0.00104, 0.00216, 0.00933, 0.03639,
                                 0.08923, 0.17420, 0.17420]),
            death_probs=np.array([0.00002, 0.00002, 0.00010, 0.00032, 0.00098, 0.00265, 0.00766,
                                  0.02439, 0.08292, 0.16190]),
        )
    return relative_prognoses(prognoses)


def relative_prognoses(prognoses):
    """Absolute -> conditional probabilities (parameters.py:272-282)."""
    out = copy.deepcopy(prognoses)
    out['death_probs'] /= out['crit_probs']
    out['crit_probs'] /= out['severe_probs']
    out['severe_probs'] /= out['symp_probs']
    return out


def absolute_prognoses(prognoses):
    """Conditional -> absolute probabilities (parameters.py:285-298)."""
    out = copy.deepcopy(prognoses)
    out['severe_probs'] *= out['symp_probs']
    out['crit_probs'] *= out['severe_probs']
    out['death_probs'] *= out['crit_probs']
    return out


def get_variant_choices():
    """Known variant names and aliases (parameters.py:317-331)."""
    choices = {
        'wild': ['wild', 'default', 'pre-existing', 'original'],
        'alpha': ['alpha', 'b117', 'uk', 'united kingdom', 'kent'],
        'beta': ['beta', 'b1351', 'sa', 'south africa'],
        'gamma': ['gamma', 'p1', 'b11248', 'brazil'],
        'delta': ['delta', 'b16172', 'india'],
    }
    mapping = {name: key for key, syns in choices.items() for name in syns}
    return choices, mapping


def get_variant_pars(default=False, variant=None):
    """Per-variant parameters (parameters.py:376-420)."""
    pars = dict(
        wild=dict(rel_beta=1.0, rel_symp_prob=1.0, rel_severe_prob=1.0, rel_crit_prob=1.0, rel_death_prob=1.0),
        alpha=dict(rel_beta=1.67, rel_symp_prob=1.0, rel_severe_prob=1.64, rel_crit_prob=1.0, rel_death_prob=1.0),
        beta=dict(rel_beta=1.0, rel_symp_prob=1.0, rel_severe_prob=3.6, rel_crit_prob=1.0, rel_death_prob=1.0),
        gamma=dict(rel_beta=2.05, rel_symp_prob=1.0, rel_severe_prob=2.6, rel_crit_prob=1.0, rel_death_prob=1.0),
        delta=dict(rel_beta=2.2, rel_symp_prob=1.0, rel_severe_prob=3.2, rel_crit_prob=1.0, rel_death_prob=1.0),
    )
    if variant is not None:
        return pars[variant]
    return pars['wild'] if default else pars


def get_cross_immunity(default=False, variant=None):
    """Cross-immunity between known variants (parameters.py:422-470)."""
    pars = dict(
        wild=dict(wild=1.0, alpha=0.5, beta=0.5, gamma=0.34, delta=0.374),
        alpha=dict(wild=0.5, alpha=1.0, beta=0.8, gamma=0.8, delta=0.689),
        beta=dict(wild=0.066, alpha=0.5, beta=1.0, gamma=0.5, delta=0.086),
        gamma=dict(wild=0.34, alpha=0.4, beta=0.4, gamma=1.0, delta=0.088),
        delta=dict(wild=0.374, alpha=0.689, beta=0.086, gamma=0.088, delta=1.0),
    )
    if variant is not None:
        return pars[variant]
    return pars['wild'] if default else pars
