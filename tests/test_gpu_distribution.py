"""Distribution parity of whole runs against the reference's own code.

Each test runs 200 seeds of a sim on the GPU (one BatchSim, the library's own
Philox streams) and compares the outcome distribution with 200 seeds of the
reference's own Sim.step (MT19937 streams; fixtures written by
tests/golden/make_golden.py through refload, which executes the reference's
function bodies).

The rule (fixed before looking at the outcomes):

* Primary statistics, one per reported series of the comparison: cumulative
  new infections, cumulative new severe cases, cumulative new deaths, the peak
  day of new infections and its height. Each must pass on its own: two-sample
  KS p > 0.01, and the means within 2 standard errors of their difference.
* Secondary statistics, the daily values of the same series on a grid of days:
  a family of m tests per criterion, held to a family-wise error of 1% with
  Holm's step-down method for the KS p-values and a Bonferroni bound on the
  mean differences (|z| below the two-sided 1 - 0.01 / m quantile). Testing m
  days at the per-test 1% / 2-SE levels would fail an exact implementation by
  chance alone with probability 1 - 0.99^m (KS) and 1 - 0.954^m (means).
"""
import json

import numpy as np
import pytest

import covasim_gb300 as cv
from common import load_npz

pytestmark = pytest.mark.gpu

SERIES = ('new_infections', 'new_severe', 'new_deaths')


def primary_stats(s):
    """The primary statistics of a [seeds, days] dict of series."""
    out = {f'cum_{k}': s[k].sum(1) for k in SERIES}
    out['peak_day'] = s['new_infections'].argmax(1)
    out['peak_height'] = s['new_infections'].max(1)
    return out


def two_sample(a, b):
    """(KS p-value, z of the mean difference) of two samples."""
    from scipy.stats import ks_2samp
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    z = 0.0 if se == 0 else (a.mean() - b.mean()) / se
    if se == 0 and a.mean() != b.mean():
        z = np.inf
    return ks_2samp(a, b).pvalue, z


def check_distribution(got, ref, days):
    """Apply the rule of this module; returns the table of every statistic."""
    from scipy.stats import norm
    table, failures = {}, []
    gp, rp = primary_stats(got), primary_stats(ref)
    for name in gp:
        p, z = two_sample(gp[name], rp[name])
        table[name] = (p, z, float(np.mean(gp[name])), float(np.mean(rp[name])))
        if p <= 0.01 or abs(z) > 2:
            failures.append(('primary', name, p, z))
    sec = {f'{k}_d{d}': (got[k][:, d], ref[k][:, d]) for k in SERIES for d in days}
    m = len(sec)
    zlim = norm.ppf(1 - 0.01 / (2 * m))
    res = {name: two_sample(a, b) for name, (a, b) in sec.items()}
    for name, (p, z) in res.items():
        table[name] = (p, z, float(np.mean(sec[name][0])), float(np.mean(sec[name][1])))
        if abs(z) > zlim:
            failures.append(('secondary mean', name, p, z))
    # Holm: the k-th smallest p-value (k = 0, 1, ...) against 0.01 / (m - k), stopping at the first pass
    for k, (name, (p, z)) in enumerate(sorted(res.items(), key=lambda kv: kv[1][0])):
        if p > 0.01 / (m - k):
            break
        failures.append(('secondary KS', name, p, z))
    return table, failures


def run_batch(pars, n_seeds, keys):
    batch = cv.BatchSim(cv.Sim(pars), n_runs=n_seeds).run()
    return {k: batch.series(k) for k in keys}


def test_distribution_random_20k_200_seeds():
    """The default 20k random sim (60 days)."""
    ref = load_npz('ref_distribution.npz')
    n_seeds, pop_size, n_days = (int(x) for x in ref['meta'])
    got = run_batch(dict(pop_size=pop_size, n_days=n_days, pop_type='random', rand_seed=0), n_seeds, SERIES)
    table, failures = check_distribution(got, {k: ref[k] for k in SERIES}, days=(10, 20, 30, 40, 50, 60))
    assert not failures, (failures, table)


def test_distribution_hybrid_waning_dynamic_200_seeds():
    """A 30k-agent hybrid sim with waning immunity (NAb kinetics, reinfections)
    and the community layer redrawn every day, 150 days: the model of the
    1M-agent benchmark. Also compares reinfections and the mean NAb level."""
    ref = load_npz('ref_distribution_hybrid.npz')
    n_seeds, pop_size, n_days = (int(x) for x in ref['meta'])
    pars = json.loads(str(ref['pars']))
    keys = SERIES + ('new_reinfections', 'pop_nabs')
    got = run_batch(dict(pars, rand_seed=0), n_seeds, keys)
    table, failures = check_distribution(got, {k: ref[k] for k in SERIES},
                                         days=(20, 35, 50, 65, 80, 100, 125, 150))
    for name, a, b in (('cum_new_reinfections', got['new_reinfections'].sum(1), ref['new_reinfections'].sum(1)),
                       ('pop_nabs_d100', got['pop_nabs'][:, 100], ref['pop_nabs'][:, 100])):
        p, z = two_sample(a, b)
        table[name] = (p, z, float(np.mean(a)), float(np.mean(b)))
        if p <= 0.01 or abs(z) > 2:
            failures.append(('primary', name, p, z))
    assert not failures, (failures, table)
