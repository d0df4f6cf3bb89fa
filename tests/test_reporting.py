"""Reporting on the results and the infection log (sim.py:853-1040):
compute_yield, compute_doubling, compute_r_eff (daily / infectious / outcome)
and compute_gen_time against the reference's own methods run on a reference
simulation with testing (tests/golden/ref_reporting.npz; sciris' smooth, which
the daily method calls, is restated because sciris is not installed)."""
import json

import numpy as np

from common import load_npz
from covasim_gb300.sim import (yield_series, doubling_series, mean_infectious_duration, r_eff_daily, r_eff_window,
                               gen_time)


def _fixture():
    d = load_npz('ref_reporting.npz')
    res = {k[4:]: d[k] for k in d if k.startswith('res.')}
    ppl = {k[7:]: d[k] for k in d if k.startswith('people.')}
    return d, res, ppl


def test_yield_and_doubling_match_reference():
    d, res, _ = _fixture()
    ty, rty = yield_series(res)
    np.testing.assert_allclose(ty, d['out.test_yield'], rtol=1e-12)
    np.testing.assert_allclose(rty, d['out.rel_test_yield'], rtol=1e-12)
    assert d['out.test_yield'].sum() > 0
    np.testing.assert_allclose(doubling_series(res['cum_infections']), d['out.doubling_time'], rtol=1e-12,
                               equal_nan=True)


def test_r_eff_methods_match_reference():
    d, res, ppl = _fixture()
    dur = json.loads(str(d['dur']))
    mean_inf = mean_infectious_duration(ppl['date_recovered'], ppl['date_dead'], ppl['date_infectious'])
    got = r_eff_daily(mean_inf, res['new_infections'], res['n_imports'], res['n_infectious'], dur)
    # the reference averages the float32 dates in float32 (numpy's pairwise sums)
    np.testing.assert_allclose(got, d['out.r_eff_daily'], rtol=1e-5)
    npts = len(res['new_infections'])
    for method, keys in (('infectious', ['date_infectious']), ('outcome', ['date_recovered', 'date_dead'])):
        got = r_eff_window(npts, [ppl[k] for k in keys], d['log.source'])
        np.testing.assert_allclose(got, d[f'out.r_eff_{method}'], rtol=1e-12, equal_nan=True, err_msg=method)


def test_gen_time_matches_reference():
    d, _, ppl = _fixture()
    g = gen_time(d['log.source'], d['log.target'], ppl['date_exposed'], ppl['date_symptomatic'])
    np.testing.assert_allclose([g['true'], g['true_std'], g['clinical'], g['clinical_std']], d['out.gen_time'],
                               rtol=1e-12)
