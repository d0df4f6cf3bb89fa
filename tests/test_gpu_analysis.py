"""TransTree, Fit and Calibration on real GPU sims, checked against the oracle's
restatement of the reference's consumers on the same sim's log and results."""
import datetime as dt

import numpy as np
import pytest

import covasim_gb300 as cv
from oracle import analysis as oa

pytestmark = pytest.mark.gpu


def make_testing_sim(datafile=None, **kw):
    pars = dict(pop_type='hybrid', pop_size=4000, n_days=45, rand_seed=5, pop_infected=30, use_waning=True,
                interventions=[cv.test_prob(symp_prob=0.2, asymp_prob=0.01), cv.contact_tracing(trace_probs=0.5)])
    pars.update(kw)
    return cv.Sim(pars, datafile=datafile)


def test_transtree_matches_the_oracle_on_a_gpu_run():
    sim = make_testing_sim().run()
    tt = sim.make_transtree()
    people = {k: sim.people[k] for k in oa.ATTRS + oa.QUAR_ATTRS + ['date_recovered']}
    o = oa.transtree(sim.people.infection_log, people, len(sim.people), sim.people.t, start_day=5, end_day=30)
    assert tt.n_days == sim.npts - 1
    assert tt.sources == o['sources'] and tt.source_dates == o['source_dates']
    assert tt.targets == o['targets'] and tt.target_dates == o['target_dates']
    np.testing.assert_array_equal(tt.n_targets, o['n_targets'])
    np.testing.assert_array_equal(tt.count_targets(5, 30), o['n_targets_window'])
    assert tt.transmissions == o['transmissions']
    assert tt.r0() == pytest.approx(o['r0_0'], rel=1e-12)
    assert tt.r0(recovered_only=True) == pytest.approx(o['r0_1'], rel=1e-12)
    for k, ref in o['detailed'].items():
        got = tt.detailed[k]
        if ref.dtype == object:
            assert [str(x) for x in got] == [str(x) for x in ref], k
        else:
            np.testing.assert_array_equal(np.asarray(got, dtype=np.float64), ref.astype(np.float64), err_msg=k)
    for k, ref in o['df'].items():
        got = np.asarray(tt.df[k])
        if ref.dtype == object:
            assert [str(x) for x in got] == [str(x) for x in ref], k
        else:
            np.testing.assert_array_equal(got, ref, err_msg=k)


def synthetic_data(sim, every=3, shift=-4):
    """Data columns (with dates) from a finished sim's cumulative results, thinned and noised."""
    rng = np.random.default_rng(0)
    days = np.arange(shift, sim.npts, every)
    start = dt.date.fromisoformat(sim['start_day'])
    cols = {'date': [start + dt.timedelta(days=int(d)) for d in days]}
    for key in ('cum_diagnoses', 'cum_deaths', 'cum_tests'):
        v = np.interp(days, np.arange(sim.npts), sim.results[key].values)
        v = np.round(v * rng.uniform(0.9, 1.1, len(v)))
        v[rng.random(len(v)) < 0.1] = np.nan
        cols[key] = v
    return cols


def test_fit_matches_the_oracle_on_a_gpu_run():
    truth = make_testing_sim(beta=0.02).run()
    data = synthetic_data(truth)
    sim = make_testing_sim(datafile=data)
    assert sim.day('2020-03-11') == 10 and sim.date(10) == '2020-03-11'
    sim.run()
    fit = sim.compute_fit()
    series = {k: sim.results[k].values for k in sim.result_keys()}
    dates = list(sim.datevec)
    mism, total = oa.fit(series, dates, {k: sim.data[k] for k in sim.data.columns if k != 'date'},
                         list(sim.data['date']))
    assert fit.mismatch == pytest.approx(total, rel=1e-12)
    for k, v in mism.items():
        assert fit.mismatches[k] == pytest.approx(v, rel=1e-12)


def test_calibration_runs_trials_in_batches():
    truth = make_testing_sim(beta=0.02).run()
    sim = make_testing_sim(beta=0.012, datafile=synthetic_data(truth))
    calib = cv.Calibration(sim, calib_pars=dict(beta=[0.012, 0.008, 0.03]), n_workers=6, n_trials=3, seed=1,
                           verbose=False)
    calib.calibrate(verbose=False)
    assert len(calib.trials) == 18
    assert all(0.008 <= t['params']['beta'] <= 0.03 for t in calib.trials)
    best = min(t['value'] for t in calib.trials)
    # a batched trial equals the same sim run alone (every draw is keyed by the sim's own seed)
    assert calib.after.fit.mismatch == pytest.approx(best, rel=1e-12)
    assert calib.after.fit.mismatch < calib.before.fit.mismatch
    assert abs(calib.best_pars['beta'] - 0.02) < 0.006
    js = calib.to_json()
    assert js[0]['mismatch'] == pytest.approx(best) and set(js[0]['pars']) == {'beta'}
