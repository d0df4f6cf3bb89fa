"""test_prob, contact_tracing and update_states_post on the GPU against the
oracle run with the same Philox draws (interventions.py:858-1145,
people.py:189-196,315-366,589-640), step mode against the graph run, and a
batch against its single runs."""
import copy

import numpy as np
import pytest

import covasim_gb300 as cv
from oracle.interventions import TestProb, ContactTracing
from test_gpu_sim import RES_KEYS, compare_runs, oracle_for

pytestmark = pytest.mark.gpu

TESTING_KEYS = RES_KEYS + ['new_tests', 'new_diagnoses', 'new_quarantined', 'new_isolated', 'n_diagnosed',
                           'n_quarantined', 'n_isolated']

CASES = [
    ('hybrid', 3000, 50, 1, True, True, dict(symp_prob=0.2, asymp_prob=0.01), dict(trace_probs=0.5, trace_time=1)),
    ('hybrid', 2500, 45, 2, True, False,
     dict(symp_prob=0.3, asymp_prob=0.02, symp_quar_prob=0.5, asymp_quar_prob=0.1, quar_policy='both',
          sensitivity=0.9, loss_prob=0.1, test_delay=2),
     dict(trace_probs={'h': 1.0, 's': 0.5, 'w': 0.5, 'c': 0.2}, trace_time={'h': 0, 's': 1, 'w': 2, 'c': 3})),
    ('random', 3000, 45, 3, True, False, dict(symp_prob=0.3, quar_policy='daily', start_day=5, end_day=30),
     dict(trace_probs=0.8, presumptive=True, start_day=8)),
    ('hybrid', 2000, 40, 4, False, True, dict(symp_prob=0.3, quar_policy=[0, 2]),
     dict(trace_probs=0.7, trace_time=0.5, quar_period=10)),
    # influenza-like illness (a constant and a daily prevalence) and fixed subtargets
    ('hybrid', 3000, 45, 5, True, True,
     dict(symp_prob=0.2, asymp_prob=0.005, quar_policy='both', ili_prev=0.02,
          subtarget=dict(inds=list(range(0, 3000, 7)), vals=0.3)),
     dict(trace_probs=0.5, trace_time=1)),
    ('random', 2500, 45, 6, False, False,
     dict(symp_prob=0.3, start_day=3, ili_prev=[0.01] * 8 + [0.05] * 12,
          subtarget=dict(inds=list(range(3, 2500, 11)), vals=[0.05 + 0.45 * (k % 3) for k in range(227)])),
     dict(trace_probs=0.6)),
    # distributions of delays from symptom onset to swab
    ('hybrid', 3000, 45, 7, True, True,
     dict(symp_prob=0.25, asymp_prob=0.01, swab_delay=dict(dist='lognormal', par1=3, par2=4)),
     dict(trace_probs=0.5, trace_time=1)),
    ('random', 2500, 45, 8, False, False,
     dict(symp_prob=0.4, quar_policy='daily', swab_delay=dict(dist='uniform', par1=0, par2=5), ili_prev=0.01),
     dict(trace_probs=0.7)),
    # a tracing capacity below the day's cases
    ('hybrid', 3000, 45, 9, True, True, dict(symp_prob=0.4, asymp_prob=0.02), dict(trace_probs=0.8, capacity=4)),
    ('random', 2500, 45, 10, False, False, dict(symp_prob=0.5, test_delay=1),
     dict(trace_probs=0.9, presumptive=True, capacity=3)),
]


def make_sim(pop_type, n, days, seed, waning, dyn, tp, ct):
    pars = dict(pop_type=pop_type, pop_size=n, n_days=days, rand_seed=seed, pop_infected=30, use_waning=waning,
                interventions=[cv.test_prob(**tp), cv.contact_tracing(**ct)])
    if dyn:
        pars['dynam_layer'] = dict(h=0, s=0, w=0, c=1)
    return cv.Sim(pars)


@pytest.mark.parametrize('case', range(len(CASES)))
def test_testing_and_tracing_match_oracle_philox(case):
    pop_type, n, days, seed, waning, dyn, tp, ct = CASES[case]
    sim = make_sim(*CASES[case])
    sim.initialize()
    orc = oracle_for(sim)
    orc.interventions = [TestProb(**tp), ContactTracing(**ct)]
    for iv in orc.interventions:
        if hasattr(iv, 'initialize'):
            iv.initialize(orc)
    orc.run()
    sim.run()
    raw = sim.raw_results()
    assert raw['new_tests'].sum() > 0 and raw['new_diagnoses'].sum() > 0 and raw['new_quarantined'].sum() > 0
    compare_runs(sim, orc, keys=TESTING_KEYS)


def test_ili_and_subtargets_add_tests():
    """interventions.py:941-972: the day's influenza-like illnesses test with the
    symptomatic probability, subtargeted agents with their own."""
    base = dict(symp_prob=0.2, asymp_prob=0.005)
    tests = []
    for extra in ({}, dict(ili_prev=0.05), dict(subtarget=dict(inds=list(range(0, 3000, 5)), vals=0.5))):
        sim = make_sim('hybrid', 3000, 30, 9, True, False, dict(base, **extra), dict(trace_probs=0.5))
        tests.append(sim.run().raw_results()['new_tests'].sum())
    assert tests[1] > 1.5 * tests[0] and tests[2] > 1.5 * tests[0], tests


def test_tracing_capacity_limits_the_traced():
    """interventions.py:1074-1078: a capacity of 0 traces nobody (no quarantines),
    one above every day's cases gives the run without a capacity."""
    raws = []
    for cap in (None, 0, 10**9):
        sim = make_sim('hybrid', 3000, 40, 11, True, False, dict(symp_prob=0.5, asymp_prob=0.02),
                       dict(trace_probs=1.0, capacity=cap))
        raws.append(sim.run().raw_results())
    assert raws[0]['new_quarantined'].sum() > 0 and raws[0]['new_diagnoses'].max() > 2
    assert raws[1]['new_quarantined'].sum() == 0
    for k in TESTING_KEYS:
        np.testing.assert_array_equal(raws[2][k], raws[0][k], err_msg=k)


def test_testing_step_mode_equals_graph_run():
    args = CASES[1]
    a = make_sim(*args).run()
    b = make_sim(*args)
    b.initialize()
    for _ in range(b.npts):
        b.step()
    b.finalize()
    ra, rb = a.raw_results(), b.raw_results()
    for k in TESTING_KEYS:
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)


def test_testing_batch_equals_single_runs():
    sims = [make_sim(*c) for c in CASES[:2]] + [cv.Sim(pop_type='random', pop_size=2000, n_days=50, rand_seed=9)]
    sims[1].pars['n_days'] = sims[2].pars['n_days'] = sims[0].pars['n_days']
    singles = [cv.Sim(copy.deepcopy(s.pars)).run() for s in sims]
    batch = cv.BatchSim([cv.Sim(copy.deepcopy(s.pars)) for s in sims]).run()
    for k, single in enumerate(singles):
        raw = single.raw_results()
        got = batch.results(k)
        for key in TESTING_KEYS:
            np.testing.assert_array_equal(got[key], raw[key], err_msg=f'sim {k} {key}')


def test_reporting_on_a_device_run():
    """finalize's compute_results and the other reporting methods on device results and log."""
    from covasim_gb300.sim import r_eff_window, mean_infectious_duration, r_eff_daily
    sim = make_sim(*CASES[0]).run()
    res = sim.results
    assert np.nansum(res['test_yield'].values) > 0 and np.isfinite(res['r_eff'].values).all()
    mean_inf = mean_infectious_duration(sim.people['date_recovered'], sim.people['date_dead'],
                                        sim.people['date_infectious'])
    want = r_eff_daily(mean_inf, res['new_infections'].values, res['n_imports'].values, res['n_infectious'].values,
                       sim['dur'])
    np.testing.assert_allclose(res['r_eff'].values, want, rtol=1e-9)
    log = sim.state.infection_log(0)
    got = sim.compute_r_eff(method='infectious')
    want = r_eff_window(sim.npts, [sim.people['date_infectious']], log[:, 0])
    np.testing.assert_allclose(got, want, rtol=1e-12, equal_nan=True)
    g = sim.compute_gen_time()
    assert 2 < g['true'] < 10


def test_testing_with_rescaling_and_importations_matches_oracle_philox():
    """The held day of a dynamic rescaling (sim.py:535-556) skips the testing,
    tracing and post passes too; daily importations at the day's scale."""
    tp, ct = dict(symp_prob=0.2, asymp_prob=0.01), dict(trace_probs=0.5, trace_time=1)
    pars = dict(pop_type='hybrid', pop_size=3000, n_days=50, rand_seed=8, pop_infected=20, pop_scale=6,
                n_imports=2, dynam_layer=dict(h=0, s=0, w=0, c=1),
                interventions=[cv.test_prob(**tp), cv.contact_tracing(**ct)])
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim)
    orc.interventions = [TestProb(**tp), ContactTracing(**ct)]
    for iv in orc.interventions:
        if hasattr(iv, 'initialize'):
            iv.initialize(orc)
    orc.run()
    assert len(np.unique(orc.rescale_vec)) > 3
    sim.run()
    compare_runs(sim, orc, keys=TESTING_KEYS + ['n_imports'])
    np.testing.assert_array_equal(sim.rescale_vec, orc.rescale_vec)


def test_rescaling_with_variant_importations_graph_step_and_batch_agree():
    """Variant days run as single steps (with their own rescale check) between
    graph segments that may be held back for a rescaling."""
    def make(seed):
        return cv.Sim(pop_type='hybrid', pop_size=3000, n_days=45, rand_seed=seed, pop_scale=8, use_waning=True,
                      variants=[cv.variant(dict(rel_beta=1.6), days=[12, 25], n_imports=10, label='v')])
    a = make(4).run()
    b = make(4)
    b.initialize()
    for _ in range(b.npts):
        b.step()
    b.finalize()
    batch = cv.BatchSim([make(4), make(5)]).run()
    for k in RES_KEYS + ['n_imports', 'new_infections_by_variant']:
        np.testing.assert_array_equal(a.raw_results()[k], b.raw_results()[k], err_msg=k)
        np.testing.assert_array_equal(a.raw_results()[k], batch.results(0)[k], err_msg=k)
    np.testing.assert_array_equal(a.rescale_vec, b.rescale_vec)
    assert len(np.unique(a.rescale_vec)) > 2 and a.raw_results()['new_infections_by_variant'][1].sum() > 0
