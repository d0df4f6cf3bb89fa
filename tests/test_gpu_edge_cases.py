"""Edge cases of the whole-sim path: tiny and empty populations, layers without
edges, zero-length runs, everyone or nobody infected, a sim ending on its first
day, and populations whose size is not a multiple of the 32-agent word."""
import numpy as np
import pytest

import covasim_gb300 as cv

pytestmark = pytest.mark.gpu


def run(**kw):
    pars = dict(pop_type='random', pop_size=100, n_days=10, rand_seed=1, pop_infected=5)
    pars.update(kw)
    return cv.Sim(pars).run()


def test_single_agent_and_tiny_populations():
    for n, k in ((1, 1), (2, 1), (31, 3), (33, 3), (257, 10)):
        sim = run(pop_size=n, pop_infected=k)
        r = sim.results
        assert r['cum_infections'].values[-1] >= k
        assert np.all(r['n_alive'].values + r['cum_deaths'].values == n)


def test_zero_days_and_one_day():
    for days in (0, 1):
        sim = run(n_days=days)
        assert len(sim.results['new_infections'].values) == days + 1


def test_nobody_and_everybody_infected_at_start():
    sim = run(pop_infected=0)
    assert sim.results['cum_infections'].values[-1] == 0
    sim = run(pop_size=64, pop_infected=64, n_days=30)
    assert sim.results['cum_infections'].values[-1] >= 64
    assert sim.results['new_infections'].values.sum() == 0 or sim['use_waning']


def test_layer_without_edges():
    n = 200
    popdict = dict(uid=np.arange(n), age=np.full(n, 30.0), sex=np.zeros(n, dtype=int),
                   contacts={'a': dict(p1=np.zeros(0, dtype=np.int32), p2=np.zeros(0, dtype=np.int32),
                                       beta=np.zeros(0, dtype=np.float32))})
    sim = cv.Sim(dict(pop_type='random', pop_size=n, n_days=15, pop_infected=10, rand_seed=3), popdict=popdict).run()
    assert sim.results['new_infections'].values.sum() == 0  # no contacts: only the seeds
    assert sim.results['cum_infections'].values[-1] == 10


def test_hybrid_with_the_dynamic_layer_only_transmitting():
    sim = run(pop_type='hybrid', pop_size=3000, n_days=30, dynam_layer=dict(h=0, s=0, w=0, c=1),
              beta_layer=dict(h=0, s=0, w=0, c=1))
    assert sim.results['cum_infections'].values[-1] > 5


def test_batch_with_sims_of_different_sizes_including_tiny_ones():
    sims = [cv.Sim(pop_type='random', pop_size=n, n_days=20, rand_seed=s, pop_infected=min(5, n))
            for s, n in enumerate((1, 33, 500, 4097))]
    batch = cv.BatchSim(sims).run()
    for k, s in enumerate(sims):
        solo = cv.Sim(dict(s.pars)).run().raw_results()['new_infections']
        np.testing.assert_array_equal(batch.results(k)['new_infections'], solo)


def test_batch_with_variant_importations_equals_single_runs():
    def make(k):
        vs = [cv.variant(dict(rel_beta=1.5), days=10 + 5 * k, n_imports=5, label='v1')]
        if k == 1:
            vs.append(cv.variant(dict(rel_beta=1.8), days=[20, 21], n_imports=3, label='v2'))
        return cv.Sim(pop_type='hybrid', pop_size=3000, n_days=40, rand_seed=7 + k, use_waning=True,
                      variants=vs, dynam_layer=dict(h=0, s=0, w=0, c=1))
    sims = [make(k) for k in range(3)] + [cv.Sim(pop_type='hybrid', pop_size=2000, n_days=40, rand_seed=3)]
    batch = cv.BatchSim(sims).run()
    for k in range(len(sims)):
        solo = (make(k) if k < 3 else cv.Sim(pop_type='hybrid', pop_size=2000, n_days=40, rand_seed=3)).run()
        ref = solo.raw_results()
        got = batch.results(k)
        for key in ('new_infections', 'new_infections_by_variant', 'n_exposed', 'new_deaths'):
            np.testing.assert_array_equal(got[key], ref[key], err_msg=f'sim {k} {key}')
