"""Parity at the benchmark's own scale: the 1,000,000-agent hybrid sim with
waning immunity and the community layer redrawn daily (the configuration
bench.py times), against the oracle run with the same Philox draws.

* The first 40 days, with the resident-bitmap edge pass ('8192r': the source
  bitmap of 1M agents, 122 KB, in shared memory beside the candidate queues),
  with the tiled pass ('8192') and with the one-wave pass ('1024w'): every
  result series and the final state.
* One day at the epidemic's peak (the day with the most new infections of a
  GPU run), started from the GPU's state of the evening before: the most
  sources, candidates and transmission events a day of this run holds.
"""
import numpy as np
import pytest

import covasim_gb300 as cv
from common import ALL_KEYS, RES_KEYS, assert_state_equal, compare_runs, oracle_for

pytestmark = pytest.mark.gpu

BENCH_PARS = dict(pop_size=1_000_000, pop_type='hybrid', pop_infected=100, use_waning=True, rand_seed=1,
                  dynam_layer=dict(h=0, s=0, w=0, c=1))
PEOPLE_KEYS = [k for k in ALL_KEYS if k not in ('age', 'sex', 'uid', 'doses')]


@pytest.fixture(scope='module')
def population():
    """The bench sim's population, built once for every test of this module."""
    sim = cv.Sim(dict(BENCH_PARS, n_days=40))
    sim.initialize()
    return sim.popdict, sim._person


@pytest.fixture(scope='module')
def oracle_40_days(population):
    """The oracle's run of the first 40 days (shared by both edge-pass variants)."""
    popdict, person = population
    sim = cv.Sim(dict(BENCH_PARS, n_days=40), popdict=popdict, person=person)
    sim.initialize()
    orc = oracle_for(sim).run()
    assert orc.results['new_infections'].sum() > 1000
    return orc


@pytest.mark.parametrize('tile', ['8192r', '8192', '1024w'])
def test_bench_config_first_40_days_match_oracle(population, oracle_40_days, tile):
    popdict, person = population
    sim = cv.Sim(dict(BENCH_PARS, n_days=40), popdict=popdict, person=person, edge_tile=tile)
    sim.initialize()
    assert str(sim.state.edge_tile_label) == tile
    sim.run()
    compare_runs(sim, oracle_40_days)


def test_bench_config_peak_day_matches_oracle(population):
    popdict, person = population
    probe = cv.Sim(dict(BENCH_PARS, n_days=120), popdict=popdict, person=person, edge_tile='8192r')
    probe.run()
    new = probe.raw_results()['new_infections']
    peak = int(np.argmax(new))
    assert 20 < peak < 120 and new[peak] > 10_000, (peak, new[peak])
    sim = cv.Sim(dict(BENCH_PARS, n_days=120), popdict=popdict, person=person, edge_tile='8192r')
    sim.initialize()
    sim.run(until=peak)
    orc = oracle_for(sim)
    for k in PEOPLE_KEYS:  # the oracle starts from the GPU's state after day peak - 1
        orc.people[k] = np.array(sim.people.gpu(k).cpu().numpy(), dtype=orc.people[k].dtype)
    orc.t = peak
    orc.step()
    sim.step()
    raw = sim.raw_results()
    for k in RES_KEYS:
        assert raw[k][peak] == orc.results[k][peak], (k, raw[k][peak], orc.results[k][peak])
    assert raw['new_infections'][peak] == new[peak]
    np.testing.assert_allclose(raw['pop_nabs'][peak], orc.results['pop_nabs'][peak], rtol=1e-5)
    assert_state_equal(lambda k: sim.people.gpu(k).cpu().numpy(), {k: orc.people[k] for k in PEOPLE_KEYS},
                       keys=PEOPLE_KEYS, float_rtol=1e-6, label=f'state after day {peak}')
