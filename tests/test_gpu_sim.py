"""Whole simulations on the GPU against the oracle run with the same Philox draws,
batch-versus-single identity, the reference's behavioural known answers, and
the distribution of outcomes against 200 seeds of the reference's own code."""
import copy

import numpy as np
import pytest
import torch

import covasim_gb300 as cv
from common import load_npz, assert_state_equal, ALL_KEYS, RES_KEYS, oracle_for, compare_runs
from oracle.sim import OracleSim

pytestmark = pytest.mark.gpu

@pytest.mark.parametrize('pop_type,n,days,dyn,seed', [('hybrid', 3000, 45, False, 1), ('random', 4000, 50, False, 2),
                                                     ('hybrid', 2500, 40, True, 3)])
def test_sim_matches_oracle_philox(pop_type, n, days, dyn, seed):
    pars = dict(pop_type=pop_type, pop_size=n, n_days=days, rand_seed=seed, pop_infected=30,
                interventions=[cv.change_beta(days=25, changes=0.6)])
    if dyn:
        pars['dynam_layer'] = dict(h=0, s=0, w=0, c=1)
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim).run()
    sim.run()
    compare_runs(sim, orc)


@pytest.mark.parametrize('pop_type,n,days,rate,seed', [('hybrid', 3000, 40, 0.7, 4), ('random', 2000, 35, 6, 5)])
def test_sim_with_daily_importations_matches_oracle_philox(pop_type, n, days, rate, seed):
    """sim.py:582-587: Poisson(n_imports) agents infected every day (graph run and
    step by step), against the oracle with the same draws."""
    pars = dict(pop_type=pop_type, pop_size=n, n_days=days, rand_seed=seed, pop_infected=10, n_imports=rate,
                dynam_layer=dict(h=0, s=0, w=0, c=1) if pop_type == 'hybrid' else dict(a=0))
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim).run()
    assert orc.results['n_imports'].sum() > 10
    sim.run()
    compare_runs(sim, orc, keys=RES_KEYS + ['n_imports'])
    stepped = cv.Sim(pars)
    stepped.initialize()
    for _ in range(stepped.npts):
        stepped.step()
    stepped.finalize()
    ra, rb = sim.raw_results(), stepped.raw_results()
    for k in RES_KEYS + ['n_imports']:
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)
    imported = sorted((e['date'], e['target']) for e in sim.people.infection_log if e['layer'] == 'importation')
    want = sorted((e['date'], int(e['target'])) for e in orc.people.infection_log if e['layer'] == 'importation')
    assert imported == want and 0 < len(imported) <= ra['n_imports'].sum()


@pytest.mark.parametrize('frac,rate', [(0.6, 0), (0.85, 2)])
def test_sim_with_nonnaive_fraction_matches_oracle_philox(frac, rate):
    """sim.py:519-522: round((1 - frac_susceptible) * n) agents start non-naive."""
    pars = dict(pop_type='hybrid', pop_size=3000, n_days=40, rand_seed=9, pop_infected=40, frac_susceptible=frac,
                n_imports=rate)
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim).run()
    sim.run()
    compare_runs(sim, orc, keys=RES_KEYS + ['n_imports'])
    never = ~sim.people['naive'] & ~sim.people['exposed'] & ~sim.people['recovered'] & ~sim.people['dead']
    assert never.sum() >= round((1 - frac) * 3000) - 40
    batch = cv.BatchSim([cv.Sim(dict(pars)), cv.Sim(dict(pars, rand_seed=10, frac_susceptible=1.0))]).run()
    np.testing.assert_array_equal(batch.results(0)['new_infections'], sim.raw_results()['new_infections'])


@pytest.mark.parametrize('pop_type,n,days,extra', [
    ('hybrid', 3000, 60, dict(pop_scale=10, pop_infected=30)),
    ('random', 2500, 50, dict(pop_scale=4, n_imports=2, rescale_factor=1.5, rescale_threshold=0.1)),
    ('hybrid', 2000, 40, dict(pop_scale=3, rescale=False, n_imports=3))])
def test_rescaling_matches_oracle_philox(pop_type, n, days, extra):
    """sim.py:535-556 dynamic rescaling (the day kernels hold the run back on the
    day one falls due, the host performs it), importations at the day's scale,
    and finalize's scaling of the results (sim.py:771-787, 838-839)."""
    pars = dict(pop_type=pop_type, pop_size=n, n_days=days, rand_seed=21, **extra)
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim).run()
    sim.run()
    compare_runs(sim, orc, keys=RES_KEYS + ['n_imports'])
    np.testing.assert_array_equal(sim.rescale_vec, orc.rescale_vec)
    if extra.get('rescale', True):
        assert len(np.unique(orc.rescale_vec)) > 2
    raw = sim.raw_results()
    np.testing.assert_allclose(sim.results['new_infections'].values, raw['new_infections'] * orc.rescale_vec)
    np.testing.assert_allclose(sim.results['n_alive'].values[-1],
                               n * sim['pop_scale'] - sim.results['cum_deaths'].values[-1])
    stepped = cv.Sim(pars)
    stepped.initialize()
    for _ in range(stepped.npts):
        stepped.step()
    stepped.finalize()
    for k in RES_KEYS + ['n_imports']:
        np.testing.assert_array_equal(stepped.raw_results()[k], raw[k], err_msg=k)
    np.testing.assert_array_equal(stepped.rescale_vec, sim.rescale_vec)


def test_rescaling_resume_until_equals_one_run():
    """run(until=...) then run() with rescalings held back inside both segments."""
    pars = dict(pop_type='random', pop_size=3000, n_days=50, rand_seed=14, pop_scale=10, n_imports=1)
    a = cv.Sim(pars).run()
    b = cv.Sim(pars)
    b.run(until=23)
    b.run()
    for k in RES_KEYS + ['n_imports']:
        np.testing.assert_array_equal(a.raw_results()[k], b.raw_results()[k], err_msg=k)
    np.testing.assert_array_equal(a.rescale_vec, b.rescale_vec)
    assert len(np.unique(a.rescale_vec)) > 2


def test_batch_with_rescaling_equals_single_runs():
    mk = [dict(pop_type='random', pop_size=2500, n_days=45, rand_seed=3, pop_scale=8),
          dict(pop_type='random', pop_size=1800, n_days=45, rand_seed=4),
          dict(pop_type='hybrid', pop_size=3000, n_days=45, rand_seed=5, pop_scale=5, n_imports=1.5)]
    singles = [cv.Sim(dict(p)).run() for p in mk]
    batch = cv.BatchSim([cv.Sim(dict(p)) for p in mk]).run()
    finals = batch.finalize()
    for k, single in enumerate(singles):
        got = batch.results(k)
        for key in RES_KEYS + ['n_imports']:
            np.testing.assert_array_equal(got[key], single.raw_results()[key], err_msg=f'sim {k} {key}')
        for key in ('new_infections', 'cum_infections', 'n_alive', 'n_susceptible'):
            np.testing.assert_array_equal(finals[k].results[key].values, single.results[key].values, err_msg=key)
    again = cv.Sim(dict(mk[0]))
    again.initialize()
    snap = again.state.snapshot()
    again.run()
    again.rewind(snap).run()  # a rerun from a snapshot starts from scale 1 again
    np.testing.assert_array_equal(again.results['new_infections'].values, singles[0].results['new_infections'].values)


def test_sim_with_variants_matches_oracle_philox():
    """Variant importations (immunity.py:117-130) with bed limits in force: the
    importations take no limits (variant.apply calls infect() without them),
    transmission does; per-variant flows against the oracle."""
    pars = dict(pop_type='hybrid', pop_size=4000, n_days=50, rand_seed=31, use_waning=True, pop_infected=40,
                n_beds_hosp=3, n_beds_icu=1, n_imports=1, dynam_layer=dict(h=0, s=0, w=0, c=1),
                variants=[cv.variant(dict(rel_beta=1.6, rel_severe_prob=2.0), days=10, n_imports=20, label='v1'),
                          cv.variant(dict(rel_beta=1.3), days=[20, 21], n_imports=8, label='v2')])
    sim = cv.Sim(pars)
    sim.initialize()
    orc = oracle_for(sim).run()
    sim.run()
    compare_runs(sim, orc, keys=RES_KEYS + ['n_imports'])
    raw = sim.raw_results()
    for k in ('new_infections_by_variant', 'new_severe_by_variant'):
        np.testing.assert_array_equal(raw[k], orc.results[k], err_msg=k)
    assert (raw['new_infections_by_variant'][1:].sum(axis=1) > 20).all()


def test_step_mode_equals_graph_run():
    pars = dict(pop_type='hybrid', pop_size=3000, n_days=30, rand_seed=7)
    a = cv.Sim(pars).run()
    b = cv.Sim(pars)
    b.initialize()
    for _ in range(b.npts):
        b.step()
    b.finalize()
    ra, rb = a.raw_results(), b.raw_results()
    for k in RES_KEYS + ['pop_nabs', 'pop_protection']:
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)
    c = cv.Sim(pars).run(use_graph=False)
    rc = c.raw_results()
    for k in RES_KEYS:
        np.testing.assert_array_equal(ra[k], rc[k], err_msg=k)


def test_steady_agent_steps_equal_the_run():
    """The agent pass skips warps of susceptible naive agents on the days after a
    full pass (every day of a launch sequence but the first, or single steps flagged
    COVGPU_DAY_STEADY): single steps with the flag, a run with waning and a redrawn
    layer in graph launches, and the full single steps all agree."""
    from covasim_gb300.sim import init_infections
    pars = dict(pop_type='hybrid', pop_size=20000, n_days=70, rand_seed=5, use_waning=True, pop_infected=10,
                dynam_layer=dict(h=0, s=0, w=0, c=1))
    ref = cv.Sim(pars).run().raw_results()
    for steady in (True, False):
        sim = cv.Sim(pars)
        sim.initialize()
        st = sim.state
        init_infections(st, 0, sim.pars)
        for t in range(sim.npts):
            st.agent_step(t, do_prev=t > 0, do_day=True, steady=steady and t > 0)
            st.edge_pass(t)
            st.infect_claims(t)
        st.agent_step(sim.npts, do_prev=True, do_day=False)
        assert st.status() == 0
        got = st.results(0)
        for k in RES_KEYS + ['pop_nabs', 'pop_protection']:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f'steady {steady} {k}')
    cum = np.cumsum(ref['new_infections'])
    assert cum[15] < 0.01 * pars['pop_size'] < 0.3 * pars['pop_size'] < cum[-1]  # steady warps early, few late


def test_graph_capture_and_replay_equal_the_direct_run():
    """covgpu_run_days launches a state's day range directly on its first run,
    captures it into a CUDA graph on the second and replays the graph after
    that: the three runs (and a run with testing, whose graph holds the testing
    passes) are identical."""
    for pars in (dict(pop_type='hybrid', pop_size=6000, n_days=40, rand_seed=9, use_waning=True,
                      dynam_layer=dict(h=0, s=0, w=0, c=1)),
                 dict(pop_type='hybrid', pop_size=4000, n_days=35, rand_seed=4,
                      interventions=[cv.test_prob(symp_prob=0.2), cv.contact_tracing(trace_probs=0.5)])):
        sim = cv.Sim(pars)
        sim.initialize()
        snap = sim.state.snapshot()
        runs = []
        for _ in range(3):
            sim.rewind(snap)
            sim.run()
            runs.append({k: np.array(v, copy=True) for k, v in sim.raw_results().items()})
        for r in runs[1:]:
            for k in RES_KEYS + ['pop_nabs', 'pop_protection']:
                np.testing.assert_array_equal(r[k], runs[0][k], err_msg=k)


def test_resume_until_equals_one_run():
    """test_resume.py:19-52: run(until=) then run() equals one run."""
    pars = dict(pop_type='random', pop_size=5000, n_days=40, rand_seed=11)
    a = cv.Sim(pars).run()
    b = cv.Sim(pars)
    b.run(until=17)
    b.run()
    for k in RES_KEYS:
        np.testing.assert_array_equal(a.results[k].values, b.results[k].values, err_msg=k)


def test_batch_equals_single_runs():
    sims = [cv.Sim(pop_type='random', pop_size=n, n_days=40, rand_seed=s, beta=b,
                   interventions=[cv.change_beta(days=20, changes=c)])
            for n, s, b, c in [(3000, 1, 0.02, 0.5), (10000, 2, 0.015, 0.9), (777, 3, 0.025, 0.3)]]
    singles = [cv.Sim(copy.deepcopy(s.pars)).run() for s in sims]
    batch = cv.BatchSim([cv.Sim(copy.deepcopy(s.pars)) for s in sims]).run()
    for k, single in enumerate(singles):
        raw = single.raw_results()
        got = batch.results(k)
        for key in RES_KEYS + ['pop_nabs']:
            np.testing.assert_array_equal(got[key], raw[key], err_msg=f'sim {k} {key}')


def test_batch_with_daily_importations_equals_single_runs():
    sims = [cv.Sim(pop_type='random', pop_size=n, n_days=30, rand_seed=s, n_imports=r)
            for n, s, r in [(3000, 1, 2.5), (1500, 2, 0), (5000, 3, 10)]]
    singles = [cv.Sim(copy.deepcopy(s.pars)).run() for s in sims]
    batch = cv.BatchSim([cv.Sim(copy.deepcopy(s.pars)) for s in sims]).run()
    for k, single in enumerate(singles):
        raw = single.raw_results()
        got = batch.results(k)
        for key in RES_KEYS + ['n_imports', 'pop_nabs']:
            np.testing.assert_array_equal(got[key], raw[key], err_msg=f'sim {k} {key}')
    assert batch.results(1)['n_imports'].sum() == 0 and batch.results(2)['n_imports'].sum() > 200


def test_beta_zero_no_transmission():
    """tests/unittests/test_transmission.py:16-35."""
    sim = cv.Sim(pop_size=5000, n_days=30, beta=0, pop_infected=50).run()
    assert sim.results['new_infections'].values.sum() == 0
    assert sim.results['cum_infections'].values[-1] == 50


@pytest.mark.parametrize('delay', [1, 5, 15])
def test_exposed_to_infectious_delay_exact(delay):
    """tests/unittests/test_progression.py:17-51: std 0 => everyone infectious on day `delay`."""
    pars = cv.make_pars(pop_size=500, pop_infected=500, n_days=30)
    pars['dur']['exp2inf'] = dict(dist='normal', par1=delay, par2=0)
    pars['rel_symp_prob'] = 0
    sim = cv.Sim(pars).run()
    ch = sim.results['new_infectious'].values
    assert ch[delay] == 500 and ch[:delay].sum() == 0


@pytest.mark.parametrize('dur', [1, 2, 5, 10, 20])
def test_recovery_day_exact(dur):
    """tests/unittests/test_progression.py:54-80: infectious after 1 day, all
    asymptomatic, asym2rec `dur` days with std 0 => all recover on day 1 + dur."""
    pars = cv.make_pars(pop_size=500, pop_infected=500, n_days=30)
    pars['dur']['exp2inf'] = dict(dist='normal', par1=1, par2=0)
    pars['dur']['asym2rec'] = dict(dist='normal', par1=dur, par2=0)
    pars['rel_symp_prob'] = 0
    ch = cv.Sim(pars).run().results['new_recoveries'].values
    assert ch[1 + dur] == 500 and ch.sum() == 500


@pytest.mark.parametrize('dur', [1, 2, 5, 10, 20])
def test_time_to_die_exact(dur):
    """tests/unittests/test_progression.py:83-108: everyone critical on day 0
    (certain prognoses, no delays), crit2die `dur` days with std 0 => all die on day dur."""
    pars = cv.make_pars(pop_size=500, pop_infected=500, n_days=30)
    for k in ('exp2inf', 'inf2sym', 'sym2sev', 'sev2crit'):
        pars['dur'][k] = dict(dist='normal', par1=0, par2=0)
    pars['dur']['crit2die'] = dict(dist='normal', par1=dur, par2=0)
    sim = cv.Sim(pars)
    progs = cv.get_prognoses(sim['prog_by_age'])  # set after creation: a pars dict with prog_by_age resets them
    for k in ('symp_probs', 'severe_probs', 'crit_probs', 'death_probs'):
        progs[k][:] = 1.0
    sim['prognoses'] = progs
    ch = sim.run().results['new_deaths'].values
    assert ch[dur] == 500 and ch.sum() == 500


def test_everyone_dies_with_certain_death():
    """tests/unittests/test_mortality.py:13-24."""
    pars = cv.make_pars(pop_size=400, pop_infected=400, n_days=60)
    for k in ('rel_symp_prob', 'rel_severe_prob', 'rel_crit_prob', 'rel_death_prob'):
        pars[k] = 1e6
    sim = cv.Sim(pars).run()
    assert sim.results['cum_deaths'].values[-1] == 400


def test_no_deaths_with_zero_death_prob():
    """tests/unittests/test_mortality.py:26-45."""
    sim = cv.Sim(pop_size=5000, n_days=60, rel_death_prob=0.0).run()
    assert sim.results['cum_deaths'].values[-1] == 0


def test_waning_raises_reinfections_and_nabs():
    """tests/test_immunity.py:88-128."""
    base = dict(pop_size=8000, n_days=150, beta=0.02)
    s0 = cv.Sim(base, use_waning=False).run()
    s1 = cv.Sim(base, use_waning=True).run()
    assert s0.results['cum_reinfections'].values[-1] == 0
    assert s1.results['cum_reinfections'].values[-1] > 0
    assert s1.results['pop_nabs'].values.max() > 0 and s0.results['pop_nabs'].values.max() == 0
    assert s1.results['pop_protection'].values.max() > 0


def test_dynamic_layer_lists_match_oracle():
    """A dynamic layer's day as per-agent contact lists (base.py:1849-1876 redraws
    every edge with uniform endpoints): each agent's lists as p1 and as p2 equal
    the oracle's draws, their lengths follow Binomial(E, 1/n) and the partners are
    uniform over the agents."""
    from scipy.stats import binom, chisquare
    from oracle import philox as ph
    n = 5001
    sim = cv.Sim(pop_type='hybrid', pop_size=n, n_days=20, rand_seed=12, dynam_layer=dict(h=0, s=0, w=0, c=1))
    sim.initialize()
    keys = [ly['key'] for ly in sim.spec.layers]
    li = keys.index('c')
    n_edges = len(sim.spec.layers[li]['p1'])
    k0, k1 = ph.seed_key(sim['rand_seed'])
    table = ph.dyn_count_table(n_edges, n)
    for t in (0, 3, 17):
        counts, offsets, partners = sim.state.layer_lists(0, li, t)
        a, d, j, g = ph.dyn_lists(k0, k1, t, li, np.arange(n), table, n)
        want = np.zeros((n, 2), dtype=np.int64)
        np.add.at(want, (a, d), 1)
        np.testing.assert_array_equal(counts.cpu().numpy(), want)
        np.testing.assert_array_equal(partners.cpu().numpy(), g)
        sub_c, sub_o, sub_p = sim.state.layer_lists(0, li, t, agents=(1000, 37))
        np.testing.assert_array_equal(sub_c.cpu().numpy(), want[1000:1037])
        np.testing.assert_array_equal(sub_p.cpu().numpy(), g[(a >= 1000) & (a < 1037)])
    c = counts.cpu().numpy().reshape(-1)
    lo, hi = 4, 18  # tails merged into the end bins, so every expected count is large
    obs = np.bincount(np.clip(c, lo, hi) - lo, minlength=hi - lo + 1)
    cdf = binom.cdf(np.arange(lo, hi), n_edges, 1 / n)
    pk = np.diff(np.concatenate([[0.0], cdf, [1.0]]))
    assert chisquare(obs, pk * len(c)).pvalue > 1e-3
    assert chisquare(np.bincount(g % 50, minlength=50)).pvalue > 1e-3
