"""The reference-signature drop-ins of the day path, one function at a time,
against the reference's own outputs (ref_day_*.npz, recorded from Covasim
3.1.7's code): People.check_infectious ... check_death and check_exit_iso in
update_states_pre's order, check_immunity, update_nab, update_peak_nab, and
People.infect with sources; plus the torch custom ops they run through."""
import numpy as np
import pytest
import torch

import covasim_gb300 as cv
from covasim_gb300 import immunity as cvimm
from covasim_gb300.people import People
from common import load_day, snap
from oracle import philox as ph
from oracle import gpu_arith as ga
from test_gpu_day import build, compare

pytestmark = pytest.mark.gpu

CASES = ['hybrid', 'variants', 'random']


def people_of(st, pars, t):
    p = People(st, 0, pars, {})
    p.__dict__['t'] = t
    return p


@pytest.mark.parametrize('case', CASES)
def test_checks_one_by_one_match_update_states_pre(case):
    """people.py:164-186 called as the reference does: each check returns the
    agents it changed, and the state after check_immunity is the reference's."""
    d, pars = load_day(case)
    t = int(d['d.t'])
    st, _ = build(d, pars)
    people = people_of(st, pars, t)
    S0, S1 = snap(d, 'd.S0'), snap(d, 'd.S1')
    got = {'new_infectious': people.check_infectious(), 'new_symptomatic': people.check_symptomatic(),
           'new_severe': people.check_severe(), 'new_critical': people.check_critical(),
           'new_recoveries': people.check_recovery()}
    released = people.check_exit_iso()
    dead, n_dead, n_known = people.check_death()
    if pars['use_waning']:
        cvimm.check_immunity(people)
    torch.cuda.synchronize()
    assert st.status() == 0
    compare(st, S1, 'checks one by one + check_immunity')
    for k, inds in got.items():
        assert len(inds) == d[f'd.flows.{k}'], k
        assert np.all(np.diff(inds) > 0), k
    assert n_dead == d['d.flows.new_deaths'] and n_known == d['d.flows.new_known_deaths']
    np.testing.assert_array_equal(got['new_infectious'], np.nonzero(S1['infectious'] & ~S0['infectious'])[0])
    np.testing.assert_array_equal(dead, np.nonzero(S1['dead'] & ~S0['dead'])[0])
    np.testing.assert_array_equal(released, np.nonzero(S0['isolated'] & ~S1['isolated'])[0])
    fv = d['d.flows_variant.new_infectious_by_variant']
    np.testing.assert_array_equal(people.flows_variant['new_infectious_by_variant'], fv)


@pytest.mark.parametrize('case', ['hybrid', 'variants'])
def test_check_immunity_and_update_nab_match_reference(case):
    """immunity.py:303-350 from the state after the checks, and immunity.py:205-213
    at the end of the day (the reference's d.S2 -> d.S3 update_nab)."""
    d, pars = load_day(case)
    t = int(d['d.t'])
    st, _ = build(d, pars, prefix='d.S1')
    for k in ('sus_imm', 'symp_imm', 'sev_imm'):
        st.set(k, np.zeros_like(d[f'd.S1.{k}']))
    people = people_of(st, pars, t)
    cvimm.check_immunity(people)
    torch.cuda.synchronize()
    for k in ('sus_imm', 'symp_imm', 'sev_imm'):
        np.testing.assert_array_equal(st.get(k).cpu().numpy(), d[f'd.S1.{k}'], err_msg=k)
    st2, _ = build(d, pars, prefix='d.S2')
    people = people_of(st2, pars, t)
    has_nabs = np.nonzero(d['d.S2.peak_nab'])[0]
    cvimm.update_nab(people, has_nabs)
    torch.cuda.synchronize()
    got, want = st2.get('nab').cpu().numpy(), d['d.S3.nab']
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=0)
    assert st2.status() == 0


def test_update_peak_nab_boost_and_initial_levels():
    """immunity.py:138-202: agents with NAbs are boosted (float32 product); the
    others get 2 ** nab_init scaled by their symptom class's rel_imm_symp and
    1 + alpha_inf_diff, with the draws of Philox block 3 of the agent's infect
    stream (formed as the oracle's float-float mirror forms them)."""
    sim = cv.Sim(pop_size=3000, n_days=10, rand_seed=7, use_waning=True)
    sim.initialize()
    st, pars = sim.state, sim.pars
    rng = np.random.default_rng(3)
    nab = np.where(rng.random(3000) < 0.4, rng.uniform(0.1, 3, 3000), 0).astype(np.float32)
    peak = np.where(nab > 0, nab * 1.3, 0).astype(np.float32)
    st.set('nab', nab)
    st.set('peak_nab', peak)
    people = people_of(st, pars, 4)
    inds = np.sort(rng.choice(3000, 600, replace=False))
    cls = rng.integers(0, 3, len(inds))
    symp = {key: inds[cls == c] for c, key in enumerate(('asymp', 'mild', 'sev'))}
    cvimm.update_peak_nab(people, inds, pars, symp=symp)
    torch.cuda.synchronize()
    got = st.get('peak_nab').cpu().numpy()
    prior = nab[inds] > 0
    np.testing.assert_array_equal(got[inds[prior]], (peak[inds[prior]] * np.float32(pars['nab_boost'])))
    fresh = inds[~prior]
    k0, k1 = ph.seed_key(sim['rand_seed'])
    w = ph.philox4x32_10(fresh, 3, 4, ph.TAG_INFECT | 2, k0, k1)
    (zh, zl), _ = ga.box_muller_ff(w[0], w[1])
    init = ga.sample_ff(pars['nab_init'], zh, zl)
    rel = np.array([pars['rel_imm_symp'][k] for k in ('asymp', 'mild', 'severe')])[cls[~prior]]
    want = ((ga.exp2_ff(init) * rel) * (1 + pars['nab_eff']['alpha_inf_diff'])).astype(np.float32)
    np.testing.assert_array_equal(got[fresh], want)
    assert np.all(st.get('t_nab_event').cpu().numpy()[inds] == 4)
    untouched = np.setdiff1d(np.arange(3000), inds)
    np.testing.assert_array_equal(got[untouched], peak[untouched])


def test_infect_keeps_first_sources_and_returns_the_infected():
    """people.py:465-511: duplicates keep their first source, only the
    susceptible are infected and returned, and the log records each source."""
    sim = cv.Sim(pop_size=2000, n_days=5, rand_seed=2, pop_infected=0)
    sim.initialize()
    people = sim.people
    people.__dict__['t'] = 1
    first = people.infect(np.array([5, 9]), layer='h')
    np.testing.assert_array_equal(first, [5, 9])
    inds = np.array([30, 9, 12, 30, 5, 40, 12])
    src = np.array([100, 101, 102, 103, 104, 105, 106])
    got = people.infect(inds, source=src, layer='s')
    np.testing.assert_array_equal(got, [12, 30, 40])  # 5 and 9 are no longer susceptible
    log = {e['target']: e for e in people.infection_log if e['layer'] == 's'}
    assert {k: v['source'] for k, v in log.items()} == {12: 102, 30: 100, 40: 105}
    assert all(v['date'] == 1 for v in log.values())
    assert people.flows['new_infections'] == 5


def test_day_path_runs_through_torch_custom_ops():
    """The fused day entry points are torch.ops.covgpu.* operators."""
    for name in ('agent_step', 'edge_pass', 'infect_claims', 'infect_list', 'import_day', 'test_trace',
                 'lik_targets', 'run_days', 'check', 'check_immunity', 'update_nab', 'update_peak_nab',
                 'layer_lists'):
        assert hasattr(torch.ops.covgpu, name), name
    sim = cv.Sim(pop_size=4000, n_days=20, rand_seed=5)
    sim.initialize()
    st = sim.state
    with torch.profiler.profile(activities=[torch.profiler.ProfilerActivity.CPU]) as prof:
        for _ in range(3):
            sim.step()  # a day at a time: one op per kernel call
        sim.run()       # the remaining days: one run_days op (a CUDA graph)
    names = {e.name for e in prof.events()}
    for op in ('covgpu::agent_step', 'covgpu::edge_pass', 'covgpu::infect_claims', 'covgpu::import_day',
               'covgpu::test_trace', 'covgpu::infect_list', 'covgpu::run_days'):
        assert op in names, op
    assert st.status() == 0
