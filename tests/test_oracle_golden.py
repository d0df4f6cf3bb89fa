"""The CPU oracle against golden vectors produced by the reference's own code.

The fixtures under tests/golden/ were made by tests/golden/make_golden.py, which
runs Covasim 3.1.7's function bodies (covasim/utils.py, people.py, immunity.py,
population.py and Sim.step) with recorded draws. Every comparison here is exact:
the oracle restates the reference in the same float32/float64 arithmetic.
"""
import json

import numpy as np
import pytest

from common import (load_npz, load_day, snap, oracle_people, n_layers, assert_state_equal, unjson, fix_pars, ALL_KEYS,
                    load_testing_case)
from oracle import kernels as ok
from oracle.people import TableDraws, update_nab
from oracle.sim import OracleSim
from oracle import philox as ph

DAY_CASES = ['hybrid', 'variants', 'random']


# ------------------------------------------------------------------ standalone kernels
def test_viral_load_matches_reference():
    d = load_npz('ref_kernels.npz')
    for i, (t, fr, lr, hc) in enumerate(d['vl.cases']):
        out = ok.compute_viral_load(int(t), d['vl.ts'], d['vl.rec'], d['vl.dead'], fr, lr, hc)
        assert out.dtype == np.float32
        assert np.array_equal(out, d[f'vl{i}.out'], equal_nan=True), i


def test_trans_sus_matches_reference():
    d = load_npz('ref_kernels.npz')
    for i, (bl, af, isf, qf) in enumerate(d['ts.cases']):
        a, b = ok.compute_trans_sus(d['ts.rt'], d['ts.rs'], d['ts.inf'], d['ts.sus'], bl, d['ts.vl'], d['ts.symp'],
                                    d['ts.iso'], d['ts.quar'], af, isf, qf, d['ts.imm'])
        assert np.array_equal(a, d[f'ts{i}.rel_trans']) and np.array_equal(b, d[f'ts{i}.rel_sus']), i


def test_infections_match_reference_with_its_draws():
    d = load_npz('ref_kernels.npz')
    for i, beta in enumerate(d['inf.betas']):
        src, tgt = ok.compute_infections(np.float32(beta), d[f'inf{i}.p1'], d[f'inf{i}.p2'], d[f'inf{i}.lb'],
                                         d[f'inf{i}.rt'], d[f'inf{i}.rs'], d[f'inf{i}.U'])
        assert np.array_equal(src, d[f'inf{i}.src']) and np.array_equal(tgt, d[f'inf{i}.tgt']), i


# ------------------------------------------------------------------ one day of the hot path
@pytest.mark.parametrize('case', DAY_CASES)
def test_day_matches_reference(case):
    d, pars = load_day(case)
    t = int(d['d.t'])
    people = oracle_people(d, 'd.S0', pars)
    people.update_states_pre(t)
    assert_state_equal(lambda k: people[k], snap(d, 'd.S1'), label='update_states_pre')
    for k, v in people.flows.items():
        assert v == d[f'd.flows.{k}'], k
    vd = pars['viral_dist']
    vl = ok.compute_viral_load(t, people.date_infectious, people.date_recovered, people.date_dead,
                               vd['frac_time'], vd['load_ratio'], vd['high_cap'])
    assert np.array_equal(vl, d['d.viral_load'], equal_nan=True)
    hosp_max, icu_max = d['d.hosp_icu']
    layers = [str(k) for k in d['d.layer_keys']]
    for v in range(pars['n_variants']):
        beta = d[f'd.v{v}.beta']
        inf_variant = people.infectious * (people.infectious_variant == v)
        for li, lkey in enumerate(layers):
            key = f'd.v{v}.L{li}'
            rt, rs = ok.compute_trans_sus(people.rel_trans, people.rel_sus, inf_variant, people.susceptible,
                                          pars['beta_layer'][lkey], vl, people.symptomatic, people.isolated,
                                          people.quarantined, pars['asymp_factor'], pars['iso_factor'][lkey],
                                          pars['quar_factor'][lkey], people.sus_imm[v, :])
            assert np.array_equal(rt, d[f'{key}.rel_trans']) and np.array_equal(rs, d[f'{key}.rel_sus']), key
            src, tgt = ok.compute_infections(beta, d[f'd.L{li}.p1'], d[f'd.L{li}.p2'], d[f'd.L{li}.beta'], rt, rs,
                                             d[f'{key}.U'])
            assert np.array_equal(src, d[f'{key}.src']) and np.array_equal(tgt, d[f'{key}.tgt']), key
            agents, table = d[f'{key}.draw_agents'], d[f'{key}.draw_table']
            lookup = dict(zip(agents.tolist(), range(len(agents))))
            draws = TableDraws(lambda inds: table[[lookup[int(a)] for a in inds]])
            inds = people.infect(tgt, hosp_max=hosp_max, icu_max=icu_max, source=src, layer=lkey, variant=v,
                                 draws=draws)
            assert np.array_equal(inds, d[f'{key}.infected']), key
    assert_state_equal(lambda k: people[k], snap(d, 'd.S2'), label='infect')
    has_nabs = people.peak_nab.nonzero()[0]
    if pars['use_waning'] and len(has_nabs):
        update_nab(people, has_nabs)
    assert_state_equal(lambda k: people[k], snap(d, 'd.S3'), label='update_nab')


# ------------------------------------------------------------------ whole runs, MT19937 mode
def test_whole_runs_match_reference_mt_mode():
    d = load_npz('ref_sims.npz')
    for i in range(int(d['n'])):
        pars = fix_pars(unjson(json.loads(str(d[f's{i}.pars']))))
        person = {k[len(f's{i}.person.'):]: v for k, v in d.items() if k.startswith(f's{i}.person.')}
        nl = len([k for k in d if k.startswith(f's{i}.L') and k.endswith('.p1')])
        keys = list(pars['beta_layer'].keys())
        contacts = {keys[li]: {c: d[f's{i}.L{li}.{c}'] for c in ('p1', 'p2', 'beta')} for li in range(nl)}
        sim = OracleSim(pars, person, contacts, rng='mt').run()
        for k, v in sim.results.items():
            ref = d[f's{i}.res.{k}']
            np.testing.assert_allclose(v, ref, rtol=1e-12, atol=0, err_msg=f'sim {i} {k}')
        for k in ('exposed', 'recovered', 'dead', 'susceptible', 'date_recovered', 'peak_nab', 'nab'):
            assert np.array_equal(sim.people[k], d[f's{i}.final.{k}'], equal_nan=True), (i, k)
        np.testing.assert_array_equal(sim.rescale_vec, d[f's{i}.rescale_vec'], err_msg=f'sim {i} rescale_vec')
    assert len(np.unique(d['s7.rescale_vec'])) > 10  # a run that rescales many times


def test_testing_and_tracing_runs_match_reference_mt_mode():
    """test_prob + contact_tracing + update_states_post (interventions.py:858-1145,
    people.py:189-196,315-366,589-640) against the reference's own code."""
    from oracle.interventions import TestProb, ContactTracing
    d = load_npz('ref_testing.npz')
    for i in range(int(d['n'])):
        pars, person, contacts, tp, ct = load_testing_case(d, i)
        sim = OracleSim(pars, person, contacts, rng='mt', interventions=[TestProb(**tp), ContactTracing(**ct)]).run()
        assert d[f's{i}.res.new_tests'].sum() > 0 and d[f's{i}.res.new_quarantined'].sum() > 0
        for k, v in sim.results.items():
            np.testing.assert_array_equal(v, d[f's{i}.res.{k}'], err_msg=f'case {i} {k}')
        for k in [k[len(f's{i}.final.'):] for k in d if k.startswith(f's{i}.final.')]:
            assert np.array_equal(sim.people[k], d[f's{i}.final.{k}'], equal_nan=True), (i, k)


# ------------------------------------------------------------------ philox
def test_philox_known_answers():
    """Random123 known-answer vectors for Philox-4x32-10."""
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for c, k, want in cases:
        got = ph.philox4x32_10(*c, *k)
        assert tuple(int(x) for x in got) == want


def test_uniform_conversions_exact_and_open():
    a = np.array([0, 0xffffffff, 123456789], dtype=np.uint32)
    u = ph.u01_52(a, a)
    assert np.all(u > 0) and np.all(u < 1)
    u32 = ph.u01_32(a)
    assert np.all(u32 > 0) and np.all(u32 < 1)
    idx = ph.uniform_index(np.array([0xffffffff]), np.array([0xffffffff]), 7)
    assert idx[0] == 6
