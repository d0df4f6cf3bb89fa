"""One day of the fused GPU path replayed against the reference's own outputs.

From a mid-epidemic state recorded from Covasim 3.1.7's code, the fused agent
pass must reproduce update_states_pre + check_immunity, the fused edge pass +
infect must reproduce every (variant, layer) round of compute_trans_sus,
compute_infections and People.infect given the reference's own draws, and the
closing pass must reproduce update_nab and the day's stock counts.
"""
import numpy as np
import pytest
import torch

from common import load_day, snap, assert_state_equal, ALL_KEYS, FLOAT_KEYS
from covasim_gb300 import _lib as L
from covasim_gb300 import defaults as cvd
from covasim_gb300.state import SimSpec, BatchState
from oracle import philox as ph

pytestmark = pytest.mark.gpu

CASES = ['hybrid', 'variants', 'random']
SETTABLE = [k for k in ALL_KEYS if k not in ('uid', 'doses', 'age', 'sex')]


def build(d, pars, prefix='d.S0'):
    keys = [str(k) for k in d['d.layer_keys']]
    layers = []
    for li, k in enumerate(keys):
        p1 = d[f'd.L{li}.p1']
        assert np.all(np.diff(p1) >= 0)  # stored order == reference order
        layers.append(dict(key=k, p1=p1, p2=d[f'd.L{li}.p2'], beta=d[f'd.L{li}.beta'], dynamic=False))
    person = {k: d[f'{prefix}.{k}'] for k in ('symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans',
                                              'rel_sus')}
    npts = int(pars['n_days']) + 1
    spec = SimSpec(pars, person, layers, np.full(npts, pars['beta']),
                   np.array([[pars['beta_layer'][k] for k in keys]] * npts))
    st = BatchState([spec])
    for k in SETTABLE:
        st.set(k, d[f'{prefix}.{k}'])
    return st, keys


def getter(st):
    def get(k):
        if k in ('uid',):
            return np.arange(st.specs[0].n)
        if k == 'doses':
            return np.zeros(st.specs[0].n, np.int32)
        if k in ('age', 'sex'):
            return None
        return st.get(k).cpu().numpy()
    return get


def compare(st, ref, label, float_rtol=0.0):
    keys = [k for k in ALL_KEYS if k not in ('age', 'sex', 'doses')]
    assert_state_equal(getter(st), ref, keys=keys, float_rtol=float_rtol, label=label)


@pytest.mark.parametrize('case', CASES)
def test_agent_pass_matches_update_states_pre(case):
    d, pars = load_day(case)
    t = int(d['d.t'])
    st, _ = build(d, pars)
    st.agent_step(t, do_prev=False, do_day=True)
    torch.cuda.synchronize()
    compare(st, snap(d, 'd.S1'), 'update_states_pre + check_immunity')
    res = st.results(0)
    for k in ('new_infectious', 'new_symptomatic', 'new_severe', 'new_critical', 'new_recoveries', 'new_deaths',
              'new_known_deaths'):
        assert res[k][t] == d[f'd.flows.{k}'], k
    fv = d['d.flows_variant.new_infectious_by_variant']
    np.testing.assert_array_equal(res['new_infectious_by_variant'][:, t], fv)
    assert res['_severe_now'][t] == np.count_nonzero(d['d.S1.severe'])
    assert res['_critical_now'][t] == np.count_nonzero(d['d.S1.critical'])
    vl = st.t['viral_load'][:st.specs[0].n].cpu().numpy()
    inf = d['d.S1.infectious']
    assert np.array_equal(vl[inf], d['d.viral_load'][inf])


@pytest.mark.parametrize('case', CASES)
def test_edge_pass_and_infect_match_reference_rounds(case):
    d, pars = load_day(case)
    t = int(d['d.t'])
    st, keys = build(d, pars)
    st.agent_step(t, do_prev=False, do_day=True)
    nv = pars['n_variants']
    n = st.specs[0].n
    # the reference's per-(variant, layer) draws, by segment
    uni = []
    for li in range(len(keys)):
        E = len(d[f'd.L{li}.p1'])
        if E == 0:
            continue
        uni.append(np.stack([d[f'd.v{v}.L{li}.U'] for v in range(nv)]).reshape(nv, 2, E))
    st.set_edge_uniforms(uni)
    table = np.full((st.n, ph.N_DRAWS), np.nan)
    for v in range(nv):
        for li in range(len(keys)):
            key = f'd.v{v}.L{li}'
            table[d[f'{key}.draw_agents']] = d[f'{key}.draw_table']
    st.set_draw_table(table)
    st.edge_pass(t)
    st.infect_claims(t)
    torch.cuda.synchronize()
    assert st.status() == 0
    compare(st, snap(d, 'd.S2'), 'edge pass + infect', float_rtol=1e-6)
    res = st.results(0)
    expect = sum(len(d[f'd.v{v}.L{li}.infected']) for v in range(nv) for li in range(len(keys)))
    assert res['new_infections'][t] == expect
    # infection log: same (source, target, layer, variant) records as the reference's rounds
    log = st.infection_log(0)
    got = {(int(r[1]), int(r[0]), int(r[3]), int(r[4])) for r in log}
    want = set()
    for v in range(nv):
        for li in range(len(keys)):
            key = f'd.v{v}.L{li}'
            tgt, src = d[f'{key}.tgt'], d[f'{key}.src']
            first = {}
            for s_, g_ in zip(src.tolist(), tgt.tolist()):
                first.setdefault(g_, s_)
            for g_ in d[f'{key}.infected'].tolist():
                want.add((g_, first[g_], li, v))
    assert got == want
    # closing pass: update_nab and the end-of-day stocks
    st.set_draw_table(None)
    st.set_edge_uniforms(None)
    st.agent_step(t + 1, do_prev=True, do_day=False)
    torch.cuda.synchronize()
    compare(st, snap(d, 'd.S3'), 'update_nab', float_rtol=1e-6)
    res = st.results(0)
    for key in cvd.result_stocks:
        assert res[f'n_{key}'][t] == np.count_nonzero(d[f'd.S3.{key}']), key
    for v in range(nv):
        assert res['n_exposed_by_variant'][v, t] == np.count_nonzero(d['d.S3.exposed_by_variant'][v])
    alive = ~d['d.S3.dead']
    nab = d['d.S3.nab'][alive]
    want_nabs = np.sum(nab[nab.nonzero()[0]]) / alive.sum()
    np.testing.assert_allclose(res['pop_nabs'][t], want_nabs, rtol=1e-6)
