"""Shared helpers for the tests: golden-fixture loading and state comparison."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, 'golden')

from oracle.people import (PERSON, STATES, VARIANT_STATES, BY_VARIANT_STATES, IMM_STATES, NAB_STATES,  # noqa: E402
                           VACC_STATES, DATES, DURS, OraclePeople)

ALL_KEYS = PERSON + STATES + VARIANT_STATES + BY_VARIANT_STATES + IMM_STATES + NAB_STATES + VACC_STATES + DATES + DURS
FLOAT_KEYS = [k for k in ALL_KEYS if k not in STATES + BY_VARIANT_STATES + ['uid', 'n_infections', 'n_breakthroughs',
                                                                              't_nab_event', 'doses', 'vaccine_source']]


def unjson(x):
    if isinstance(x, dict):
        if '__array__' in x:
            return np.array(x['__array__'], dtype=x['dtype'])
        return {k: unjson(v) for k, v in x.items()}
    if isinstance(x, list):
        return [unjson(v) for v in x]
    return x


def fix_pars(p):
    """JSON round trip turns int dict keys into strings; restore them."""
    p = dict(p)
    if 'variant_map' in p:
        p['variant_map'] = {int(k): v for k, v in p['variant_map'].items()}
    if 'vaccine_map' in p:
        p['vaccine_map'] = {int(k): v for k, v in p['vaccine_map'].items()}
    return p


def load_npz(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def load_testing_case(d, i):
    """Inputs of case ``i`` of ref_testing.npz: (pars, person, contacts, test_prob kwargs, contact_tracing kwargs)."""
    pars = fix_pars(unjson(json.loads(str(d[f's{i}.pars']))))
    pars['interventions'] = []
    person = {k[len(f's{i}.person.'):]: v for k, v in d.items() if k.startswith(f's{i}.person.')}
    nl = len([k for k in d if k.startswith(f's{i}.L') and k.endswith('.p1')])
    keys = list(pars['beta_layer'].keys())
    contacts = {keys[li]: {c: d[f's{i}.L{li}.{c}'] for c in ('p1', 'p2', 'beta')} for li in range(nl)}
    ivs = json.loads(str(d[f's{i}.interventions']))
    return pars, person, contacts, ivs['test_prob'], ivs['contact_tracing']


def load_day(name):
    d = load_npz(f'ref_day_{name}.npz')
    pars = fix_pars(unjson(json.loads(str(d['pars']))))
    return d, pars


def snap(d, prefix):
    return {k: d[f'{prefix}.{k}'] for k in ALL_KEYS}


def oracle_people(d, prefix, pars):
    n = len(d[f'{prefix}.uid'])
    p = OraclePeople(pars, n)
    for k in ALL_KEYS:
        p[k] = np.array(d[f'{prefix}.{k}'], copy=True)
    return p


def n_layers(d):
    return len([k for k in d if k.startswith('d.L') and k.endswith('.p1')])


def assert_state_equal(get, ref, keys=ALL_KEYS, float_rtol=0.0, label=''):
    """``get(key)`` -> array; ``ref`` dict of reference arrays. Exact for ints/bools,
    ``float_rtol`` relative tolerance for floats (NaN must match NaN)."""
    for k in keys:
        a = np.asarray(get(k))
        b = np.asarray(ref[k])
        assert a.shape == b.shape, (label, k, a.shape, b.shape)
        if k in FLOAT_KEYS and float_rtol:
            assert np.array_equal(np.isnan(a), np.isnan(b)), (label, k, 'NaN pattern')
            m = ~np.isnan(b)
            np.testing.assert_allclose(a[m], b[m], rtol=float_rtol, atol=0, err_msg=f'{label} {k}')
        else:
            if a.dtype.kind == 'f' or b.dtype.kind == 'f':
                ok = np.array_equal(a.astype(np.float64), b.astype(np.float64), equal_nan=True)
            else:
                ok = np.array_equal(a.astype(np.int64), b.astype(np.int64))
            if not ok:
                bad = np.nonzero(~((a == b) | (np.isnan(a.astype(float)) & np.isnan(b.astype(float)))))
                raise AssertionError(f'{label} {k}: {len(bad[0])} mismatches, first at {bad[0][:5]}: '
                                     f'{a[bad][:5]} vs {b[bad][:5]}')


RES_KEYS = ['new_infections', 'new_reinfections', 'new_infectious', 'new_symptomatic', 'new_severe', 'new_critical',
            'new_recoveries', 'new_deaths', 'new_known_deaths', 'n_susceptible', 'n_exposed', 'n_infectious',
            'n_symptomatic', 'n_severe', 'n_critical', 'n_recovered', 'n_dead']


def _host(x):
    import torch
    return x.cpu().numpy() if torch.is_tensor(x) else x


def oracle_for(sim):
    """The oracle (Philox mode) for an initialised GPU Sim: the same population, layers and beta schedule."""
    import copy
    from oracle.sim import OracleSim
    spec = sim.spec
    contacts = {}
    for ly in spec.layers:
        p1 = _host(ly['p1'])
        beta = ly['beta'] if ly.get('beta') is not None else np.ones(len(p1), dtype=np.float32)
        contacts[ly['key']] = dict(p1=p1, p2=_host(ly['p2']), beta=_host(beta))
    pars = copy.deepcopy(sim.pars)
    pars['interventions'] = []
    return OracleSim(pars, {k: _host(v) for k, v in spec.person.items()}, contacts, rng='philox',
                     beta_schedule=spec.beta_sched)


def compare_runs(sim, orc, keys=RES_KEYS):
    """Every result series and the final agent state of a GPU run equal to the oracle's."""
    raw = sim.raw_results()
    for k in keys:
        np.testing.assert_array_equal(raw[k], orc.results[k], err_msg=k)
    np.testing.assert_allclose(raw['pop_nabs'], orc.results['pop_nabs'], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(raw['pop_protection'], orc.results['pop_protection'], rtol=1e-5, atol=1e-12)
    people_keys = [k for k in ALL_KEYS if k not in ('age', 'sex', 'uid', 'doses')]
    assert_state_equal(lambda k: sim.people.gpu(k).cpu().numpy(), {k: orc.people[k] for k in people_keys},
                       keys=people_keys, float_rtol=1e-6, label='final state')
