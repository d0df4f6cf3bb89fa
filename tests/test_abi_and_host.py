"""CPU checks of the C ABI and the host-side logic (no kernel launches)."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

import covasim_gb300 as cv
from covasim_gb300 import _lib as L
from covasim_gb300 import build as B
from common import GOLDEN, unjson

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'covgpu.h')).read()
    return sorted(set(re.findall(r'^\s*(?:int|int64_t)\s+(covgpu_\w+)\s*\(', src, flags=re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    B.build()
    lib = C.CDLL(B.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(L.EXPORTED) == syms


def test_abi_layout_matches_ctypes_mirror():
    lib_vals, mine = L.abi_layout()
    assert lib_vals == mine


def test_entry_points_reject_bad_arguments_without_a_gpu():
    lib = L.lib()
    # rejected on the host before any CUDA call
    assert lib.covgpu_viral_load(0, None, None, None, -1, 0.3, 2.0, 4.0, None, None) == L.BADARG
    assert lib.covgpu_infections_scratch_bytes(-5) == -1
    assert lib.covgpu_infections(0.1, None, None, None, 10, None, None, 5, None, 0, 0, 0, 0, None, None, 0, None,
                                 None, None, 0, None) == L.BADARG
    assert lib.covgpu_agent_step(None, 0, 1, 1, None) == L.BADARG
    assert lib.covgpu_run_days(None, 0, 10, 0, 1, 1, None) == L.BADARG
    st = L.State()
    assert lib.covgpu_edge_pass(C.pointer(st), 0, None) == L.BADARG
    assert lib.covgpu_import_day(None, 0, None) == L.BADARG
    assert lib.covgpu_import_day(C.pointer(st), 0, None) == L.BADARG
    assert lib.covgpu_rescale_check(None, 0, None) == L.BADARG
    assert lib.covgpu_rescale_check(C.pointer(st), 0, None) == L.BADARG
    assert lib.covgpu_layer_lists(None, 0, 0, 0, 10, None, None, None, None) == L.BADARG
    assert lib.covgpu_check(None, 0, L.CHECK_DEATH, 0, 1, None, 0, 10, None, 0, None, None) == L.BADARG
    assert lib.covgpu_check_immunity(C.pointer(st), 0, 0, 1, None) == L.BADARG
    assert lib.covgpu_update_nab(None, 0, 0, None, 5, None) == L.BADARG
    assert lib.covgpu_update_peak_nab(None, 0, 0, None, 5, None, L.DurPar(2, 0, 0.0, 2.0), 1.5, 1.0, 2,
                                      None) == L.BADARG


def test_day_path_is_registered_as_torch_custom_ops():
    """Every day-path entry point the state calls is a torch.ops.covgpu operator
    (registration needs no GPU)."""
    import torch
    import covasim_gb300  # noqa: F401
    for name in ('compute_viral_load', 'compute_trans_sus', 'compute_infections', 'agent_step', 'edge_pass',
                 'infect_claims', 'infect_list', 'import_day', 'test_trace', 'lik_targets', 'rescale_check',
                 'run_days', 'layer_lists', 'check', 'check_immunity', 'update_nab', 'update_peak_nab'):
        assert hasattr(torch.ops.covgpu, name), name


def test_dynamic_layer_count_table_matches_the_oracle():
    """The list-length table of a redrawn layer (Binomial(E, 1/n) thresholds) is
    the same in the library's host code and in the oracle, and is a distribution."""
    from covasim_gb300.state import dynamic_count_table
    from oracle.philox import dyn_count_table
    from scipy.stats import binom
    for E, n in [(10_000_000, 1_000_000), (300, 30), (5, 1), (123_457, 5001), (15 * 20_000, 20_000)]:
        a, b = dynamic_count_table(E, n), dyn_count_table(E, n)
        np.testing.assert_array_equal(a, b)
        assert a[-1] == 2 ** 64 - 1 and np.all(np.diff(a.astype(object)) >= 0)
        k = np.arange(len(a) - 1)
        np.testing.assert_allclose(a[:-1].astype(np.float64) / 2.0 ** 64, binom.cdf(k, E, 1 / n), rtol=1e-9, atol=1e-15)


def _same(got, want, path):
    if isinstance(want, dict):
        assert isinstance(got, dict), path
        want_keys = {str(k) for k in want}
        got_keys = {str(k) for k in got}
        assert want_keys == got_keys, (path, want_keys ^ got_keys)
        gmap = {str(k): v for k, v in got.items()}
        for k, v in want.items():
            _same(gmap[str(k)], v, f'{path}.{k}')
    elif isinstance(want, (list, tuple)) and not (want and isinstance(want[0], (int, float))):
        assert len(got) == len(want), path
        for i, (g, w) in enumerate(zip(got, want)):
            _same(g, w, f'{path}[{i}]')
    elif isinstance(want, str) or want is None or isinstance(want, bool):
        assert got == want, (path, got, want)
    else:
        np.testing.assert_array_equal(np.asarray(got, dtype=float), np.asarray(want, dtype=float), err_msg=path)


def test_make_pars_matches_reference_values():
    ref = json.load(open(os.path.join(GOLDEN, 'ref_pars.json')))
    for pop_type in ('random', 'hybrid'):
        want = unjson(ref[pop_type])
        got = cv.make_pars(pop_type=pop_type)
        got['prognoses'] = cv.get_prognoses(True)
        cv.init_immunity(got, int(got['n_days']) + 1)
        for k, v in want.items():
            if k in ('verbose', 'interventions', 'analyzers', 'variants'):
                continue
            _same(got[k], v, f'{pop_type}.{k}')
    want3 = np.asarray(unjson(ref['immunity_3var']))
    p = cv.make_pars(pop_type='hybrid')
    p['variant_map'] = {0: 'wild', 1: 'alpha', 2: 'delta'}
    p['variant_pars'] = {k: cv.get_variant_pars(variant=k) for k in ('wild', 'alpha', 'delta')}
    p['n_variants'] = 3
    cv.init_immunity(p, 61, create=True)
    np.testing.assert_array_equal(p['immunity'], want3)


def test_population_generators_follow_reference_distributions():
    pars = cv.make_pars(pop_type='hybrid', pop_size=200_000, rand_seed=3)
    pop = cv.make_randpop(pars, rng=np.random.default_rng(3))
    age = pop['age']
    assert 36 < np.median(age) < 39
    n = len(age)
    # community: round(Poisson(20)/2) per agent -> mean 10 undirected edges per agent
    c = pop['contacts']['c']
    assert abs(len(c['p1']) / n - 10.0) < 0.05
    assert np.all(np.diff(c['p1']) >= 0)
    # households: Poisson(2) cluster sizes, all pairs within a cluster
    h = pop['contacts']['h']
    assert np.all(h['p2'] > h['p1'])
    s_inds = np.nonzero((age >= 6) & (age < 22))[0]
    s = pop['contacts']['s']
    assert np.isin(s['p1'], s_inds).all() and np.isin(s['p2'], s_inds).all()
    w = pop['contacts']['w']
    w_inds = np.nonzero((age >= 22) & (age < 65))[0]
    assert abs(len(w['p1']) / len(w_inds) - 8.0) < 0.1
    # mean household-layer degree: E[m(m-1)/2]/E[m] with m ~ Poisson(2) -> 1.0 edge per agent
    assert abs(len(h['p1']) / n - 1.0) < 0.03


def test_prognoses_and_rel_trans_distribution():
    pars = cv.make_pars(pop_size=100_000)
    pars['prognoses'] = cv.get_prognoses(True)
    age = cv.sample_ages(100_000, np.random.default_rng(0))
    from covasim_gb300.population import set_prognoses
    out = set_prognoses(age, pars, np.random.default_rng(1))
    rt = out['rel_trans']
    assert abs(rt.mean() - 1.0) < 0.03
    assert 0.06 < (rt == 0).mean() < 0.12  # negative binomial(mean 1, dispersion 0.45, step 0.01) has P(0) ~ 9%


def test_change_beta_schedule():
    sim = cv.Sim(pop_size=100, n_days=40, interventions=[cv.change_beta(days=[10, 30], changes=[0.5, 0.8]),
                                                       cv.change_beta(days=20, changes=0.1, layers='a')])
    sim.validate_pars()
    sim.init_interventions()
    from covasim_gb300.sim import build_spec
    pars = sim.pars
    pars['prognoses'] = cv.get_prognoses(True)
    cv.init_immunity(pars, sim.npts)
    spec, _, _ = build_spec(pars, None, None, pars['interventions'])
    b = spec.beta_sched
    assert b[9] == 0.016 and b[10] == 0.016 * 0.5 and b[29] == 0.016 * 0.5 and b[30] == 0.016 * 0.8
    bl = spec.beta_layer_sched[:, 0]
    assert bl[19] == 1.0 and bl[20] == 0.1 and bl[40] == 0.1


def test_daily_importations_schedule():
    """sim.py:582-587 drawn ahead of the run: Poisson counts, distinct agents in
    range, the same schedule as the oracle's philox mode, and the reference's
    error for a count above the population."""
    from covasim_gb300.state import daily_importations
    from oracle.sim import philox_mode_importations
    days = daily_importations(7, 2.5, 1000, 400)
    counts = np.array([len(d) for d in days])
    assert abs(counts.mean() - 2.5) < 4 * np.sqrt(2.5 / 400) and abs(counts.var() - 2.5) < 0.6
    for t, d in enumerate(days):
        assert len(np.unique(d)) == len(d) and (d >= 0).all() and (d < 1000).all()
        np.testing.assert_array_equal(d, philox_mode_importations(7, 2.5, 1000, t))
    assert [len(d) for d in daily_importations(8, 2.5, 1000, 50)] != list(counts[:50])
    with pytest.raises(ValueError):
        daily_importations(1, 50, 5, 3)


def test_importation_redraw_from_a_day_and_variant_counts():
    """After a rescaling on day s the schedule is redrawn from s on with the new
    rates: the days before s keep their draws, the redrawn days equal a full draw
    with the new rates; a variant's importations at a scale (immunity.py:121-124)."""
    from covasim_gb300.state import daily_importations
    from covasim_gb300.sim import variant_import_count
    n, npts, s = 5000, 60, 25
    rates = np.full(npts, 4.0)
    full = daily_importations(3, rates, n, npts)
    rates[s:] /= 2.5
    tail = daily_importations(3, rates, n, npts, start=s)
    again = daily_importations(3, rates, n, npts)
    assert len(tail) == npts - s
    for t in range(npts):
        np.testing.assert_array_equal(again[t], full[t] if t < s else tail[t - s])
    assert sum(len(d) for d in tail) < sum(len(d) for d in full[s:])

    class V:
        n_imports, rescale = 10, True
    rng = np.random.default_rng(1)
    assert variant_import_count(V, 1.0, rng) == 10 and variant_import_count(V, 2.0, rng) == 5
    counts = [variant_import_count(V, 3.0, np.random.default_rng(k)) for k in range(2000)]
    assert set(counts) == {3, 4} and abs(np.mean(counts) - 10 / 3) < 0.05
    V.rescale = False
    assert variant_import_count(V, 3.0, rng) == 10


def test_infection_log_layer_tags_round_trip():
    """people.py:508-511 records the infect() call's layer: contact layers by index,
    seed infections, importations, None and other labels by their own tags."""
    from covasim_gb300.people import log_layer_tag, log_layer_label
    keys, extra = ['h', 's', 'w', 'c'], []
    for layer in keys + ['seed_infection', 'importation', None, 'custom', 'other', 'custom']:
        tag = log_layer_tag(layer, keys, extra)
        assert 0 <= tag <= 0xFF and log_layer_label(tag, keys, extra) == layer
    assert extra == ['custom', 'other']
    assert log_layer_tag('seed_infection', keys, extra) == L.LOG_SEED
    assert log_layer_tag('importation', keys, extra) == L.LOG_IMPORT


def test_test_prob_subtarget_and_ili_inputs():
    """get_subtargets (interventions.py:150-187) with fixed indices and values and
    process_daily_data (interventions.py:111-147) for ILI prevalence, as the host
    prepares them; the ILI agents are the oracle's draws in its Philox mode."""
    from covasim_gb300.interventions import test_prob
    from covasim_gb300.state import ili_agents
    from oracle.interventions import ili_agents as oracle_ili
    inds, vals = test_prob._fixed_subtarget(dict(inds=[4, 9, 2], vals=0.25), 10)
    np.testing.assert_array_equal(inds, [4, 9, 2])
    np.testing.assert_array_equal(vals, [0.25, 0.25, 0.25])
    inds, vals = test_prob._fixed_subtarget(dict(inds=np.array([1, 3]), vals=[0.1, 0.9]), 10)
    np.testing.assert_array_equal(vals, [0.1, 0.9])
    with pytest.raises(ValueError):
        test_prob._fixed_subtarget(dict(inds=[1, 2], vals=[0.1]), 10)
    with pytest.raises(ValueError):
        test_prob._fixed_subtarget(dict(vals=[0.1]), 10)
    with pytest.raises(ValueError):
        test_prob._fixed_subtarget(dict(inds=[10], vals=0.5), 10)
    with pytest.raises(NotImplementedError):
        test_prob._fixed_subtarget(dict(inds=lambda sim: [1], vals=0.5), 10)
    np.testing.assert_array_equal(test_prob._daily(0.02, 4), [0.02] * 4)
    np.testing.assert_array_equal(test_prob._daily([0.01, 0.03], 10), [0.01, 0.03])
    with pytest.raises(NotImplementedError):
        test_prob._daily('data', 10)
    for seed, t, n, k in ((1, 0, 1000, 20), (7, 33, 5000, 250), (3, 2, 10, 10)):
        got = ili_agents(seed, t, n, k)
        assert len(np.unique(got)) == k and got.min() >= 0 and got.max() < n
        np.testing.assert_array_equal(got, oracle_ili(seed, t, n, k))


def test_edge_pass_labels_parse():
    """The edge-pass labels the autotuner and Sim(edge_tile=...) take."""
    from covasim_gb300.state import parse_edge_tile
    assert parse_edge_tile(4096) == dict(tile=4096)
    assert parse_edge_tile('8192') == dict(tile=8192)
    assert parse_edge_tile('8192r') == dict(tile=8192, resident=True)
    assert parse_edge_tile('2048w') == dict(tile=2048, wave=True)
    assert parse_edge_tile('1024w4') == dict(tile=1024, wave=4)
    assert parse_edge_tile(L.EDGE_TILE) == dict(tile=2048, wave=True)  # the default
    assert L.DAY_STEADY == 2
