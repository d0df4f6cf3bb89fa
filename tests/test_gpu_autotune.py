"""The edge tile is a pure performance knob: every supported tile size gives
bit-identical runs (with testing and tracing, whose edge scan uses the same
tiles), and the autotuner picks one of them and leaves the sim runnable."""
import numpy as np
import pytest

import covasim_gb300 as cv
from covasim_gb300 import _lib as L
from test_gpu_testing import TESTING_KEYS, make_sim, CASES

pytestmark = pytest.mark.gpu


def test_every_edge_tile_gives_the_same_run():
    """Every tile size, the one-wave stored-layer pass (as many blocks per SM as fit,
    and one or two), and the resident-bitmap variant, with testing and tracing."""
    ref = None
    variants = ([str(t) for t in L.EDGE_TILES] + [f'{t}w' for t in L.EDGE_TILES] + ['1024w1', '4096w2']
                + ['4096r', '8192r'])
    for label in variants:
        sim = make_sim(*CASES[0])
        sim.initialize()
        assert sim.state.resident_possible()
        sim.state.apply_edge_tile(label)
        assert str(sim.state.edge_tile_label) == label
        raw = sim.run().raw_results()
        if ref is None:
            ref = raw
        else:
            for k in TESTING_KEYS:
                np.testing.assert_array_equal(raw[k], ref[k], err_msg=f'edge pass {label} {k}')


def test_wave_pass_over_a_batch_equals_single_runs():
    """The one-wave pass over many sims' segments (shares cross sims and layers)."""
    pars = [dict(pop_type='hybrid', pop_size=n, n_days=30, rand_seed=s, pop_infected=50)
            for n, s in ((3000, 1), (9000, 2), (500, 3), (6000, 4))]
    solo = [cv.Sim(p).run().raw_results() for p in pars]
    for label in ('1024w', '8192w', '2048w3'):
        batch = cv.BatchSim([cv.Sim(p) for p in pars], edge_tile=label).run()
        for k in range(len(pars)):
            got = batch.results(k)
            for key in ('new_infections', 'new_recoveries', 'n_susceptible', 'n_exposed', 'pop_nabs'):
                np.testing.assert_array_equal(got[key], solo[k][key], err_msg=f'{label} sim {k} {key}')


def test_resident_variant_with_the_likelihood_matches():
    from covasim_gb300.adjoint import LikelihoodRun
    out = []
    for label in ('4096', '4096r', '1024w'):
        sim = cv.Sim(pop_type='hybrid', pop_size=6000, n_days=40, rand_seed=3, pop_infected=40,
                     dynam_layer=dict(h=0, s=0, w=0, c=1))
        sim.initialize()
        sim.state.apply_edge_tile(label)
        run = LikelihoodRun(sim, checkpoint_every=10)
        ll, e = run.forward(run.params.theta0)
        out.append((ll, e, run.backward(1.0, np.ones(run.npts))))
    l0, e0, g0 = out[0]
    for l1, e1, g1 in out[1:]:
        assert abs(l0 - l1) <= 1e-9 * abs(l0)
        np.testing.assert_allclose(e0, e1, rtol=1e-9)
        np.testing.assert_allclose(g0, g1, rtol=1e-9)


def test_resident_variant_is_refused_for_batches():
    sims = [cv.Sim(pop_type='random', pop_size=2000, n_days=10, rand_seed=s) for s in (1, 2)]
    batch = cv.BatchSim(sims).initialize()
    assert not batch.state.resident_possible()
    with pytest.raises(ValueError):
        batch.state.set_edge_tile(4096, resident=True)


def test_autotuned_sim_equals_default_run():
    pars = dict(pop_type='hybrid', pop_size=20000, n_days=40, rand_seed=4, dynam_layer=dict(h=0, s=0, w=0, c=1))
    a = cv.Sim(pars).run().raw_results()
    s = cv.Sim(pars, edge_tile='auto')
    s.initialize()
    assert s.state.edge_tile in L.EDGE_TILES and s.state.edge_tile_label is not None
    b = s.run().raw_results()
    for k in ('new_infections', 'n_exposed', 'new_deaths'):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
