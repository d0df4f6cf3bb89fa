"""The quiet-day walk of the stored layers (covgpu_state.src_walk) is a pure
performance choice: walking every indexed stored layer from the day's sources
(-1), streaming every edge (0, the default without a redrawn layer) and the
per-day choice (8 or 128, the default with a redrawn layer: walk while a sim's
infectious agents are under that fraction of its agents) queue the same
candidates and draw, key and claim them alike, so whole runs are bit-identical,
with testing and tracing, in batches and with the likelihood passes; with a
redrawn layer the walk runs in that layer's launch, otherwise in its own."""
import numpy as np
import pytest

import covasim_gb300 as cv
from common import ALL_KEYS, RES_KEYS, assert_state_equal
from test_gpu_testing import TESTING_KEYS, make_sim, CASES

pytestmark = pytest.mark.gpu

MODES = (0, -1, 8, 128)
PEOPLE_KEYS = [k for k in ALL_KEYS if k not in ('age', 'sex', 'uid', 'doses')]


def _run(make, mode):
    sim = make()
    sim.initialize()
    sim.state.set_src_walk(mode)
    assert sim.state.src_walk == mode
    sim.run()
    return sim


def test_walk_default_follows_the_redrawn_layers():
    hybrid = cv.Sim(pop_type='hybrid', pop_size=3000, n_days=5, dynam_layer=dict(h=0, s=0, w=0, c=1)).initialize()
    assert hybrid.state.src_walk == 128
    plain = cv.Sim(pop_type='random', pop_size=3000, n_days=5).initialize()
    assert plain.state.src_walk == 0


@pytest.mark.parametrize('tile', ['2048w', '4096', '8192r'])
def test_walked_and_streamed_runs_are_identical(tile):
    """Hybrid with waning and the community layer redrawn: the epidemic passes
    through quiet and busy days, so mode 8 uses both paths."""
    pars = dict(pop_type='hybrid', pop_size=30000, n_days=90, rand_seed=6, pop_infected=30, use_waning=True,
                dynam_layer=dict(h=0, s=0, w=0, c=1))
    sims = [_run(lambda: cv.Sim(pars, edge_tile=tile), m) for m in MODES]
    ref = sims[0].raw_results()
    peak = ref['n_infectious'].max() / 30000
    assert peak > 1 / 8, peak  # mode 8 streams on the busiest days
    for sim, m in zip(sims[1:], MODES[1:]):
        raw = sim.raw_results()
        for k in RES_KEYS:
            np.testing.assert_array_equal(raw[k], ref[k], err_msg=f'src_walk {m}: {k}')
        assert_state_equal(lambda k: sim.people.gpu(k).cpu().numpy(),
                           {k: sims[0].people.gpu(k).cpu().numpy() for k in PEOPLE_KEYS},
                           keys=PEOPLE_KEYS, label=f'src_walk {m}')


def test_walk_with_testing_and_tracing():
    ref = None
    for m in MODES:
        raw = _run(lambda: make_sim(*CASES[0]), m).raw_results()
        if ref is None:
            ref = raw
            continue
        for k in TESTING_KEYS:
            np.testing.assert_array_equal(raw[k], ref[k], err_msg=f'src_walk {m}: {k}')


def test_walk_in_a_batch():
    """Sims of different sizes and seeds in one state: each sim's path is chosen
    from its own infectious count."""
    def batch(mode):
        sims = [cv.Sim(pop_type='random', pop_size=n, n_days=50, rand_seed=s, pop_infected=20)
                for n, s in ((4000, 1), (9000, 2), (2500, 3))]
        b = cv.BatchSim(sims).initialize()
        b.state.set_src_walk(mode)
        return b.run()
    runs = [batch(m) for m in MODES]
    for b, m in zip(runs[1:], MODES[1:]):
        for k in range(3):
            for key in RES_KEYS:
                np.testing.assert_array_equal(b.results(k)[key], runs[0].results(k)[key],
                                              err_msg=f'src_walk {m}: sim {k} {key}')


def test_walk_with_the_likelihood():
    from covasim_gb300.adjoint import LikelihoodRun
    out = []
    for m in (0, -1):
        sim = cv.Sim(pop_type='hybrid', pop_size=6000, n_days=40, rand_seed=3, pop_infected=40,
                     dynam_layer=dict(h=0, s=0, w=0, c=1))
        sim.initialize()
        sim.state.set_src_walk(m)
        run = LikelihoodRun(sim)
        ll, e = run.forward(run.params.theta0)
        out.append((ll, e, run.backward(1.0, np.ones(run.npts))))
    (l0, e0, g0), (l1, e1, g1) = out
    assert abs(l0 - l1) <= 1e-9 * abs(l0)
    np.testing.assert_allclose(e0, e1, rtol=1e-9)
    np.testing.assert_allclose(g0, g1, rtol=1e-9)
