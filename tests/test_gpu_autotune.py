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
    ref = None
    for tile in L.EDGE_TILES:
        sim = make_sim(*CASES[0])
        sim.edge_tile = tile
        raw = sim.run().raw_results()
        if ref is None:
            ref = raw
        else:
            for k in TESTING_KEYS:
                np.testing.assert_array_equal(raw[k], ref[k], err_msg=f'tile {tile} {k}')


def test_autotuned_sim_equals_default_run():
    pars = dict(pop_type='hybrid', pop_size=20000, n_days=40, rand_seed=4, dynam_layer=dict(h=0, s=0, w=0, c=1))
    a = cv.Sim(pars).run().raw_results()
    s = cv.Sim(pars, edge_tile='auto')
    s.initialize()
    assert s.state.edge_tile in L.EDGE_TILES
    b = s.run().raw_results()
    for k in ('new_infections', 'n_exposed', 'new_deaths'):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
