"""GPU parity of the standalone kernels (covgpu_viral_load / _trans_sus / _infections)
against the reference's own outputs and against the oracle."""
import numpy as np
import pytest
import torch

import covasim_gb300 as cv
from common import load_npz
from oracle import kernels as ok
from oracle import philox as ph

pytestmark = pytest.mark.gpu


def test_viral_load_bit_exact_vs_reference():
    d = load_npz('ref_kernels.npz')
    for i, (t, fr, lr, hc) in enumerate(d['vl.cases']):
        out = cv.compute_viral_load(int(t), d['vl.ts'], d['vl.rec'], d['vl.dead'], fr, lr, hc)
        assert out.dtype == np.float32
        assert np.array_equal(out, d[f'vl{i}.out'], equal_nan=True), i


def test_trans_sus_bit_exact_vs_reference():
    d = load_npz('ref_kernels.npz')
    for i, (bl, af, isf, qf) in enumerate(d['ts.cases']):
        a, b = cv.compute_trans_sus(d['ts.rt'], d['ts.rs'], d['ts.inf'], d['ts.sus'], bl, d['ts.vl'], d['ts.symp'],
                                    d['ts.iso'], d['ts.quar'], af, isf, qf, d['ts.imm'])
        assert np.array_equal(a, d[f'ts{i}.rel_trans']), i
        assert np.array_equal(b, d[f'ts{i}.rel_sus']), i


def test_infections_exact_vs_reference_draws():
    """Same sources and targets, in the reference's order, given the reference's draws."""
    d = load_npz('ref_kernels.npz')
    for i, beta in enumerate(d['inf.betas']):
        src, tgt = cv.compute_infections(np.float32(beta), d[f'inf{i}.p1'], d[f'inf{i}.p2'], d[f'inf{i}.lb'],
                                         d[f'inf{i}.rt'], d[f'inf{i}.rs'], uniforms=d[f'inf{i}.U'])
        assert np.array_equal(src, d[f'inf{i}.src']), i
        assert np.array_equal(tgt, d[f'inf{i}.tgt']), i


@pytest.mark.parametrize('E,frac', [(1, 1.0), (4097, 0.3), (300_000, 0.05), (2_000_000, 0.01)])
def test_infections_philox_exact_vs_oracle(E, frac):
    rng = np.random.default_rng(E)
    n = max(10, E // 8)
    p1 = np.sort(rng.integers(0, n, E)).astype(np.int32)
    p2 = rng.integers(0, n, E).astype(np.int32)
    lb = np.where(rng.random(E) < 0.7, 1.0, rng.random(E)).astype(np.float32)
    rt = np.where(rng.random(n) < frac, rng.random(n), 0).astype(np.float32)
    rs = np.where(rng.random(n) < 0.8, rng.random(n), 0).astype(np.float32)
    seed, day, variant, layer = 12345, 7, 1, 3
    src, tgt = cv.compute_infections(np.float32(0.2), p1, p2, lb, rt, rs, seed=seed, day=day, variant=variant,
                                     layer=layer)
    k0, k1 = ph.seed_key(seed)
    u0, u1 = ph.edge_uniforms(k0, k1, day, layer, variant, np.arange(E))
    osrc, otgt = ok.compute_infections(np.float32(0.2), p1, p2, lb, rt, rs, np.stack([u0, u1]))
    assert np.array_equal(src, osrc) and np.array_equal(tgt, otgt)


def test_empty_and_torch_inputs():
    e = np.zeros(0, np.int32)
    src, tgt = cv.compute_infections(0.1, e, e, np.zeros(0, np.float32), np.ones(5, np.float32),
                                     np.ones(5, np.float32))
    assert len(src) == 0 and len(tgt) == 0
    ts = torch.tensor([0.0, 1.0, float('nan')], device='cuda')
    out = cv.compute_viral_load(3, ts, ts + 10, torch.full_like(ts, float('nan')), 0.3, 2.0, 4.0)
    assert torch.is_tensor(out) and out.is_cuda
    ref = ok.compute_viral_load(3, ts.cpu().numpy(), ts.cpu().numpy() + 10, np.full(3, np.nan, np.float32), 0.3, 2.0,
                                4.0)
    assert np.array_equal(out.cpu().numpy(), ref, equal_nan=True)
