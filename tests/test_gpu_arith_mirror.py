"""The float-float NAb arithmetic (as the CUDA library does it, mirrored in
numpy) against the reference's float64 calc_VE and update_nab, rounded to float32."""
import numpy as np

from oracle import gpu_arith as ga
from oracle.people import calc_VE

NAB_EFF = dict(alpha_inf=1.08, beta_inf=0.967, alpha_symp_inf=-0.739, beta_symp_inf=0.038, alpha_sev_symp=-0.014,
               beta_sev_symp=0.079)
AXES = {'sus': ('alpha_inf', 'beta_inf'), 'symp': ('alpha_symp_inf', 'beta_symp_inf'),
        'sev': ('alpha_sev_symp', 'beta_sev_symp')}


def test_calc_ve_float_float_rounds_like_the_reference():
    rng = np.random.default_rng(11)
    nab = np.concatenate([rng.lognormal(0, 3, 400_000),
                          [1e-35, 1e-20, 1e-10, 1e-5, 0.5, 1.0, 2.0, 10, 100, 1e4, 1e7, 3e-38]]).astype(np.float32)
    imm = rng.choice([1.0, 0.5, 0.066, 0.374, 0.8, 0.34], len(nab)).astype(np.float32)
    eff = nab.astype(np.float64) * imm.astype(np.float64)
    lnh, lnl = ga.ff_log(nab)
    logs = {v: ga.split_log(v) for v in np.unique(imm)}
    lih = np.array([logs[v][0] for v in imm], np.float32)
    lil = np.array([logs[v][1] for v in imm], np.float32)
    eh, el = ga.ff_add(lnh, lnl, lih, lil)
    for ax, (a, b) in AXES.items():
        ref = calc_VE(eff, ax, NAB_EFF).astype(np.float32)
        got = ga.ve_ff(eh, el, NAB_EFF[a], NAB_EFF[b])
        ulps = np.abs(got.view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64))
        assert ulps.max() <= 1, ax
        assert (ulps > 0).mean() < 1e-5, (ax, (ulps > 0).sum())


def test_update_nab_float_float_rounds_like_the_reference():
    rng = np.random.default_rng(12)
    n = 300_000
    kin = np.concatenate([rng.normal(0, 0.05, n // 2), 1 / 21 * np.ones(n // 2)])
    peak = rng.lognormal(0, 2, n).astype(np.float32)
    nab0 = (peak * rng.random(n)).astype(np.float32)
    ref = (nab0.astype(np.float64) + kin * peak.astype(np.float64)).astype(np.float32)
    ref = np.where(ref < 0, 0, ref)
    ref = np.where(ref > peak, peak, ref).astype(np.float32)
    kh, kl = ga.split_kin(kin)
    got = ga.update_nab_ff(nab0, peak, kh, kl)
    assert (got != ref).sum() <= 2


def test_tables_match_the_cuda_header():
    import os
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    h = open(os.path.join(root, 'covasim_gb300', 'csrc', 'covgpu_tables.h')).read()
    vals = [float.fromhex(x[:-1]) for x in re.findall(r'-?0x[0-9a-f.]+p[-+]\d+f', h)]
    consts = [ga.LN2_HI, ga.LN2_LO, ga.LN2_LO2, ga.INV_LN2_64, ga.LN2_64_HI, ga.LN2_64_MID, ga.LN2_64_LO]
    assert vals[:7] == [float(c) for c in consts]
    tab = np.array(vals[7:], dtype=np.float32)
    n_ln, n_exp = 2 * len(ga.LN_TAB), 2 * len(ga.EXP_TAB)
    assert np.array_equal(tab[:n_ln].reshape(-1, 2), ga.LN_TAB)
    assert np.array_equal(tab[n_ln:n_ln + n_exp].reshape(-1, 2), ga.EXP_TAB)
    rest = tab[n_ln + n_exp:]
    assert list(rest[:4]) == [ga.PI_2_HI, ga.PI_2_LO, ga.LN2_FF_HI, ga.LN2_FF_LO]
    n_sc = ga.SINCOS_TAB.size
    assert np.array_equal(rest[4:4 + n_sc].reshape(-1, 4), ga.SINCOS_TAB)
    assert np.array_equal(rest[4 + n_sc:], ga.LN_INV)


def test_float_float_infection_draws_track_float64():
    """Box-Muller, exp and the duration samples in float-float (the GPU's infect
    arithmetic) against the reference's float64 formulas."""
    rng = np.random.default_rng(5)
    a = rng.integers(0, 2 ** 32, 300_000, dtype=np.uint64)
    b = rng.integers(0, 2 ** 32, 300_000, dtype=np.uint64)
    (z0h, z0l), (z1h, z1l) = ga.box_muller_ff(a, b)
    u1, u2 = (a.astype(np.float64) + 0.5) * 2.0 ** -32, (b.astype(np.float64) + 0.5) * 2.0 ** -32
    r = np.sqrt(-2 * np.log(u1))
    assert np.abs(ga.ff2d(z0h, z0l) - r * np.cos(2 * np.pi * u2)).max() < 1e-12
    assert np.abs(ga.ff2d(z1h, z1l) - r * np.sin(2 * np.pi * u2)).max() < 1e-12
    z = rng.standard_normal(300_000)
    for dist in (dict(dist='lognormal_int', par1=4.5, par2=1.5), dict(dist='lognormal_int', par1=18.1, par2=6.3),
                 dict(dist='normal_int', par1=3.0, par2=2.0)):
        code, m, s = ga.dist_code(dist)
        ref = np.round(np.exp(m + s * z)) if code == 0 else np.round(np.abs(m + s * z))
        assert np.array_equal(ga.sample_ff(dist, *ga.d2ff(z)), ref), dist
    x = rng.normal(0, 2, 300_000)
    assert np.abs(ga.exp2_ff(x) / 2 ** x - 1).max() < 1e-11
    rint_in = np.array([2.5, 3.5, -2.5, 2.0, 2.0, 7.5], dtype=np.float32)
    rint_lo = np.array([0, 0, 0, -1e-9, 1e-9, 1e-9], dtype=np.float32)
    assert list(ga.ff_rint(rint_in, rint_lo)) == [2, 4, -2, 2, 2, 8]
