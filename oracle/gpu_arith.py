"""numpy mirror of the CUDA library's float-float arithmetic.

TEST INFRASTRUCTURE ONLY (part of the CPU oracle).

GB300 executes float64 at a small fraction of its float32 rate, so the CUDA
library evaluates the reference's float64 NAb-efficacy (immunity.py:216-247
calc_VE) and update_nab (immunity.py:205-213) in float-float arithmetic and
rounds once to float32, and decides the Bernoulli test u < p of utils.py:123
exactly in integers. This module performs the same IEEE float32 operations in
the same order (the fused multiply-adds of the GPU code only form exact
product residuals, which float64 reproduces exactly), so an oracle run in its
'gpu' arithmetic mode agrees with the GPU bit for bit. Both stay within
rounding of the reference's float64 values (tested against them).

Tables (ln of the reduction points, 2^(j/64), split constants) are generated
with Python's decimal module, as the CUDA header's are.
"""
import math
import struct
from decimal import Decimal, getcontext

import numpy as np

F32 = np.float32
getcontext().prec = 50


def _f32(x):
    return struct.unpack('<f', struct.pack('<f', float(x)))[0]


def _split(d):
    hi = _f32(d)
    return hi, _f32(d - Decimal(hi))


LN_J0, LN_J1, EXP_N = -40, 55, 64
_LN2 = Decimal(2).ln()
LN_TAB = np.array([_split((Decimal(1) + Decimal(j) / Decimal(128)).ln()) for j in range(LN_J0, LN_J1 + 1)], F32)
EXP_TAB = np.array([_split((Decimal(j) / Decimal(EXP_N) * _LN2).exp()) for j in range(EXP_N)], F32)
_ln2_hi = float(round(_LN2 * 2 ** 16) / Decimal(2 ** 16))
LN2_HI = F32(_ln2_hi)
LN2_LO = F32(_f32(_LN2 - Decimal(_ln2_hi)))
LN2_LO2 = F32(_f32(_LN2 - Decimal(_ln2_hi) - Decimal(float(LN2_LO))))
INV_LN2_64 = F32(_f32(Decimal(64) / _LN2))
_c = _LN2 / Decimal(64)
_be = math.floor(math.log2(float(_c)))
_c_hi = float(round(_c / Decimal(2) ** (_be - 10)) * Decimal(2) ** (_be - 10))
LN2_64_HI = F32(_c_hi)
LN2_64_MID = F32(_f32(_c - Decimal(_c_hi)))
LN2_64_LO = F32(_f32(_c - Decimal(_c_hi) - Decimal(float(LN2_64_MID))))


# ----------------------------------------------------------------- float-float primitives (vectorised)
def _a(x):
    return np.asarray(x, dtype=F32)


def two_sum(a, b):
    a, b = _a(a), _a(b)
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def fast_two_sum(a, b):
    a, b = _a(a), _a(b)
    s = a + b
    return s, b - (s - a)


def two_prod(a, b):
    a, b = _a(a), _a(b)
    p = a * b
    e = (a.astype(np.float64) * b.astype(np.float64) - p.astype(np.float64)).astype(F32)  # exact residual
    return p, e


def ff_add(xh, xl, yh, yl):
    s, e = two_sum(xh, yh)
    return fast_two_sum(s, e + (_a(xl) + _a(yl)))


def ff_mul(xh, xl, yh, yl):
    p, e = two_prod(xh, yh)
    return fast_two_sum(p, e + (_a(xh) * _a(yl) + _a(xl) * _a(yh)))


def ff_div(ah, al, bh, bl):
    ah, al, bh, bl = _a(ah), _a(al), _a(bh), _a(bl)
    q1 = ah / bh
    ph, pl = two_prod(q1, bh)
    r = (ah - ph) - pl
    r = r + al
    r = r - q1 * bl
    return fast_two_sum(q1, r / bh)


def _fma_residual_div(rh, c, d):
    """fmaf(-rh, c, d) / c: the residual d - rh*c is exact in float64 and in float32."""
    res = (d.astype(np.float64) - rh.astype(np.float64) * c.astype(np.float64)).astype(F32)
    return res / c


# ----------------------------------------------------------------- ln, exp, VE, update_nab
def ff_log(x):
    """ln(x) for finite x > 0 as (hi, lo), as covgpu_ff.cuh ff_log computes it."""
    x = _a(x).copy()
    sub = x < F32(1.17549435e-38)
    x = np.where(sub, x * F32(16777216.0), x).astype(F32)
    bits = x.view(np.int32)
    e = ((bits >> 23) & 0xFF) - 127 - np.where(sub, 24, 0)
    m = ((bits & 0x7FFFFF) | 0x3F800000).astype(np.int32).view(F32)
    big = m > F32(1.41421356)
    m = np.where(big, m * F32(0.5), m).astype(F32)
    e = e + big
    j = np.rint((m - F32(1)) * F32(128)).astype(np.int32)
    c = F32(1) + j.astype(F32) * F32(0.0078125)
    d = m - c
    rh = d / c
    rl = _fma_residual_div(rh, c, d)
    sqh, sql = two_prod(rh, rh)
    qh = sqh * F32(0.5)
    ql = sql * F32(0.5) + rh * rl
    poly = F32(0.166666672) - rh * F32(0.142857149)
    poly = F32(0.200000003) - rh * poly
    poly = F32(0.25) - rh * poly
    poly = F32(0.333333343) - rh * poly
    tail = (sqh * rh) * poly
    ah, al = two_sum(rh, -qh)
    l1h, l1l = fast_two_sum(ah, al + ((rl + tail) - ql))
    ef = e.astype(F32)
    th, tl = LN_TAB[j - LN_J0, 0], LN_TAB[j - LN_J0, 1]
    s1h, s1l = two_sum(ef * LN2_HI, th)
    s2h, s2l = two_sum(s1h, l1h)
    small = (ef * LN2_LO + ef * LN2_LO2) + (tl + l1l)
    return fast_two_sum(s2h, (s1l + s2l) + small)


def ff_exp_neg(yh, yl):
    """exp(y) for y <= 0, y >= -87, as (hi, lo)."""
    yh, yl = _a(yh), _a(yl)
    k = np.rint(yh * INV_LN2_64).astype(np.int32)
    j = k & 63
    m = k >> 6
    kf = k.astype(F32)
    t0 = yh - kf * LN2_64_HI
    pmh, pml = two_prod(kf, LN2_64_MID)
    sh, sl = two_sum(t0, -pmh)
    e = ((sl - pml) - kf * LN2_64_LO) + yl
    rh, rl = fast_two_sum(sh, e)
    poly = F32(0.0416666679) + rh * F32(0.00833333377)
    poly = F32(0.166666672) + rh * poly
    poly = F32(0.5) + rh * poly
    tail = (rh * rh) * poly
    ah, al = two_sum(F32(1), rh)
    erh, erl = fast_two_sum(ah, al + (rl + tail))
    xh, xl = ff_mul(erh, erl, EXP_TAB[j, 0], EXP_TAB[j, 1])
    scale = ((m + 127) << 23).astype(np.int32).view(F32)
    return xh * scale, xl * scale


def ve_ff(ln_h, ln_l, alpha, beta):
    """calc_VE for eff with ln(eff) = ln_h + ln_l: logistic(alpha + beta ln eff), one rounding."""
    ah, al = _split_f(alpha)
    bh, bl = _split_f(beta)
    ph, pl = ff_mul(bh, bl, ln_h, ln_l)
    zh, zl = ff_add(ah, al, ph, pl)
    pos = zh >= 0
    yh = np.where(pos, -zh, zh).astype(F32)
    yl = np.where(pos, -zl, zl).astype(F32)
    big = yh < F32(-87)
    yh_c = np.where(big, F32(0), yh).astype(F32)
    yl_c = np.where(big, F32(0), yl).astype(F32)
    xh, xl = ff_exp_neg(yh_c, yl_c)
    dh, dl = fast_two_sum(F32(1), xh)
    qh, ql = ff_div(xh, xl, dh, dl + xl)
    omh, oml = two_sum(F32(1), -qh)
    ve = np.where(pos, omh + (oml - ql), qh + ql).astype(F32)
    ve = np.where(big, np.where(pos, F32(1), F32(0)), ve).astype(F32)
    return ve


def _split_f(x):
    x = float(x)
    hi = F32(x)
    return hi, F32(x - float(hi))


def split_log(x):
    """ln(x) of a positive float as (hi, lo), from the decimal module (host-side tables)."""
    d = Decimal(float(x)).ln()
    return _split(d)


def check_immunity_gpu(people):
    """immunity.py:303-350 with calc_VE evaluated as the GPU does (float-float, one rounding)."""
    pars = people.pars
    ne = pars['nab_eff']
    nv = pars['n_variants']
    n = people.n
    imm_tab = np.asarray(pars['immunity'], dtype=F32)
    with np.errstate(invalid='ignore'):
        was_inf = people.t >= people.date_recovered
    rv = people.recovered_variant
    nab = people.nab.astype(F32)
    nab_pos = nab > 0
    lnh, lnl = ff_log(np.where(nab_pos, nab, F32(1)))
    axes = [('alpha_inf', 'beta_inf', 'sus_imm'), ('alpha_symp_inf', 'beta_symp_inf', 'symp_imm'),
            ('alpha_sev_symp', 'beta_sev_symp', 'sev_imm')]
    for v in range(nv):
        nat = np.zeros(n, dtype=F32)
        ok = was_inf & ~np.isnan(rv)
        nat[ok] = imm_tab[v, rv[ok].astype(int)]
        if len(pars['vaccine_pars']) and people.vaccinated.any():
            raise NotImplementedError('vaccine immunity is not in the GPU arithmetic mirror')
        imm = nat
        eff_pos = nab_pos & (imm > 0)
        # ln(imm) per distinct value, from the decimal module (as the host fills the GPU tables)
        lih = np.zeros(n, dtype=F32)
        lil = np.zeros(n, dtype=F32)
        for val in np.unique(imm[eff_pos]):
            h, l = split_log(val)
            sel = eff_pos & (imm == val)
            lih[sel], lil[sel] = h, l
        eh, el = ff_add(lnh, lnl, lih, lil)
        for a, b, key in axes:
            ve = ve_ff(eh, el, ne[a], ne[b])
            people[key][v, :] = np.where(eff_pos, ve, F32(0))


def split_kin(nab_kin):
    """nab_kin as float pairs (hi, lo)."""
    kin = np.asarray(nab_kin, dtype=np.float64)
    hi = kin.astype(F32)
    lo = (kin - hi.astype(np.float64)).astype(F32)
    return hi, lo


def update_nab_ff(nab, peak, kh, kl):
    """nab + kin * peak rounded once to float32 (kin = kh + kl), clamped to [0, peak]."""
    nab, peak = _a(nab), _a(peak)
    ph, pl = two_prod(kh, peak)
    t = _a(kl) * peak
    sh, sl = two_sum(nab, ph)
    x = sh + (sl + (pl + t))
    x = np.where(x < 0, F32(0), x)
    x = np.where(x > peak, peak, x)
    return x.astype(F32)


def update_nab_gpu(people, inds):
    """immunity.py:205-213 as the GPU computes it."""
    kh, kl = split_kin(people.pars['nab_kin'])
    k = people.t - people.t_nab_event[inds]
    people.nab[inds] = update_nab_ff(people.nab[inds], people.peak_nab[inds], kh[k], kl[k])
