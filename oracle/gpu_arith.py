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
LN_INV = np.array([F32(1) / F32(1 + j / 128) for j in range(LN_J0, LN_J1 + 1)], F32)  # 1 / c_j, one rounding
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
    """a / b with one correctly rounded reciprocal (covgpu_ff.cuh ff_div)."""
    ah, al, bh, bl = _a(ah), _a(al), _a(bh), _a(bl)
    rcp = F32(1) / bh
    q1 = ah * rcp
    ph, pl = two_prod(q1, bh)
    r = (ah - ph) - pl
    r = r + al
    r = r - q1 * bl
    return fast_two_sum(q1, r * rcp)


def _fma_residual(rh, c, d):
    """fmaf(-rh, c, d): d - rh*c is exact in float64, then rounded once to float32."""
    return (d.astype(np.float64) - rh.astype(np.float64) * c.astype(np.float64)).astype(F32)


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
    ic = LN_INV[j - LN_J0]
    rh = d * ic
    rl = _fma_residual(rh, c, d) * ic
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


# ----------------------------------------------------------------- infection draws (People.infect)
def _pi_decimal():
    def atan_inv(n):
        x = Decimal(1) / n
        x2, term, total, k = x * x, x, x, 1
        while True:
            term *= -x2
            k += 2
            nxt = total + term / k
            if nxt == total:
                return total
            total = nxt
    return 16 * atan_inv(5) - 4 * atan_inv(239)


def _sin_cos(x):
    s, c = Decimal(0), Decimal(0)
    term, k = x, 1
    while abs(term) > Decimal(10) ** -60:
        s += term
        term = -term * x * x / ((k + 1) * (k + 2))
        k += 2
    term, k = Decimal(1), 0
    while abs(term) > Decimal(10) ** -60:
        c += term
        term = -term * x * x / ((k + 1) * (k + 2))
        k += 2
    return s, c


_PI = _pi_decimal()
PI_2_HI, PI_2_LO = (F32(v) for v in _split(_PI / 2))
LN2_FF_HI, LN2_FF_LO = (F32(v) for v in _split(_LN2))
SINCOS_TAB = np.array([[*_split(s), *_split(c)] for s, c in (_sin_cos(_PI * j / 64) for j in range(33))], F32)


def ff_exp(yh, yl):
    """exp of a float-float (covgpu_ff.cuh ff_exp): 0 below -87, inf above 87."""
    yh, yl = _a(yh), _a(yl)
    under, over, pos = yh < F32(-87), yh > F32(87), yh > 0
    ah = np.where(pos, -yh, yh)
    al = np.where(pos, -yl, yl)
    ah = np.where(under | over, F32(0), ah).astype(F32)
    al = np.where(under | over, F32(0), al).astype(F32)
    eh, el = ff_exp_neg(ah, al)
    ih, il = ff_div(np.ones_like(eh), np.zeros_like(el), eh, el)
    hi = np.where(pos, ih, eh)
    lo = np.where(pos, il, el)
    hi = np.where(under, F32(0), np.where(over, F32(np.inf), hi)).astype(F32)
    lo = np.where(under | over, F32(0), lo).astype(F32)
    return hi, lo


def ff_log_ff(xh, xl):
    lh, ll = ff_log(xh)
    return fast_two_sum(lh, ll + _a(xl) * (F32(1) / _a(xh)))


def ff_sqrt(xh, xl):
    xh, xl = _a(xh), _a(xl)
    s = np.sqrt(xh)
    ph, pl = two_prod(s, s)
    r = ((xh - ph) - pl) + xl
    return fast_two_sum(s, r * (F32(1) / (F32(2) * s)))


def u01_ff(a):
    """(a + 1/2) * 2^-32 of 32-bit words as exact float-float pairs."""
    k = 2 * np.asarray(a, dtype=np.uint64).astype(np.int64) + 1
    hi = k.astype(np.float64).astype(F32)
    lo = (k - hi.astype(np.int64)).astype(F32)
    return hi * F32(2.0 ** -33), lo * F32(2.0 ** -33)


def ll_to_ff(k):
    k = np.asarray(k, dtype=np.int64)
    hi = k.astype(np.float64).astype(F32)
    return hi, (k - hi.astype(np.int64)).astype(F32)


def ff_cossin_2pi(b):
    """(cos, sin) of 2 pi (b + 1/2) 2^-32 as float-float pairs (covgpu_ff.cuh ff_cossin_2pi)."""
    k = 2 * np.asarray(b, dtype=np.uint64).astype(np.int64) + 1
    q = k >> 31
    fk = k & 0x7FFFFFFF
    j = (fk + (1 << 25)) >> 26
    rh, rl = ll_to_ff(fk - (j << 26))
    ph, pl = ff_mul(PI_2_HI, PI_2_LO, rh * F32(2.0 ** -31), rl * F32(2.0 ** -31))
    p2h, p2l = ff_mul(ph, pl, ph, pl)
    x2 = p2h
    dh, dl = ff_div(p2h, p2l, F32(6), F32(0))
    th, tl = ff_mul(ph, pl, dh, dl)
    st = (x2 * x2) * (F32(0.00833333377) - x2 * F32(0.000198412701))
    ah, al = ff_add(ph, pl, -th, -tl)
    bh, bl = two_prod(ph, st)
    sph, spl = ff_add(ah, al, bh, bl)
    ct = (x2 * x2) * (F32(0.0416666679) - x2 * F32(0.00138888892))
    hh, hl = p2h * F32(0.5), p2l * F32(0.5)
    ch_, cl_ = ff_add(F32(1), F32(0), -hh, -hl)
    cph, cpl = ff_add(ch_, cl_, ct, F32(0))
    sjh, sjl, cjh, cjl = (SINCOS_TAB[j, i] for i in range(4))
    msh, msl = ff_mul(sjh, sjl, sph, spl)
    mch, mcl = ff_mul(cjh, cjl, sph, spl)
    x1h, x1l = ff_mul(sjh, sjl, cph, cpl)
    snh, snl = ff_add(x1h, x1l, mch, mcl)
    x2h, x2l = ff_mul(cjh, cjl, cph, cpl)
    csh, csl = ff_add(x2h, x2l, -msh, -msl)
    ch = np.select([q == 0, q == 1, q == 2], [csh, -snh, -csh], snh).astype(F32)
    cl = np.select([q == 0, q == 1, q == 2], [csl, -snl, -csl], snl).astype(F32)
    sh = np.select([q == 0, q == 1, q == 2], [snh, csh, -snh], -csh).astype(F32)
    sl = np.select([q == 0, q == 1, q == 2], [snl, csl, -snl], -csl).astype(F32)
    return (ch, cl), (sh, sl)


def box_muller_ff(wa, wb):
    """(z0, z1) as float-float pairs from two Philox words (covgpu_ff.cuh box_muller_ff)."""
    lh, ll = ff_log_ff(*u01_ff(wa))
    rh, rl = ff_sqrt(lh * F32(-2), ll * F32(-2))
    (ch, cl), (sh, sl) = ff_cossin_2pi(wb)
    return ff_mul(rh, rl, ch, cl), ff_mul(rh, rl, sh, sl)


def ff_rint(xh, xl):
    """Round half to even of a float-float, as a float32."""
    xh, xl = _a(xh), _a(xl)
    k = np.floor(xh)
    d = (xh - k) - F32(0.5)
    up = d > -xl
    down = d < -xl
    even = np.fmod(k, F32(2)) == 0
    return np.where(up, k + F32(1), np.where(down, k, np.where(even, k, k + F32(1)))).astype(F32)


def d2ff(x):
    x = np.asarray(x, dtype=np.float64)
    hi = x.astype(F32)
    return hi, (x - hi.astype(np.float64)).astype(F32)


def ff2d(xh, xl):
    return _a(xh).astype(np.float64) + _a(xl).astype(np.float64)


DIST_LOGNORMAL_INT, DIST_LOGNORMAL, DIST_NORMAL, DIST_NORMAL_INT, DIST_NORMAL_POS, DIST_ZERO = range(6)


def dist_code(dist):
    """(code, a, b) of a duration distribution as the host packs it (lognormal: the normal's mean and sd)."""
    name, p1, p2 = dist['dist'], dist['par1'], dist['par2']
    codes = {'lognormal_int': 0, 'lognorm_int': 0, 'lognormal': 1, 'lognorm': 1, 'normal': 2, 'norm': 2,
             'normal_int': 3, 'normal_pos': 4}
    code = codes[name]
    if code in (0, 1):
        if not p1 > 0:
            return DIST_ZERO, 0.0, 0.0
        return code, float(np.log(p1 ** 2 / np.sqrt(p2 ** 2 + p1 ** 2))), float(np.sqrt(np.log(p2 ** 2 / p1 ** 2 + 1)))
    return code, float(p1), float(p2)


def sample_ff(dist, zh, zl):
    """utils.py:156-236 sample() of a one-normal distribution in float-float (covgpu_ff.cuh sample_ff)."""
    code, a, b = dist_code(dist)
    zh, zl = _a(zh), _a(zl)
    if code == DIST_ZERO:
        return np.zeros(zh.shape)
    ah, al = d2ff(a)
    bh, bl = d2ff(b)
    mh, ml = ff_mul(np.full_like(zh, bh), np.full_like(zl, bl), zh, zl)
    yh, yl = ff_add(np.full_like(zh, ah), np.full_like(zl, al), mh, ml)
    if code == DIST_LOGNORMAL_INT:
        return ff_rint(*ff_exp(yh, yl)).astype(np.float64)
    if code == DIST_LOGNORMAL:
        return ff2d(*ff_exp(yh, yl))
    if code == DIST_NORMAL:
        return ff2d(yh, yl)
    if code == DIST_NORMAL_INT:
        neg = yh < 0
        return ff_rint(np.where(neg, -yh, yh), np.where(neg, -yl, yl)).astype(np.float64)
    return np.abs(ff2d(yh, yl))


def exp2_ff(x):
    """2^x of float64 values as the GPU computes update_peak_nab's 2**init (float-float)."""
    xh, xl = d2ff(x)
    yh, yl = ff_mul(xh, xl, np.full_like(xh, LN2_FF_HI), np.full_like(xl, LN2_FF_LO))
    return ff2d(*ff_exp(yh, yl))
