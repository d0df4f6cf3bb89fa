"""Generate covgpu_tables.h: float-float tables for the float64 steps of the path.

ln(c_j) for the reduction points c_j = 1 + j/128 (j = -40..55) and 1 / c_j, 2^(j/64)
(j = 0..63), and sin / cos of j * pi / 64 (j = 0..32), each as a pair of
float32 (hi, lo) with hi + lo equal to the value to about 2^-48, plus pi / 2
and ln 2 as pairs. Values come from Python's decimal module at 50 digits
(sin and cos by their Taylor series, pi by Machin's formula), so the tables
are the same on every platform. Run from the repository root:

    python covasim_gb300/csrc/gen_tables.py
"""
import math
import os
import struct
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 50

LN_J0, LN_J1 = -40, 55          # c_j = 1 + j/128 covers m in [0.6875, 1.4297]
EXP_N = 64


def f32(x):
    return struct.unpack('<f', struct.pack('<f', float(x)))[0]


def split(d):
    """Decimal -> (hi, lo) float32 pair."""
    hi = f32(d)
    lo = f32(d - Decimal(hi))
    return hi, lo


def ln_table():
    out = []
    for j in range(LN_J0, LN_J1 + 1):
        c = Decimal(1) + Decimal(j) / Decimal(128)
        out.append(split(c.ln()))
    return out


def ln_inv_table():
    """1 / c_j rounded once to float32 (c_j is exact in float32; float32 division
    is correctly rounded)."""
    return [float(np.float32(1.0) / np.float32(1.0 + j / 128.0)) for j in range(LN_J0, LN_J1 + 1)]


def exp_table():
    ln2 = Decimal(2).ln()
    return [split((Decimal(j) / Decimal(EXP_N) * ln2).exp()) for j in range(EXP_N)]


def ln2_64_parts():
    """ln(2)/64 as C_HI (11 significant bits, so k * C_HI is exact for |k| < 2^13) + C_MID + C_LO."""
    c = Decimal(2).ln() / Decimal(64)
    be = math.floor(math.log2(float(c)))
    hi = float(round(c / Decimal(2) ** (be - 10)) * Decimal(2) ** (be - 10))
    mid = f32(c - Decimal(hi))
    lo = f32(c - Decimal(hi) - Decimal(mid))
    return f32(hi), mid, lo


def pi_decimal():
    """pi = 16 atan(1/5) - 4 atan(1/239) (Machin), to the context precision."""
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


def sin_cos(x):
    """(sin x, cos x) by their Taylor series, for |x| <= pi / 2."""
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


def sincos_table():
    pi = pi_decimal()
    return [tuple(split(v) for v in sin_cos(pi * j / 64)) for j in range(33)]


def hexf(x):
    return float(x).hex() + 'f'


def main():
    lt, et = ln_table(), exp_table()
    lines = ['// Generated by covasim_gb300/csrc/gen_tables.py -- do not edit.',
             '// float-float (hi, lo) tables for the NAb efficacy math in covgpu_device.cuh.',
             '#pragma once',
             f'#define COVGPU_LN_J0 ({LN_J0})',
             f'#define COVGPU_LN_N {len(lt)}',
             f'#define COVGPU_EXP_N {EXP_N}',
             ]
    ln2 = Decimal(2).ln()
    ln2_hi = float(round(ln2 * 2 ** 16) / Decimal(2 ** 16))  # 16 significant bits: e * LN2_HI exact for |e| < 2^8
    ln2_lo = f32(ln2 - Decimal(ln2_hi))
    ln2_lo2 = f32(ln2 - Decimal(ln2_hi) - Decimal(ln2_lo))
    lines += [f'#define COVGPU_LN2_HI {hexf(f32(ln2_hi))}', f'#define COVGPU_LN2_LO {hexf(ln2_lo)}',
              f'#define COVGPU_LN2_LO2 {hexf(ln2_lo2)}',
              f'#define COVGPU_INV_LN2_64 {hexf(f32(Decimal(64) / ln2))}']
    ch, cm, cl = ln2_64_parts()
    lines += [f'#define COVGPU_LN2_64_HI {hexf(ch)}', f'#define COVGPU_LN2_64_MID {hexf(cm)}',
              f'#define COVGPU_LN2_64_LO {hexf(cl)}',
              '__device__ const float COVGPU_LN_TAB[COVGPU_LN_N][2] = {']
    lines += [f'  {{{hexf(h)}, {hexf(l)}}},' for h, l in lt]
    lines += ['};', '__device__ const float COVGPU_EXP_TAB[COVGPU_EXP_N][2] = {']
    lines += [f'  {{{hexf(h)}, {hexf(l)}}},' for h, l in et]
    lines += ['};']
    pi = pi_decimal()
    ph, pl = split(pi / 2)
    lh, ll = split(Decimal(2).ln())
    lines += [f'#define COVGPU_PI_2_HI {hexf(ph)}', f'#define COVGPU_PI_2_LO {hexf(pl)}',
              f'#define COVGPU_LN2_FF_HI {hexf(lh)}', f'#define COVGPU_LN2_FF_LO {hexf(ll)}',
              '// sin and cos of j * pi / 64, j = 0..32: {sin hi, sin lo, cos hi, cos lo}',
              '__device__ const float COVGPU_SINCOS_TAB[33][4] = {']
    lines += [f'  {{{hexf(sv[0])}, {hexf(sv[1])}, {hexf(cv[0])}, {hexf(cv[1])}}},' for sv, cv in sincos_table()]
    lines += ['};', '// 1 / c_j of the ln reduction points, rounded once to float32',
              '__device__ const float COVGPU_LN_INV[COVGPU_LN_N] = {']
    lines += [f'  {hexf(v)},' for v in ln_inv_table()]
    lines += ['};', '']
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'covgpu_tables.h')
    with open(path, 'w') as f:
        f.write('\n'.join(lines))
    print(path)


if __name__ == '__main__':
    main()
