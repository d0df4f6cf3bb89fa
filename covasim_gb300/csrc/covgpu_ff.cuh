// Float-float ("two-float", ~44-bit) arithmetic for the float64 steps of the
// reference, so that they run on GB300's float32 units.
//
// GB300 executes float64 at a small fraction of its float32 rate. The
// reference computes the NAb efficacy (immunity.py:216-247 calc_VE, called by
// check_immunity for every agent every day), update_nab (immunity.py:205-213),
// and the normals, lognormal durations and initial NAb levels of infect
// (people.py:514-577, immunity.py:138-202) in float64 and stores float32 or
// whole days; here the same quantities are computed with error-free
// transformations (two-sum, two-product via fused multiply-add) to about
// 2^-40 relative and rounded once, which reproduces the reference's result
// except when the exact value lies that close to a rounding boundary.
//
// Only IEEE round-to-nearest add/sub/mul/div and fused multiply-add (used for
// exact product residuals only) appear, in a fixed order: the numpy mirror in
// the oracle (oracle/gpu_arith.py) performs the same operations and gets the
// same bits. ln uses the reduction x = 2^e * c_j * (1 + r), |r| < 2^-7.5 (r
// formed with a table of 1 / c_j and the exact residual), and the series of
// ln(1 + r); exp uses Cody-Waite reduction by ln2/64, a table
// of 2^(j/64) and the Taylor series of exp(r), |r| <= ln2/128; cos and sin of
// 2 pi u reduce exactly to a quadrant and the nearest of the points
// j pi / 64 and use the Taylor series of the residual |phi| <= pi / 128.
#pragma once
#include <stdint.h>
#include "covgpu_tables.h"

namespace covgpu {

struct ff { float hi, lo; };

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return ff{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ ff ff_mul(ff x, ff y) {
  const ff p = two_prod(x.hi, y.hi);
  return fast_two_sum(p.hi, __fadd_rn(p.lo, __fadd_rn(__fmul_rn(x.hi, y.lo), __fmul_rn(x.lo, y.hi))));
}

// a / b as float-float with one correctly rounded reciprocal instead of two
// divisions: q1 = a.hi * (1 / b.hi), then the residual a - q1 b (exact product
// residual) times the same reciprocal
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float rcp = __frcp_rn(b.hi);
  const float q1 = __fmul_rn(a.hi, rcp);
  const ff p = two_prod(q1, b.hi);
  float r = __fsub_rn(__fsub_rn(a.hi, p.hi), p.lo);
  r = __fadd_rn(r, a.lo);
  r = __fsub_rn(r, __fmul_rn(q1, b.lo));
  return fast_two_sum(q1, __fmul_rn(r, rcp));
}

// ln(x) for finite x > 0, as float-float. tab: COVGPU_LN_TAB, inv: COVGPU_LN_INV
// (shared-memory copies or the tables themselves).
__device__ __forceinline__ ff ff_log(float x, const float (*tab)[2], const float* inv) {
  int e_adj = 0;
  if (x < 1.17549435e-38f) { x = __fmul_rn(x, 16777216.0f); e_adj = -24; }
  const int bits = __float_as_int(x);
  int e = ((bits >> 23) & 0xff) - 127 + e_adj;
  float m = __int_as_float((bits & 0x7fffff) | 0x3f800000);
  if (m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
  const int j = (int)rintf(__fmul_rn(__fsub_rn(m, 1.0f), 128.0f));
  const float c = __fadd_rn(1.0f, __fmul_rn((float)j, 0.0078125f));
  const float d = __fsub_rn(m, c);
  const float ic = inv[j - COVGPU_LN_J0];
  const float rh = __fmul_rn(d, ic);                  // d / c to about an ulp
  const float rl = __fmul_rn(__fmaf_rn(-rh, c, d), ic);  // the exact residual over c
  // ln(1 + r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6 + r^4/7)
  const ff sq = two_prod(rh, rh);
  const float qh = __fmul_rn(sq.hi, 0.5f);
  const float ql = __fadd_rn(__fmul_rn(sq.lo, 0.5f), __fmul_rn(rh, rl));
  float poly = __fsub_rn(0.166666672f, __fmul_rn(rh, 0.142857149f));   // 1/6 - r/7
  poly = __fsub_rn(0.200000003f, __fmul_rn(rh, poly));                  // 1/5 - r(...)
  poly = __fsub_rn(0.25f, __fmul_rn(rh, poly));                         // 1/4 - r(...)
  poly = __fsub_rn(0.333333343f, __fmul_rn(rh, poly));                  // 1/3 - r(...)
  const float tail = __fmul_rn(__fmul_rn(sq.hi, rh), poly);
  const ff a = two_sum(rh, -qh);
  const ff l1p = fast_two_sum(a.hi, __fadd_rn(a.lo, __fsub_rn(__fadd_rn(rl, tail), ql)));
  const float ef = (float)e;
  const ff s1 = two_sum(__fmul_rn(ef, COVGPU_LN2_HI), tab[j - COVGPU_LN_J0][0]);
  const ff s2 = two_sum(s1.hi, l1p.hi);
  const float small = __fadd_rn(__fadd_rn(__fmul_rn(ef, COVGPU_LN2_LO), __fmul_rn(ef, COVGPU_LN2_LO2)),
                                __fadd_rn(tab[j - COVGPU_LN_J0][1], l1p.lo));
  return fast_two_sum(s2.hi, __fadd_rn(__fadd_rn(s1.lo, s2.lo), small));
}

// exp(y) for y <= 0, y.hi >= -87, as float-float. tab: COVGPU_EXP_TAB.
__device__ __forceinline__ ff ff_exp_neg(ff y, const float (*tab)[2]) {
  const int k = (int)rintf(__fmul_rn(y.hi, COVGPU_INV_LN2_64));
  const int j = k & 63;
  const int m = k >> 6;
  const float kf = (float)k;
  const float t0 = __fsub_rn(y.hi, __fmul_rn(kf, COVGPU_LN2_64_HI));
  const ff pm = two_prod(kf, COVGPU_LN2_64_MID);
  const ff s = two_sum(t0, -pm.hi);
  const float e = __fadd_rn(__fsub_rn(__fsub_rn(s.lo, pm.lo), __fmul_rn(kf, COVGPU_LN2_64_LO)), y.lo);
  const ff r = fast_two_sum(s.hi, e);
  // exp(r) = 1 + r + r^2 (1/2 + r (1/6 + r (1/24 + r/120)))
  float poly = __fadd_rn(0.0416666679f, __fmul_rn(r.hi, 0.00833333377f));
  poly = __fadd_rn(0.166666672f, __fmul_rn(r.hi, poly));
  poly = __fadd_rn(0.5f, __fmul_rn(r.hi, poly));
  const float tail = __fmul_rn(__fmul_rn(r.hi, r.hi), poly);
  const ff a = two_sum(1.0f, r.hi);
  const ff er = fast_two_sum(a.hi, __fadd_rn(a.lo, __fadd_rn(r.lo, tail)));
  const ff x = ff_mul(er, ff{tab[j][0], tab[j][1]});
  const float scale = __int_as_float((m + 127) << 23);  // 2^m, m in [-126, 0]
  return ff{__fmul_rn(x.hi, scale), __fmul_rn(x.lo, scale)};
}

// exp(y) for any float-float y: exp_neg of -y and a reciprocal for y > 0;
// 0 below -87 and +inf above 87 (the float32 range of the values it feeds)
__device__ __forceinline__ ff ff_exp(ff y, const float (*tab)[2]) {
  if (y.hi < -87.0f) return ff{0.0f, 0.0f};
  if (y.hi > 87.0f) return ff{__int_as_float(0x7f800000), 0.0f};
  if (y.hi <= 0.0f) return ff_exp_neg(y, tab);
  return ff_div(ff{1.0f, 0.0f}, ff_exp_neg(ff{-y.hi, -y.lo}, tab));
}

// ln of a positive float-float: ln(hi) + lo / hi (|lo / hi| <= 2^-24, so the
// dropped term is below 2^-49; lo / hi as lo times the reciprocal of hi)
__device__ __forceinline__ ff ff_log_ff(ff x, const float (*tab)[2], const float* inv) {
  const ff l = ff_log(x.hi, tab, inv);
  return fast_two_sum(l.hi, __fadd_rn(l.lo, __fmul_rn(x.lo, __frcp_rn(x.hi))));
}

// sqrt of a positive float-float: the float32 root and one correction by the
// exact residual x - s^2 (over 2s, as a product with its reciprocal)
__device__ __forceinline__ ff ff_sqrt(ff x) {
  const float s = __fsqrt_rn(x.hi);
  const ff p = two_prod(s, s);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p.hi), p.lo), x.lo);
  return fast_two_sum(s, __fmul_rn(r, __frcp_rn(__fmul_rn(2.0f, s))));
}

// the uniform (a + 1/2) * 2^-32 of a 32-bit word, exactly, as float-float: the
// odd 33-bit k = 2a + 1 is kh * 2^16 + kl with both halves exact in float32,
// and the two-sum of the halves is (k rounded to float32, the exact remainder);
// 32-bit operations only (64-bit conversions are slow on GB300)
__device__ __forceinline__ ff u01_ff(uint32_t a) {
  const float kh = (float)(a >> 15), kl = (float)(((a << 1) | 1u) & 0xFFFFu);
  const ff k = two_sum(__fmul_rn(kh, 65536.0f), kl);
  return ff{__fmul_rn(k.hi, 0x1p-33f), __fmul_rn(k.lo, 0x1p-33f)};
}

// a 32-bit integer as float-float, exactly (the same split)
__device__ __forceinline__ ff i32_to_ff(int32_t k) {
  return two_sum(__fmul_rn((float)(k >> 12), 4096.0f), (float)(k & 0xFFF));
}

// cos and sin of 2 pi u for u = (b + 1/2) * 2^-32: the quadrant and the nearest
// of the points j pi / 64 from the word's bits (exact), then the Taylor series
// of the residual angle |phi| <= pi / 128 (tables: COVGPU_SINCOS_TAB)
__device__ __forceinline__ void ff_cossin_2pi(uint32_t b, const float (*tab)[4], ff& c, ff& s) {
  // k = 2b + 1 (33 bits), 4u = k * 2^-31, in 32-bit pieces
  const unsigned q = b >> 30;                                      // quadrant 0..3
  const uint32_t fk = ((b << 1) | 1u) & 0x7FFFFFFFu;               // f = fk * 2^-31 in [0, 1)
  const uint32_t j = (fk + (1u << 25)) >> 26;                      // nearest j / 32, j = 0..32
  const ff r = i32_to_ff((int32_t)(fk - (j << 26)));               // (f - j/32) * 2^31, |.| <= 2^25
  const ff phi = ff_mul(ff{COVGPU_PI_2_HI, COVGPU_PI_2_LO}, ff{__fmul_rn(r.hi, 0x1p-31f), __fmul_rn(r.lo, 0x1p-31f)});
  const ff p2 = ff_mul(phi, phi);
  const float x2 = p2.hi;
  // sin phi = phi - phi^3/6 + phi (phi^4/120 - phi^6/5040); cos phi = 1 - phi^2/2 + phi^4/24 - phi^6/720
  const ff third = ff_mul(phi, ff_div(p2, ff{6.0f, 0.0f}));
  const float st = __fmul_rn(__fmul_rn(x2, x2), __fsub_rn(0.00833333377f, __fmul_rn(x2, 0.000198412701f)));
  const ff sphi = ff_add(ff_add(phi, ff{-third.hi, -third.lo}), two_prod(phi.hi, st));
  const float ct = __fmul_rn(__fmul_rn(x2, x2), __fsub_rn(0.0416666679f, __fmul_rn(x2, 0.00138888892f)));
  const ff half = ff{__fmul_rn(p2.hi, 0.5f), __fmul_rn(p2.lo, 0.5f)};
  const ff cphi = ff_add(ff_add(ff{1.0f, 0.0f}, ff{-half.hi, -half.lo}), ff{ct, 0.0f});
  const ff sj = ff{tab[j][0], tab[j][1]}, cj = ff{tab[j][2], tab[j][3]};
  const ff ms = ff_mul(sj, sphi), mc = ff_mul(cj, sphi);
  const ff sn = ff_add(ff_mul(sj, cphi), mc);                     // sin(j pi/64 + phi)
  const ff cs = ff_add(ff_mul(cj, cphi), ff{-ms.hi, -ms.lo});      // cos(j pi/64 + phi)
  switch (q) {                                                      // + q * pi / 2
    case 0: c = cs; s = sn; break;
    case 1: c = ff{-sn.hi, -sn.lo}; s = cs; break;
    case 2: c = ff{-cs.hi, -cs.lo}; s = ff{-sn.hi, -sn.lo}; break;
    default: c = sn; s = ff{-cs.hi, -cs.lo}; break;
  }
}

// Box-Muller in float-float: z0 = r cos(2 pi u2), z1 = r sin(2 pi u2), r = sqrt(-2 ln u1)
__device__ __forceinline__ void box_muller_ff(uint32_t wa, uint32_t wb, const float (*ln_tab)[2],
                                              const float* ln_inv, const float (*sc_tab)[4], ff& z0, ff& z1) {
  const ff l = ff_log_ff(u01_ff(wa), ln_tab, ln_inv);
  const ff r = ff_sqrt(ff{__fmul_rn(l.hi, -2.0f), __fmul_rn(l.lo, -2.0f)});
  ff c, s;
  ff_cossin_2pi(wb, sc_tab, c, s);
  z0 = ff_mul(r, c);
  z1 = ff_mul(r, s);
}

// round half to even of a float-float (|x| < 2^22)
__device__ __forceinline__ float ff_rint(ff x) {
  const float k = floorf(x.hi);
  const float f = __fsub_rn(x.hi, k);                // exact
  const float d = __fsub_rn(f, 0.5f);                // exact
  if (d > -x.lo) return __fadd_rn(k, 1.0f);          // above the midpoint
  if (d < -x.lo) return k;                           // below it
  return fmodf(k, 2.0f) == 0.0f ? k : __fadd_rn(k, 1.0f);  // a tie: to even
}

// a float64 as float-float (to about 2^-48)
__device__ __forceinline__ ff d2ff(double x) {
  const float hi = __double2float_rn(x);
  return ff{hi, __double2float_rn(__dsub_rn(x, (double)hi))};
}
__device__ __forceinline__ double ff2d(ff x) { return __dadd_rn((double)x.hi, (double)x.lo); }

// A distribution parameter pair (a, b) of covgpu_dur_par as float-float, so that
// the float64 conversions can be issued ahead of the normal they are applied to.
struct DistFF {
  int code;
  ff a, b;
};
__device__ __forceinline__ DistFF dist_ff(const covgpu_dur_par& d) { return DistFF{d.code, d2ff(d.a), d2ff(d.b)}; }

// utils.py:156-236 sample() of a distribution that is a function of one standard
// normal z, in float-float; the result as the float64 the reference stores.
// etab: COVGPU_EXP_TAB or its shared-memory copy.
__device__ __forceinline__ double sample_ff(const DistFF& d, ff z, const float (*etab)[2]) {
  const ff y = ff_add(d.a, ff_mul(d.b, z));
  switch (d.code) {
    case COVGPU_DIST_LOGNORMAL_INT: return (double)ff_rint(ff_exp(y, etab));
    case COVGPU_DIST_LOGNORMAL: return ff2d(ff_exp(y, etab));
    case COVGPU_DIST_NORMAL: return ff2d(y);
    case COVGPU_DIST_NORMAL_INT: return (double)ff_rint(y.hi < 0.0f ? ff{-y.hi, -y.lo} : y);
    case COVGPU_DIST_NORMAL_POS: return fabs(ff2d(y));
    default: return 0.0;
  }
}
__device__ __forceinline__ double sample_ff(const covgpu_dur_par& d, ff z) {
  return sample_ff(dist_ff(d), z, COVGPU_EXP_TAB);
}

// 2^x for a float-float x: exp(x ln 2)
__device__ __forceinline__ double exp2_ff(ff x, const float (*etab)[2]) {
  return ff2d(ff_exp(ff_mul(x, ff{COVGPU_LN2_FF_HI, COVGPU_LN2_FF_LO}), etab));
}
__device__ __forceinline__ double exp2_ff(ff x) { return exp2_ff(x, COVGPU_EXP_TAB); }

// calc_VE (immunity.py:216-247) for eff = nab * imm with ln(imm) given:
// exp(alpha) * eff^beta / (1 + exp(alpha) * eff^beta) = logistic(z),
// z = alpha + beta * (ln nab + ln imm); rounded once to float32.
__device__ __forceinline__ float ve_ff(ff ln_eff, ff alpha, ff beta, const float (*etab)[2]) {
  const ff z = ff_add(alpha, ff_mul(beta, ln_eff));
  const bool pos = z.hi >= 0.0f;
  const ff y = pos ? ff{-z.hi, -z.lo} : z;
  if (y.hi < -87.0f) return pos ? 1.0f : 0.0f;  // |z| > 87: 1 - 1e-38 rounds to 1; e^-87 flushed to 0
  const ff x = ff_exp_neg(y, etab);
  const ff den = fast_two_sum(1.0f, x.hi);
  const ff q = ff_div(x, ff{den.hi, __fadd_rn(den.lo, x.lo)});
  if (pos) {
    const ff om = two_sum(1.0f, -q.hi);
    return __fadd_rn(om.hi, __fsub_rn(om.lo, q.lo));
  }
  return __fadd_rn(q.hi, q.lo);
}

// update_nab (immunity.py:205-213): nab + kin * peak, rounded once to float32,
// with kin given as a float pair (hi, lo); then clamped to [0, peak].
__device__ __forceinline__ float update_nab_ff(float nab, float peak, float kh, float kl) {
  const ff p = two_prod(kh, peak);
  const float t = __fmul_rn(kl, peak);
  const ff s = two_sum(nab, p.hi);
  float x = __fadd_rn(s.hi, __fadd_rn(s.lo, __fadd_rn(p.lo, t)));
  if (x < 0.0f) x = 0.0f;
  if (x > peak) x = peak;
  return x;
}

// u < p with u = lhs * 2^-nbits (lhs odd, lhs < 2^nbits) and p a float32,
// decided exactly in integers: the same answer as comparing the two values
// in float64, where both are exact.
__device__ __forceinline__ bool frac_less(uint64_t lhs, int nbits, float p) {
  if (!(p > 0.0f)) return false;
  if (p >= 1.0f) return true;
  const uint32_t bits = __float_as_uint(p);
  const int ex = (bits >> 23) & 0xff;
  uint64_t mant = bits & 0x7fffffu;
  int e2;
  if (ex) { mant |= 0x800000u; e2 = ex - 150; } else { e2 = -149; }
  const int sh = e2 + nbits;  // u < p  <=>  lhs < mant * 2^sh
  if (sh >= 0) return lhs < (mant << sh);   // p < 1: mant * 2^sh < 2^nbits, no overflow
  if (sh <= -64) return false;
  const uint64_t q = mant >> (-sh);
  const uint64_t rem = mant & ((1ull << (-sh)) - 1ull);
  return lhs < q || (lhs == q && rem != 0);
}
// Philox words -> the (0,1) doubles of u01_52 / u01_32, compared with p exactly
__device__ __forceinline__ bool bern52(uint32_t a, uint32_t b, float p) {
  const uint64_t k = ((uint64_t)(a >> 6) << 26) | (uint64_t)(b >> 6);
  return frac_less(2 * k + 1, 53, p);
}
__device__ __forceinline__ bool bern32(uint32_t a, float p) {
  return frac_less(2 * (uint64_t)a + 1, 33, p);
}
// u01_52(a, b) < p for a float64 p given as its threshold ceil(p * 2^53)
__device__ __forceinline__ bool bern52_thr(uint32_t a, uint32_t b, uint64_t thr) {
  const uint64_t k = ((uint64_t)(a >> 6) << 26) | (uint64_t)(b >> 6);
  return 2 * k + 1 < thr;
}

}  // namespace covgpu
