// Correctly rounded elementary functions for the adapt path, host and
// device, so that the same argument gives the same double on either side
// (every step is an IEEE operation or an explicit fused multiply-add).
//
// cbrt_cr: the cube root rounded to nearest.  Newton iterates, the last one
// with its residual computed in double-double, give the answer within about
// 2^-88; when that is not far enough from a halfway point to settle the
// rounding, the answer is decided exactly, in 192-bit integer arithmetic, by
// comparing the cubes of the halfway points between neighbouring doubles
// with the argument.  With the
// argument reduced to m in [1, 8) (m = M 2^-52, M an integer below 2^55)
// and a candidate y = C 2^-52 in [1, 2], the halfway point (2C+1) 2^-53 lies
// below cbrt(m) exactly when (2C+1)^3 < M 2^107.  The left side is odd and
// the right side even, so there are no ties.
//
// log_cr, exp_cr: table-driven reductions in the manner of P. T. P. Tang
// ("Table-driven implementation of the exponential function", ACM TOMS 15,
// 1989; "... of the logarithm function", ACM TOMS 16, 1990), evaluated in
// double-double arithmetic (T. J. Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971) to a relative
// error near 2^-90 before the one final rounding, which is therefore the
// correct rounding unless the exact value lies within about 2^-90 of a
// halfway point between doubles.  A quick evaluation to about 2^-69 comes
// first; it is returned when Ziv's rounding test shows that its error cannot
// change the rounding (nearly always), else the accurate one decides.
//   log: x = 2^E f, f in [sqrt(1/2), sqrt(2)); with c = j/256 nearest f and
//   inv = the double nearest 1/c, log x = E ln 2 + log(1/inv) + log1p(r),
//   r = f inv - 1 exactly (|r| < 2^-8.4), log1p(r) = 2 atanh(r / (2 + r)).
//   exp: x = k ln2/128 + r, |r| <= ln2/256; exp x = 2^(k div 128)
//   2^((k mod 128)/128) exp(r), exp(r) - 1 by its Taylor series.
//   Results in the subnormal range are rounded twice.
// The tables come from gen_libm_tables.py (mpmath, 200 bits).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef OHG_HD
#ifdef __CUDACC__
#define OHG_HD __host__ __device__ __forceinline__
#else
#define OHG_HD inline
#endif
#endif

#include "ohg_libm_tables.inc"

#if defined(__CUDA_ARCH__)
#define OHG_LIBM_TAB(name) ohg_libm_d_##name
#else
#define OHG_LIBM_TAB(name) ohg_libm_h_##name
#endif

// The quick evaluations are on by default; OHG_LIBM_QUICK=0 leaves only the
// accurate ones (a test hook: both must give the same doubles).
#ifndef OHG_LIBM_QUICK
#define OHG_LIBM_QUICK 1
#endif

namespace ohg {

// ------------------------------------------------------------ double-double
struct DD {
  double hi, lo;
};
// a + b exactly (Knuth's TwoSum)
OHG_HD DD two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// a + b exactly when |a| >= |b| (Dekker's Fast2Sum)
OHG_HD DD fast_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  return {s, e};
}
// a b exactly, by a fused multiply-add
OHG_HD DD two_prod(double a, double b) {
  double p = a * b;
  double e = fma(a, b, -p);
  return {p, e};
}
OHG_HD DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  DD t = two_sum(a.lo, b.lo);
  s.lo = s.lo + t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return fast_two_sum(s.hi, s.lo);
}
OHG_HD DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
OHG_HD DD dd_mul(DD a, DD b) {
  DD p = two_prod(a.hi, b.hi);
  p.lo = p.lo + (a.hi * b.lo + a.lo * b.hi);
  return fast_two_sum(p.hi, p.lo);
}
OHG_HD DD dd_mul_d(DD a, double b) {
  DD p = two_prod(a.hi, b);
  p.lo = p.lo + a.lo * b;
  return fast_two_sum(p.hi, p.lo);
}
OHG_HD DD dd_div(DD a, DD b) {
  double q1 = a.hi / b.hi;
  DD r = dd_add(a, dd_neg(dd_mul_d(b, q1)));
  double q2 = r.hi / b.hi;
  r = dd_add(r, dd_neg(dd_mul_d(b, q2)));
  double q3 = r.hi / b.hi;
  DD q = fast_two_sum(q1, q2);
  return dd_add(q, DD{q3, 0.0});
}

// Whether the exact value, known to lie within err of the normalised pair
// hi + lo (hi = fl(hi + lo), hi normal), rounds to hi: it must stay strictly
// between the halfway points around hi (the one below |hi| is closer when
// |hi| is a power of two).  This is the rounding test of Ziv's strategy:
// a quick evaluation is returned when the test passes, else an accurate one
// decides.
// the bits of a double and back
OHG_HD std::uint64_t d2u(double x) {
#ifdef __CUDA_ARCH__
  return std::uint64_t(__double_as_longlong(x));
#else
  std::uint64_t u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}
OHG_HD double u2d(std::uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

OHG_HD bool rounds_to_hi(double hi, double lo, double err) {
  if (!(fabs(hi) >= 0x1p-1020) || !(fabs(hi) <= 0x1p1020)) return false;
  std::uint64_t b = d2u(hi) & 0x7fffffffffffffffull;
  std::uint64_t eb = b >> 52;  // biased exponent, 3 .. 2043 here
  double half_up = u2d((eb - 53) << 52);  // 2^(exponent - 53): half an ulp of hi
  bool pow2 = (b & 0xfffffffffffffull) == 0;
  bool toward_zero = (lo < 0.0) == (hi > 0.0);
  double margin = (toward_zero && pow2) ? 0.5 * half_up : half_up;
  return fabs(lo) + err < margin;
}

// ------------------------------------------------------------ cbrt
// 64 x 64 -> 128-bit product
OHG_HD void mul_64x64(std::uint64_t a, std::uint64_t b, std::uint64_t* hi, std::uint64_t* lo) {
#ifdef __CUDA_ARCH__
  *lo = a * b;
  *hi = __umul64hi(a, b);
#else
  unsigned __int128 p = (unsigned __int128)a * b;
  *lo = std::uint64_t(p);
  *hi = std::uint64_t(p >> 64);
#endif
}

// a^3 < M 2^107 for odd a < 2^55 and M < 2^55, exactly
OHG_HD bool cube_below(std::uint64_t a, std::uint64_t M) {
  std::uint64_t sh, sl;  // a^2 = sh 2^64 + sl (< 2^110)
  mul_64x64(a, a, &sh, &sl);
  std::uint64_t lh, ll, hh, hl;  // sl a and sh a; a^3 = (hh, hl + lh, ll) in 64-bit words
  mul_64x64(sl, a, &lh, &ll);
  mul_64x64(sh, a, &hh, &hl);
  std::uint64_t w1 = lh + hl;
  std::uint64_t w2 = hh + (w1 < lh ? 1u : 0u);
  // M 2^107 = (M >> 21) 2^128 + (M << 43 mod 2^64) 2^64
  std::uint64_t r2 = M >> 21, r1 = M << 43;
  if (w2 != r2) return w2 < r2;
  if (w1 != r1) return w1 < r1;
  return false;  // equal high words: a^3 has a nonzero (odd) low word, M 2^107 none
}

OHG_HD double cbrt_cr(double x) {
  if (x == 0.0 || !(x == x) || x - x != 0.0) return x + x;  // zero (sign kept), NaN, inf
  double ax = fabs(x);
  int kadj = 0;
  if (ax < 0x1p-1022) {  // subnormal: scale by 2^162, exactly
    ax *= 0x1p162;
    kadj = -54;
  }
  std::uint64_t bits = d2u(ax);
  int E = int(bits >> 52) - 1023;  // ax = g 2^E, g in [1, 2)
  int k = E >= 0 ? E / 3 : -((2 - E) / 3);
  int r = E - 3 * k;  // 0, 1 or 2
  // m = g 2^r in [1, 8); the cube root of ax is cbrt(m) 2^k
  double m = u2d((bits & 0xfffffffffffffull) | (std::uint64_t(1023 + r) << 52));
  k += kadj;
  // w ~ m^(-1/3): a float start and one division-free Newton step
  // w (4 - m w^3) / 3 (about 2^-45 relative); y = m w^2 ~ m^(1/3)
  double w = double(1.0f / cbrtf(float(m)));
  w = (w * (4.0 - m * (w * (w * w)))) * (1.0 / 3.0);
  double y = m * (w * w);
  {
    // one more Newton step with the residual y^3 - m computed to about
    // 2^-104 relative and 1 / (3 y^2) taken as w^2 / 3: y - res w^2 / 3 as
    // a pair, within about 2^-85
    DD y2 = two_prod(y, y);
    DD y3 = two_prod(y2.hi, y);
    double res = ((y3.hi - m) + y3.lo) + y2.lo * y;
    DD z = fast_two_sum(y, -(res * (w * w)) * (1.0 / 3.0));
    if (OHG_LIBM_QUICK && z.hi >= 1.0 && z.hi < 2.0 && rounds_to_hi(z.hi, z.lo, 0x1p-80)) {
      // z.hi 2^k: the exponent field moves by k (the result is normal)
      double r1 = u2d(d2u(z.hi) + (std::uint64_t(std::int64_t(k)) << 52));
      return x < 0.0 ? -r1 : r1;
    }
    y = z.hi;
  }
  const std::uint64_t one = std::uint64_t(1) << 52, two = std::uint64_t(1) << 53;
  double ys = ldexp(y, 52);
  std::uint64_t C = ys <= double(one) ? one : ys >= double(two) ? two : std::uint64_t(ys);
  std::uint64_t M = std::uint64_t(ldexp(m, 52));
  // raise C while the halfway point above it is below cbrt(m), lower it while
  // the halfway point below it is above; a few steps at most
  for (int it = 0; it < 8 && C < two && cube_below(2 * C + 1, M); ++it) ++C;
  for (int it = 0; it < 8 && C > one && !cube_below(2 * C - 1, M); ++it) --C;
  double res = ldexp(double(C), k - 52);
  return x < 0.0 ? -res : res;
}

// ------------------------------------------------------------ log
OHG_HD double log_cr(double x) {
  if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;  // zero, negative, NaN
  if (x - x != 0.0) return x;                            // +inf
  if (x == 1.0) return 0.0;
  int E = 0;
  if (x < 0x1p-1022) {  // subnormal: scale by 2^54, exactly
    x *= 0x1p54;
    E = -54;
  }
  std::uint64_t bits = d2u(x);
  E += int(bits >> 52) - 1023;  // x = f 2^E, f in [1, 2)
  double f = u2d((bits & 0xfffffffffffffull) | (std::uint64_t(1023) << 52));
  if (f >= 1.4142135623730951) {
    f = 0.5 * f;
    E += 1;
  }
  int j = int(f * 256.0 + 0.5);  // c_j = j/256 within 2^-9 of f
  j = j < OHG_LOG_J0 ? OHG_LOG_J0 : j > OHG_LOG_J1 ? OHG_LOG_J1 : j;
  double inv = OHG_LIBM_TAB(log_inv)[j - OHG_LOG_J0];
  DD p = two_prod(f, inv);
  DD r = two_sum(p.hi - 1.0, p.lo);  // f inv - 1, exactly
  double Ed = double(E);
  DD L = {OHG_LIBM_TAB(log_hi)[j - OHG_LOG_J0], OHG_LIBM_TAB(log_lo)[j - OHG_LOG_J0]};
  {
    // quick evaluation, within 2^-69 relative: E ln2 + L + r - r^2/2 with the
    // leading terms added exactly, the series from r^3 on in double
    double rh = r.hi, rl = r.lo;
    DD q = two_prod(rh, rh);
    double p3 = (rh * q.hi) *
                (1.0 / 3.0 +
                 rh * (-1.0 / 4.0 +
                       rh * (1.0 / 5.0 +
                             rh * (-1.0 / 6.0 +
                                   rh * (1.0 / 7.0 + rh * (-1.0 / 8.0 + rh * (1.0 / 9.0 - rh / 10.0)))))));
    DD a = two_sum(Ed * OHG_LN2_HI, L.hi);
    DD b = two_sum(a.hi, rh);
    DD c = two_sum(b.hi, -0.5 * q.hi);
    double lo = ((a.lo + b.lo) + c.lo) +
                ((Ed * OHG_LN2_MID + L.lo) + ((rl - 0.5 * q.lo) + ((rl * q.hi - rh * rl) + p3)));
    DD y = fast_two_sum(c.hi, lo);
    if (OHG_LIBM_QUICK && rounds_to_hi(y.hi, y.lo, 0x1p-66 * fabs(y.hi))) return y.hi;
  }
  // accurate evaluation, within about 2^-90:
  // log1p(r) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = r / (2 + r)
  DD s = dd_div(r, dd_add(DD{2.0, 0.0}, r));
  DD s2 = dd_mul(s, s);
  DD s3 = dd_mul(s2, s);
  double t = s2.hi;
  double tail = (s3.hi * t) *
                (2.0 / 5.0 + t * (2.0 / 7.0 + t * (2.0 / 9.0 + t * (2.0 / 11.0))));
  const DD two_thirds = {0.66666666666666663, 3.7007434154171883e-17};
  DD l1p = dd_add(DD{2.0 * s.hi, 2.0 * s.lo}, dd_add(dd_mul(s3, two_thirds), DD{tail, 0.0}));
  // E ln 2: E HI exact (|E| < 2^11), E MID exact by two_prod, E LO rounded
  DD eln2 = dd_add(DD{Ed * OHG_LN2_HI, 0.0}, two_prod(Ed, OHG_LN2_MID));
  eln2 = dd_add(eln2, DD{Ed * OHG_LN2_LO, 0.0});
  DD res = dd_add(dd_add(eln2, L), l1p);
  return res.hi + res.lo;
}

// ------------------------------------------------------------ exp
OHG_HD double exp_cr(double x) {
  if (!(x == x)) return x;
  if (x > 709.78271289338400) return INFINITY;
  if (x < -745.13321910194122) return 0.0;
  double kd = rint(x * OHG_INV_LN2_128);  // |k| < 2^17
  // r = x - k ln2/128: x - k HI exactly, then the MID and LO products
  double a = x - kd * OHG_LN2_128_HI;
  DD pm = two_prod(kd, OHG_LN2_128_MID);
  DD r = two_sum(a, -pm.hi);
  r.lo = (r.lo - pm.lo) - kd * OHG_LN2_128_LO;
  r = fast_two_sum(r.hi, r.lo);
  long long k = (long long)kd;
  int jj = int(k & 127);
  int q = int((k - jj) / 128);
  DD T = {OHG_LIBM_TAB(exp_hi)[jj], OHG_LIBM_TAB(exp_lo)[jj]};
  if (q > -1000 && q < 1000) {
    // quick evaluation, within 2^-69 relative: T (1 + r + r^2/2 + ...) with
    // T, T r and T r^2/2 added exactly, the rest in double
    double rh = r.hi, rl = r.lo;
    DD sq = two_prod(rh, rh);
    double p3 = (rh * sq.hi) *
                (1.0 / 6.0 + rh * (1.0 / 24.0 + rh * (1.0 / 120.0 + rh * (1.0 / 720.0 + rh / 5040.0))));
    DD a = two_prod(T.hi, rh);
    DD b = two_sum(T.hi, a.hi);
    DD c = two_prod(T.hi, 0.5 * sq.hi);
    DD d = two_sum(b.hi, c.hi);
    double lo = ((b.lo + d.lo) + (a.lo + c.lo)) +
                (T.lo + (T.hi * ((rl + 0.5 * sq.lo) + (rh * rl + p3)) + T.lo * rh));
    DD y = fast_two_sum(d.hi, lo);
    // y.hi 2^q: the exponent field moves by q (the result stays normal)
    if (OHG_LIBM_QUICK && rounds_to_hi(y.hi, y.lo, 0x1p-66 * fabs(y.hi)))
      return u2d(d2u(y.hi) + (std::uint64_t(std::int64_t(q)) << 52));
  }
  // accurate evaluation, within about 2^-90:
  // exp(r) - 1 = r + r^2/2 + r^3/6 + r^4 (1/24 + r/120 + ...), |r| < 2^-8.5
  DD r2 = dd_mul(r, r);
  DD r3 = dd_mul(r2, r);
  double rh = r.hi;
  double tail = (r2.hi * r2.hi) *
                (1.0 / 24.0 +
                 rh * (1.0 / 120.0 + rh * (1.0 / 720.0 + rh * (1.0 / 5040.0 + rh / 40320.0))));
  const DD sixth = {0.16666666666666666, 9.2518585385429707e-18};
  DD em1 = dd_add(r, dd_add(DD{0.5 * r2.hi, 0.5 * r2.lo}, dd_add(dd_mul(r3, sixth), DD{tail, 0.0})));
  DD res = dd_add(T, dd_mul(T, em1));
  double y = res.hi + res.lo;
  if (q > 1000) return 2.0 * ldexp(y, q - 1);  // keeps ldexp's argument in range
  return ldexp(y, q);
}

// ------------------------------------------------------------ sin, cos
// sin and cos of a double-double a with |a| <= pi/4 + 2^-7: a = c + t with
// c = j/64 from the table and |t| <= 2^-7, then the addition formulas with
// the Taylor series of sin t and cos t.  sn or cs may be null: only the
// other one is formed.
OHG_HD void sincos_dd(DD a, DD* sn, DD* cs) {
  bool neg = a.hi < 0.0;
  if (neg) a = dd_neg(a);
  int j = int(rint(a.hi * 64.0));
  j = j < 0 ? 0 : j > 51 ? 51 : j;
  DD t = two_sum(a.hi - double(j) * (1.0 / 64.0), a.lo);  // the subtraction is exact
  DD t2 = dd_mul(t, t);
  double th = t2.hi;
  // sin t = t - t^3/6 + t^5 (1/120 - t^2/5040 + t^4/362880)
  DD t3 = dd_mul(t2, t);
  const DD sixth = {0.16666666666666666, 9.2518585385429707e-18};
  double s5 = (t3.hi * th) * (1.0 / 120.0 + th * (-1.0 / 5040.0 + th * (1.0 / 362880.0)));
  DD st = dd_add(t, dd_add(dd_neg(dd_mul(t3, sixth)), DD{s5, 0.0}));
  // cos t = 1 - t^2/2 + t^4/24 - t^6/720 + t^8/40320 - t^10/3628800
  DD t4 = dd_mul(t2, t2);
  const DD inv24 = {0.041666666666666664, 2.3129646346357427e-18};
  double c6 = (t4.hi * th) * (-1.0 / 720.0 + th * (1.0 / 40320.0 + th * (-1.0 / 3628800.0)));
  DD ct = dd_add(DD{1.0, 0.0}, dd_add(DD{-0.5 * t2.hi, -0.5 * t2.lo},
                                      dd_add(dd_mul(t4, inv24), DD{c6, 0.0})));
  DD S = {OHG_LIBM_TAB(sin_hi)[j], OHG_LIBM_TAB(sin_lo)[j]};
  DD C = {OHG_LIBM_TAB(cos_hi)[j], OHG_LIBM_TAB(cos_lo)[j]};
  if (sn) {
    DD s_ = dd_add(dd_mul(S, ct), dd_mul(C, st));
    *sn = neg ? dd_neg(s_) : s_;
  }
  if (cs) *cs = dd_add(dd_mul(C, ct), dd_neg(dd_mul(S, st)));
}

// sin and cos of a double w with |w| <= pi/4 + 2^-7 in plain double
// arithmetic, the same table and series to degree 7: to a few units of
// 2^-53, for Newton steps whose result is refined in double-double.
OHG_HD void sincos_d(double w, double* sn, double* cs) {
  bool neg = w < 0.0;
  double a = neg ? -w : w;
  int j = int(rint(a * 64.0));
  j = j < 0 ? 0 : j > 51 ? 51 : j;
  double t = a - double(j) * (1.0 / 64.0);  // exact
  double t2 = t * t;
  double st = fma(t * t2, fma(t2, fma(t2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), t);
  double ct = fma(t2, fma(t2, fma(t2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0);
  double S = OHG_LIBM_TAB(sin_hi)[j], C = OHG_LIBM_TAB(cos_hi)[j];
  double s_ = fma(S, ct, C * st);
  *sn = neg ? -s_ : s_;
  *cs = fma(C, ct, -(S * st));
}

// cos x, correctly rounded for |x| <= 2^20 (the reduction by multiples of
// pi/2 carries about 139 bits of pi/2); beyond, the same steps run with
// less accuracy.
OHG_HD double cos_cr(double x) {
  if (x - x != 0.0) return NAN;  // inf, NaN
  double ax = fabs(x);
  if (ax < 0x1p-27) return 1.0;  // 1 - x^2/2 rounds to 1
  double kd = rint(ax * OHG_2_OVER_PI);
  DD r;
  if (kd == 0.0) {
    r = DD{ax, 0.0};
  } else {
    double a = ax - kd * OHG_PIO2_HI;  // exact for k < 2^20
    DD pm = two_prod(kd, OHG_PIO2_MID);
    r = two_sum(a, -pm.hi);
    r.lo = (r.lo - pm.lo) - kd * OHG_PIO2_LO;
    r = fast_two_sum(r.hi, r.lo);
  }
  long long q = (long long)fmod(kd, 4.0);
  DD v;
  if (q & 1) {
    sincos_dd(r, &v, nullptr);  // cos(r + k pi/2) = -+ sin r
    if (q == 1) v = dd_neg(v);
  } else {
    sincos_dd(r, nullptr, &v);
    if (q == 2) v = dd_neg(v);
  }
  return v.hi + v.lo;
}

// asin z for |z| <= 0.5 + 2^-10 as a double-double: a series start refined
// by Newton's iteration on sin w = z (cos w >= 0.85 there), twice in double
// (sincos_d) and once in double-double.
OHG_HD DD asin_dd_small(DD z) {
  double zh = z.hi, z2 = zh * zh;
  double w = zh * (1.0 + z2 * (1.0 / 6.0 + z2 * (3.0 / 40.0 + z2 * (15.0 / 336.0))));
  for (int it = 0; it < 2; ++it) {
    double sn, cs;
    sincos_d(w, &sn, &cs);
    w = w + (zh - sn) / cs;
  }
  DD sn, cs;
  DD wd = {w, 0.0};
  sincos_dd(wd, &sn, &cs);
  DD num = dd_add(z, dd_neg(sn));
  return dd_add(wd, dd_div(num, cs));
}

// square root of a non-negative double as a double-double
OHG_HD DD sqrt_dd(double a) {
  double s = sqrt(a);
  if (s == 0.0) return {0.0, 0.0};
  double e = fma(-s, s, a);  // a - s^2, exactly
  return fast_two_sum(s, e / (2.0 * s));
}

// acos x, correctly rounded (to about 2^-90 before the final rounding):
// pi/2 - asin x for |x| <= 1/2, 2 asin(sqrt((1 - x)/2)) above and
// pi - 2 asin(sqrt((1 + x)/2)) below (1 -+ x is exact there).
OHG_HD double acos_cr(double x) {
  if (!(fabs(x) <= 1.0)) return NAN;
  const DD pi = {OHG_PI_DD_HI, OHG_PI_DD_LO}, pio2 = {OHG_PIO2_DD_HI, OHG_PIO2_DD_LO};
  DD r;
  if (fabs(x) <= 0.5) {
    r = dd_add(pio2, dd_neg(asin_dd_small(DD{x, 0.0})));
  } else if (x > 0.0) {
    DD a = asin_dd_small(sqrt_dd((1.0 - x) * 0.5));
    r = DD{2.0 * a.hi, 2.0 * a.lo};
  } else {
    DD a = asin_dd_small(sqrt_dd((1.0 + x) * 0.5));
    r = dd_add(pi, DD{-2.0 * a.hi, -2.0 * a.lo});
  }
  return r.hi + r.lo;
}

}  // namespace ohg
