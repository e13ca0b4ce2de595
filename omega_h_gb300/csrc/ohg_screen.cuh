// FP32 screening of metric edge lengths and tet mean-ratio qualities with
// rigorous enclosures of the FP64 values.
//
// Every function here returns an interval [lo, hi] of floats that provably
// contains the value the FP64 kernels (ohg_math.cuh, the reference's
// arithmetic) compute for the same inputs.  Callers decide in FP32 where the
// interval settles a comparison and recompute in FP64 only where it does
// not, so every decision, and every real that is output, equals the FP64 one.
//
// How the enclosure is argued:
//  * inputs are FP64 values; each is carried as a float with an absolute
//    error bound (coordinates as hi + lo float pairs, so coordinate
//    differences are accurate to the edge length, not the coordinate size);
//  * sums of products (triple product, v^T M v) get the classical bound
//    gamma_k * (the same expression on absolute values) for the rounding of
//    both the float and the double evaluation, plus a first-order-exact
//    perturbation term for the input errors;
//  * monotone steps (sqrt, cbrt, the final division, the logarithmic mean)
//    map interval endpoints with directed rounding: a correctly rounded or
//    1-ulp double operation of a value inside [lo, hi] lands inside the same
//    float interval because rounding is monotone and float endpoints are
//    doubles;
//  * bound arithmetic itself is done in round-to-nearest on non-negative
//    terms and inflated by (1 + 2^-15), which covers the relative error of
//    the at most ~200 roundings along any chain;
//  * cbrtf, logf (CUDA: at most 1 ulp) and the double cbrt and log
//    (correctly rounded) are covered by widening their results by
//    2^-20 / 2^-15 relative;
//  * anything non-finite widens the interval to [-inf, +inf].
#pragma once
#include <cfloat>
#include <cstring>

#include "ohg_common.cuh"
#include "ohg_math.cuh"

namespace ohg {

constexpr float kU = 0x1p-24f;          // float unit roundoff
constexpr float kInflate = 1.0f + 0x1p-15f;
constexpr float kTiny = 1e-35f;         // covers subnormal rounding
// relative rounding of one float and one double operation, with margin:
// kC1 >= (u + u_double)(1 + u), kC2 >= 2 kC1
constexpr float kC1 = 0x1.004p-24f;
constexpr float kC2 = 0x1.004p-23f;
constexpr float kSixth = 1.0f / 6.0f;    // float(1/6), within u of 1/6
constexpr float kSixthUp = 0.16666669f;  // above 1/6

// Per-vertex screening data (built by build_vert_screen).
//  xh = (x_hi, y_hi, z_hi, max |hi|), xl = (x_lo, y_lo, z_lo, 0) with
//  x = x_hi + x_lo to about 2^-48 |x|;
//  ma = (xx, yy, zz, yx), mb = (zy, zx, S0 = sum |M_ij|, sqrt(det M) as float);
//  dkey = order-preserving integer key of det M (maxdet choice, exact);
//  sdet = sqrt(det M) in double, identical to what the reference computes
//  per element from the same metric.
//  An isotropic metric m (one component) is held as the tensor diag(m):
//  its float products and sums bound the reference's scalar evaluation as
//  they bound the tensor one; dkey orders m itself and sdet is the
//  reference's size factor power<dim, 2>(m).  mc is the number of metric
//  components of the mesh (1: isotropic).
struct VertScreen {
  Arr<float4> xh, xl, ma, mb;
  Arr<long long> dkey;
  Arr<double> sdet;
  int mc = 0;
};

struct ScreenView {
  View<const float4> xh, xl, ma, mb;
  View<const long long> dkey;
  View<const double> sdet;
  int mc;
};
inline ScreenView screen_view(const VertScreen& s) {
  return {cview(s.xh), cview(s.xl), cview(s.ma), cview(s.mb), cview(s.dkey), cview(s.sdet), s.mc};
}

// order-preserving map of a double to a signed 64-bit key (+0 and -0 equal)
__host__ __device__ __forceinline__ long long order_key(double d) {
  if (d == 0.0) return 0;
#ifdef __CUDA_ARCH__
  long long b = __double_as_longlong(d);
#else
  long long b;
  std::memcpy(&b, &d, sizeof(b));
#endif
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// inverse of order_key (zero comes back as +0)
__host__ __device__ __forceinline__ double key_to_double(long long k) {
  long long b = k >= 0 ? k : (k ^ 0x7fffffffffffffffLL);
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double d;
  std::memcpy(&d, &b, sizeof(d));
  return d;
#endif
}

struct FIv {
  float lo, hi;
};

__device__ __forceinline__ FIv widen_all() { return {-INFINITY, INFINITY}; }
__device__ __forceinline__ bool finite_iv(FIv a) { return a.lo >= -FLT_MAX && a.hi <= FLT_MAX && a.lo <= a.hi; }

// coordinate difference p1 - p0 (3 floats) and its infinity-norm error bound
// against fl64(p1 - p0)
__device__ __forceinline__ float sdiff3(float4 h1, float4 l1, float4 h0, float4 l0, float v[3]) {
  v[0] = __fadd_rn(__fsub_rn(h1.x, h0.x), __fsub_rn(l1.x, l0.x));
  v[1] = __fadd_rn(__fsub_rn(h1.y, h0.y), __fsub_rn(l1.y, l0.y));
  v[2] = __fadd_rn(__fsub_rn(h1.z, h0.z), __fsub_rn(l1.z, l0.z));
  float n = fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2])));
  // 2u|v| from the float roundings, ~6u^2 |x| from the lo parts and the
  // hi/lo split, u_double |v| from the double subtraction
  return __fmaf_rn(n, kC2, __fmaf_rn(__fadd_rn(h1.w, h0.w), 0x1p-44f, kTiny));
}

// q = v^T M v in float with the absolute-value sums the bound needs:
// A = |v|^T |M| |v|, S1 = 1^T |M| |v|
__device__ __forceinline__ float mprod(float4 ma, float4 mb, const float v[3], float& A, float& S1) {
  float xx = ma.x, yy = ma.y, zz = ma.z, yx = ma.w, zy = mb.x, zx = mb.y;
  float y0 = __fmaf_rn(zx, v[2], __fmaf_rn(yx, v[1], __fmul_rn(xx, v[0])));
  float y1 = __fmaf_rn(zy, v[2], __fmaf_rn(yy, v[1], __fmul_rn(yx, v[0])));
  float y2 = __fmaf_rn(zz, v[2], __fmaf_rn(zy, v[1], __fmul_rn(zx, v[0])));
  float q = __fmaf_rn(v[2], y2, __fmaf_rn(v[1], y1, __fmul_rn(v[0], y0)));
  float a0 = fabsf(v[0]), a1 = fabsf(v[1]), a2 = fabsf(v[2]);
  float axx = fabsf(xx), ayy = fabsf(yy), azz = fabsf(zz), ayx = fabsf(yx), azy = fabsf(zy),
        azx = fabsf(zx);
  float w0 = __fmaf_rn(azx, a2, __fmaf_rn(ayx, a1, __fmul_rn(axx, a0)));
  float w1 = __fmaf_rn(azy, a2, __fmaf_rn(ayy, a1, __fmul_rn(ayx, a0)));
  float w2 = __fmaf_rn(azz, a2, __fmaf_rn(azy, a1, __fmul_rn(azx, a0)));
  S1 = __fadd_rn(__fadd_rn(w0, w1), w2);
  A = __fmaf_rn(a2, w2, __fmaf_rn(a1, w1, __fmul_rn(a0, w0)));
  return q;
}

// error bound of one v^T M v against the double evaluation of the same
// product from the double inputs, given the infinity-norm error e of v:
// rounding of both evaluations (6 roundings per term, float and double) and
// of the metric's conversion to float (u A), plus the input perturbation
// 2 e S1 + e^2 S0 (exact to first and second order for a symmetric M)
__device__ __forceinline__ float mprod_err(float A, float S1, float S0, float e) {
  float pert = __fmaf_rn(e, __fmaf_rn(2.0f, S1, __fmul_rn(e, S0)), 0.0f);
  return __fmaf_rn(7.1f * kU, A, __fmaf_rn(pert, 1.0f + kU, kTiny));
}

// Interval of the double metric edge length (edge_length3: the logarithmic
// mean of sqrt(v^T M0 v) and sqrt(v^T M1 v)) between vertices a and b.
// Enclosures [lo[k], hi[k]] of the double v^T M_k v at the two ends (k = 0:
// vertex a) of the edge a-b; false when an enclosure is not positive and
// finite (the length enclosure is then unbounded).
__device__ __forceinline__ bool edge_q_bounds3(const ScreenView& s, LO a, LO b, float lo[2],
                                               float hi[2]) {
  float4 ha = s.xh[a], la = s.xl[a], hb = s.xh[b], lb = s.xl[b];
  float v[3];
  float e = sdiff3(hb, lb, ha, la, v);  // p1 - p0 with p0 = a
  LO vs[2] = {a, b};
  bool ok = true;
  for (int k = 0; k < 2; ++k) {
    float4 ma = s.ma[vs[k]], mb = s.mb[vs[k]];
    float A, S1;
    float q = mprod(ma, mb, v, A, S1);
    float qe = __fmul_rn(mprod_err(A, S1, mb.z, e), kInflate);
    lo[k] = __fsub_rd(q, qe);
    hi[k] = __fadd_ru(q, qe);
    ok = ok && lo[k] > 0.0f && hi[k] <= FLT_MAX;
  }
  return ok;
}

__device__ __forceinline__ FIv log_mean_bounds(const float l_lo[2], const float l_hi[2]);

// the length enclosure from positive, finite end enclosures
__device__ __forceinline__ FIv len_from_q(const float lo[2], const float hi[2]) {
  float l_lo[2], l_hi[2];
  for (int k = 0; k < 2; ++k) {
    l_lo[k] = __fsqrt_rd(lo[k]);
    l_hi[k] = __fsqrt_ru(hi[k]);
  }
  return log_mean_bounds(l_lo, l_hi);
}

__device__ __forceinline__ FIv edge_len_bounds(const ScreenView& s, LO a, LO b) {
  float lo[2], hi[2];
  if (!edge_q_bounds3(s, a, b, lo, hi)) return widen_all();
  return len_from_q(lo, hi);
}

// A threshold test of the double edge length from the end enclosures alone.
// The logarithmic mean lies between the two end lengths, so when both end
// lengths are below (at or above) a threshold, so is the exact mean; the
// double evaluation then adds a relative error d <= 2^-50 (1 + 300 l) for
// end lengths l (the bound log_mean_bounds applies), at most
// 2^-50 (1 + 300 * 1025) = 307501 * 2^-50 while the squared enclosures stay
// below kLenCutQCap = 2^20.  For floats t_dn <= T <= t_up, below_q and
// above_q are squared end lengths under which the double length is < t_dn,
// and over which it is >= t_up: below_q <= (t_dn / (1 + d))^2 and
// above_q >= (t_up / (1 - d))^2, rounded outward.
constexpr float kLenCutQCap = 0x1p20f;
constexpr float kLenCutD = 307501.0f * 0x1p-50f;
struct LenCut {
  float below_q, above_q;
};
__device__ __forceinline__ LenCut len_cut(float t_dn, float t_up) {
  if (!(t_dn > 0.0f) || !(t_up <= FLT_MAX)) return {-1.0f, INFINITY};
  float sb = __fdiv_rd(t_dn, __fadd_ru(1.0f, kLenCutD));
  float sa = __fdiv_ru(t_up, __fsub_rd(1.0f, kLenCutD));
  return {__fmul_rd(sb, sb), __fmul_ru(sa, sa)};
}
// -1: the double length is < t_dn; +1: it is >= t_up; 0: not settled (also
// when the enclosures are not positive and finite)
__device__ __forceinline__ int len_cut_side(const float lo[2], const float hi[2], bool ok,
                                            const LenCut& c) {
  if (!ok) return 0;
  float hmax = fmaxf(hi[0], hi[1]), lmin = fminf(lo[0], lo[1]);
  if (!(hmax <= kLenCutQCap)) return 0;
  if (hmax < c.below_q) return -1;
  if (lmin >= c.above_q) return 1;
  return 0;
}


// index (0..3) of the vertex whose metric has the largest determinant, the
// first one on ties (maxdet_metric, src/Omega_h_metric.hpp:170-182)
__device__ __forceinline__ int maxdet_vertex(const ScreenView& s, const LO vv[4]) {
  int best = 0;
  long long bk = s.dkey[vv[0]];
  for (int i = 1; i < 4; ++i) {
    long long k = s.dkey[vv[i]];
    if (k > bk) {
      best = i;
      bk = k;
    }
  }
  return best;
}

// Running sums over a tet's edges v (float) with error bounds e for the mean
// squared metric length: G = sum v v^T, H = the off-diagonal of sum |v||v|^T,
// W = sum e |v| and sum e^2.  Each entry is a sum of at most six products,
// whose float rounding bound (gamma_6) holds in any order of accumulation.
struct GramAcc {
  float gxx = 0.0f, gyy = 0.0f, gzz = 0.0f, gxy = 0.0f, gyz = 0.0f, gzx = 0.0f;
  float hxy = 0.0f, hyz = 0.0f, hzx = 0.0f;
  float wx = 0.0f, wy = 0.0f, wz = 0.0f, esq = 0.0f;
  __device__ __forceinline__ void add(const float v[3], float e) {
    float ax = fabsf(v[0]), ay = fabsf(v[1]), az = fabsf(v[2]);
    gxx = __fmaf_rn(v[0], v[0], gxx);
    gyy = __fmaf_rn(v[1], v[1], gyy);
    gzz = __fmaf_rn(v[2], v[2], gzz);
    gxy = __fmaf_rn(v[0], v[1], gxy);
    gyz = __fmaf_rn(v[1], v[2], gyz);
    gzx = __fmaf_rn(v[2], v[0], gzx);
    hxy = __fmaf_rn(ax, ay, hxy);
    hyz = __fmaf_rn(ay, az, hyz);
    hzx = __fmaf_rn(az, ax, hzx);
    wx = __fmaf_rn(e, ax, wx);
    wy = __fmaf_rn(e, ay, wy);
    wz = __fmaf_rn(e, az, wz);
    esq = __fmaf_rn(e, e, esq);
  }
};

// The parts of a tet quality interval from the triple product T (six times
// the signed volume, against the double T by at most eT) and the edge sums
// of G: the size s = T/6 sqrt(det M) within es, the mean squared length msl
// within [msl_lo, msl_hi], and y = (s / s_equilateral)^2 within ey.  The
// return value says which case holds: 0 the parts are valid (s settled
// non-negative), 1 unbounded, 2 the size is surely negative (the quality is
// s itself: [s_lo, s_hi]), 3 the size's sign is not settled.
struct TetTail {
  float sv, es, msl_lo, msl_hi, y, ey;
};
__device__ __forceinline__ int tet_tail_parts(float T, float eT, const GramAcc& G, float4 ma,
                                              float4 mb, TetTail& o) {
  // rs = T / 6 (here T times float(1/6): one more rounding, so kC2), s = rs * sqrt(det M)
  float rs = __fmul_rn(T, kSixth);
  float ers = __fmaf_rn(fabsf(rs), kC2, __fmul_rn(eT, kSixthUp));
  float sd = mb.w;
  float sv = __fmul_rn(rs, sd);
  float es = __fmaf_rn(fabsf(sv), kC2, __fmul_rn(__fmul_rn(ers, fabsf(sd)), 1.0f + 0x1p-20f));
  es = __fmul_rn(es, kInflate);
  o.sv = sv;
  o.es = es;
  if (!(fabsf(sv) <= FLT_MAX) || !(es <= FLT_MAX)) return 1;
  if (__fadd_ru(sv, es) < 0.0f) return 2;  // negative size
  float s_lo = __fsub_rd(sv, es);
  // mean squared metric length: the sum over the six edges of v^T M v is
  // the contraction M : G with G = sum v v^T.  Its float evaluation differs
  // from the exact value for the float edges and float metric by at most
  // (gamma_6 for G, gamma_4 for the contraction) times
  // asum = sum |v|^T |M| |v| = |M| : (sum |v| |v|^T); the metric's
  // conversion to float adds u asum and the double evaluation far less
  // (12.2 u asum in all).  The edge errors e_i perturb the sum by at most
  // sum 2 e_i 1^T |M| |v_i| + e_i^2 S0 = 2 c . w + S0 sum e_i^2, with c the
  // column sums of |M| and w = sum e_i |v_i|.
  float mxx = ma.x, myy = ma.y, mzz = ma.z, myx = ma.w, mzy = mb.x, mzx = mb.y;
  float dg = __fmaf_rn(mzz, G.gzz, __fmaf_rn(myy, G.gyy, __fmul_rn(mxx, G.gxx)));
  float od = __fmaf_rn(mzx, G.gzx, __fmaf_rn(mzy, G.gyz, __fmul_rn(myx, G.gxy)));
  float msum = __fmaf_rn(2.0f, od, dg);
  float axx = fabsf(mxx), ayy = fabsf(myy), azz = fabsf(mzz), ayx = fabsf(myx), azy = fabsf(mzy),
        azx = fabsf(mzx);
  float adg = __fmaf_rn(azz, G.gzz, __fmaf_rn(ayy, G.gyy, __fmul_rn(axx, G.gxx)));
  float aod = __fmaf_rn(azx, G.hzx, __fmaf_rn(azy, G.hyz, __fmul_rn(ayx, G.hxy)));
  float asum = __fmaf_rn(2.0f, aod, adg);
  float cx = __fadd_rn(__fadd_rn(axx, ayx), azx);
  float cy = __fadd_rn(__fadd_rn(ayx, ayy), azy);
  float cz = __fadd_rn(__fadd_rn(azx, azy), azz);
  float cw = __fmaf_rn(cz, G.wz, __fmaf_rn(cy, G.wy, __fmul_rn(cx, G.wx)));
  float pert = __fmul_rn(__fmaf_rn(2.0f, cw, __fmul_rn(mb.z, G.esq)), 1.0f + kU);
  float msl = __fmul_rn(msum, kSixth);
  float emsl = __fmaf_rn(fabsf(msl), kC2,
                         __fmul_rn(__fmaf_rn(12.2f * kU, asum, __fadd_rn(pert, 16.0f * kTiny)),
                                   kSixthUp));
  emsl = __fmul_rn(emsl, kInflate);
  o.msl_lo = __fsub_rd(msl, emsl);
  o.msl_hi = __fadd_ru(msl, emsl);
  // the range keeps __fdividef within its documented 2-ulp error
  if (!(o.msl_lo > 1e-30f) || !(o.msl_hi < 1e30f)) return 1;
  if (s_lo < 0.0f) return 3;
  // x = s / 0.1178511301977579, y = x * x
  float x = __fmul_rn(sv, 8.485281374238571f);
  float ex = __fmaf_rn(fabsf(x), kC2, __fmul_rn(es, 8.4853f));
  float y = __fmul_rn(x, x);
  float ey = __fmaf_rn(fabsf(y), kC1, __fmul_rn(ex, __fmaf_rn(2.0f, fabsf(x), ex)));
  o.y = y;
  o.ey = __fmul_rn(ey, kInflate);
  if (!(y < 1e30f) || !(o.ey < 1e30f)) return 1;  // keeps __fdividef in range
  return 0;
}

// The quality interval: q = cbrt(y) / msl.
__device__ __forceinline__ FIv tet_bounds_tail(float T, float eT, const GramAcc& G, float4 ma,
                                               float4 mb) {
  TetTail t;
  int c = tet_tail_parts(T, eT, G, ma, mb, t);
  if (c == 1) return widen_all();
  if (c == 2) return {__fsub_rd(t.sv, t.es), __fadd_ru(t.sv, t.es)};
  // sign of the size not settled: the value is either s (>= s_lo) or a
  // non-negative quality
  if (c == 3) return {__fsub_rd(t.sv, t.es), INFINITY};
  float y = t.y, ey = t.ey;
  // cbrt over [y - ey, y + ey] from one cbrtf (at most 1 ulp; the double
  // cbrt is correctly rounded): with d = ey / y,
  //   (1 + d)^(1/3) <= 1 + d/3 and (1 - d)^(1/3) >= 1 - d/3 - d^2 (d <= 1/2)
  float r_lo, r_hi;
  if (!(y > 1e-30f)) {
    r_lo = 0.0f;
    r_hi = __fmul_ru(cbrtf(__fadd_ru(fmaxf(y, 0.0f), ey)), 1.0f + 0x1p-20f);
  } else {
    float cy = cbrtf(y);
    float d = __fmul_ru(__fdividef(ey, y), 1.0f + 0x1p-21f);
    r_hi = __fmul_ru(__fmul_ru(cy, 1.0f + 0x1p-21f), __fmaf_ru(d, 0.33333334f, 1.0f));
    if (d <= 0.5f) {
      float f = __fsub_rd(__fmaf_rd(-d, 0.33333334f, 1.0f), __fmul_ru(d, d));
      r_lo = __fmul_rd(__fmul_rd(cy, 1.0f - 0x1p-21f), f);
    } else {
      r_lo = 0.0f;
    }
  }
  // q = r / msl; __fdividef is within 2 ulp for divisors in [2^-126, 2^126]
  FIv q = {__fmul_rd(__fdividef(r_lo, t.msl_hi), 1.0f - 0x1p-21f),
           __fmul_ru(__fdividef(r_hi, t.msl_lo), 1.0f + 0x1p-21f)};
  if (!finite_iv(q)) return widen_all();
  return q;
}

// The cube of the quality interval, without a cube root: q^3 = y / msl^3
// is monotone in q, so minima and comparisons with a threshold's cube carry
// over.  The double quality is fl(cbrt(Y) / M) with Y the double y and M the
// double msl (correctly rounded cbrt, rounded division: within 2 u_double of
// cbrt(Y) / M), so its cube lies within (1 +- 6.1 u_double) of Y / M^3;
// [y_lo, y_hi] holds Y and [msl_lo, msl_hi] holds M.  The float quotient
// (__fdividef, 2 ulp, divisor kept in [1e-30, 1e30]) is widened by 2^-20.
// A surely negative size gives [-inf, 0] (the quality is negative); an
// unsettled sign [-inf, inf].
__device__ __forceinline__ FIv tet_bounds_tail_cubed(float T, float eT, const GramAcc& G,
                                                     float4 ma, float4 mb) {
  TetTail t;
  int c = tet_tail_parts(T, eT, G, ma, mb, t);
  if (c == 1 || c == 3) return widen_all();
  if (c == 2) return {-INFINITY, 0.0f};
  if (!(t.msl_lo > 1e-10f) || !(t.msl_hi < 1e10f)) return widen_all();
  float y_lo = fmaxf(__fsub_rd(t.y, t.ey), 0.0f), y_hi = __fadd_ru(t.y, t.ey);
  float m3_hi = __fmul_ru(__fmul_ru(t.msl_hi, t.msl_hi), t.msl_hi);
  float m3_lo = __fmul_rd(__fmul_rd(t.msl_lo, t.msl_lo), t.msl_lo);
  FIv q = {__fmul_rd(__fdividef(y_lo, m3_hi), 1.0f - 0x1p-20f),
           __fmul_ru(__fdividef(y_hi, m3_lo), 1.0f + 0x1p-20f)};
  if (!finite_iv(q)) return widen_all();
  return q;
}

// Interval of the double tet quality (tet_quality on the maxdet metric), from
// the four vertices' coordinate pairs and the maxdet vertex's metric record.
template <bool cubed = false>
__device__ __forceinline__ FIv tet_quality_bounds_of(const float4 h[4], const float4 l[4],
                                                     float4 ma, float4 mb) {
  // the six edges in the reference's order; the third, -b1, has the same
  // v^T M v as b1
  float ev[6][3], ee[6];
  ee[0] = sdiff3(h[1], l[1], h[0], l[0], ev[0]);
  ee[1] = sdiff3(h[2], l[2], h[1], l[1], ev[1]);
  ee[2] = sdiff3(h[2], l[2], h[0], l[0], ev[2]);
  ee[3] = sdiff3(h[3], l[3], h[0], l[0], ev[3]);
  ee[4] = sdiff3(h[3], l[3], h[1], l[1], ev[4]);
  ee[5] = sdiff3(h[3], l[3], h[2], l[2], ev[5]);
  const float* b0 = ev[0];
  const float* b1 = ev[2];
  const float* b2 = ev[3];
  float e0 = ee[0], e1 = ee[2], e2 = ee[3];
  // triple product T = (b0 x b1) . b2
  float c0 = __fmaf_rn(b0[1], b1[2], -__fmul_rn(b0[2], b1[1]));
  float c1 = __fmaf_rn(b0[2], b1[0], -__fmul_rn(b0[0], b1[2]));
  float c2 = __fmaf_rn(b0[0], b1[1], -__fmul_rn(b0[1], b1[0]));
  float T = __fmaf_rn(c2, b2[2], __fmaf_rn(c1, b2[1], __fmul_rn(c0, b2[0])));
  float P = __fmaf_rn(
      fabsf(b2[2]), __fmaf_rn(fabsf(b0[0]), fabsf(b1[1]), __fmul_rn(fabsf(b0[1]), fabsf(b1[0]))),
      __fmaf_rn(fabsf(b2[1]),
                __fmaf_rn(fabsf(b0[2]), fabsf(b1[0]), __fmul_rn(fabsf(b0[0]), fabsf(b1[2]))),
                __fmul_rn(fabsf(b2[0]), __fmaf_rn(fabsf(b0[1]), fabsf(b1[2]),
                                                  __fmul_rn(fabsf(b0[2]), fabsf(b1[1]))))));
  float n0 = fmaxf(fabsf(b0[0]), fmaxf(fabsf(b0[1]), fabsf(b0[2])));
  float n1 = fmaxf(fabsf(b1[0]), fmaxf(fabsf(b1[1]), fabsf(b1[2])));
  float n2 = fmaxf(fabsf(b2[0]), fmaxf(fabsf(b2[1]), fabsf(b2[2])));
  // input perturbation of the trilinear T: first order |d0 . (b1 x b2)| <=
  // e0 * sum |b1 x b2| (absolute-value form) and cyclically; every term of
  // second and third order is below 6 e e n
  float a0[3] = {fabsf(b0[0]), fabsf(b0[1]), fabsf(b0[2])};
  float a1[3] = {fabsf(b1[0]), fabsf(b1[1]), fabsf(b1[2])};
  float a2[3] = {fabsf(b2[0]), fabsf(b2[1]), fabsf(b2[2])};
  float c12 = 0.0f, c20 = 0.0f, c01 = 0.0f;
  for (int i = 0; i < 3; ++i) {
    int j = (i + 1) % 3, k = (i + 2) % 3;
    c12 = __fadd_rn(c12, __fmaf_rn(a1[j], a2[k], __fmul_rn(a1[k], a2[j])));
    c20 = __fadd_rn(c20, __fmaf_rn(a2[j], a0[k], __fmul_rn(a2[k], a0[j])));
    c01 = __fadd_rn(c01, __fmaf_rn(a0[j], a1[k], __fmul_rn(a0[k], a1[j])));
  }
  float first = __fmaf_rn(e0, c12, __fmaf_rn(e1, c20, __fmul_rn(e2, c01)));
  float second = __fmul_rn(
      6.0f, __fmaf_rn(__fmul_rn(e0, e1), __fadd_rn(n2, e2),
                      __fmaf_rn(__fmul_rn(e0, e2), n1, __fmul_rn(__fmul_rn(e1, e2), n0))));
  float eT = __fmaf_rn(5.1f * kU, P, __fadd_rn(__fadd_rn(first, second), kTiny));
  GramAcc G;
#pragma unroll
  for (int i = 0; i < 6; ++i) G.add(ev[i], ee[i]);
  return cubed ? tet_bounds_tail_cubed(T, eT, G, ma, mb) : tet_bounds_tail(T, eT, G, ma, mb);
}

// The same interval for the tets of a collapse, with the parts that do not
// depend on the vertex moved onto computed once per element.
//
// A star element of the collapsing vertex keeps the face opposite that
// vertex's slot k; the new tet puts the vertex p moved onto at slot k.  With
// the face's vertices f0, f1, f2 in slot order, the triple product of the
// reference, det[x1 - x0, x2 - x0, x3 - x0] in slot order, equals
// (u x w) . (p - f0) with (u, w) = (f2 - f0, f1 - f0) for k even and
// (f1 - f0, f2 - f0) for k odd (expand the determinant along the column of
// p).  So n = u x w, its absolute-value form and the face's three edges'
// Gram sums are invariants of the element.
//
// The float evaluation of (u x w) . d has the same structure, and the same
// rounding bound 5.1 u P with P = |d| . (|u| x |w|)_abs, as the reference
// order's (b0 x b1) . b2; its input perturbation is bounded as there, with
// the first-order terms e_u sum|w x d|_abs <= e_u |w|_1 |d|_1 (likewise for
// w) and e_d sum (|u| x |w|)_abs.  The double value differs from the exact
// triple product of the exact coordinate differences by at most
// 8.1 u_double P_ref (five roundings of the evaluation and one per edge
// difference), P_ref <= 6 L^3 with L bounding every edge component of the
// new tet: 2^-47 L^3 covers it.
struct TetFaceInv {
  float4 a, b, c, d, e, f;
  // a = (n, sum (|u| x |w|)_abs), b = ((|u| x |w|)_abs, e_u |w|_1 + e_w |u|_1),
  // c = (e_u e_w, e_u |w|_inf + e_w |u|_inf, L of the face edges, sum e^2),
  // d..f = the face edges' Gram sums (gxx gyy gzz gxy | gyz gzx hxy hyz |
  // hzx wx wy wz)
};

__device__ __forceinline__ TetFaceInv tet_face_invariants(const float4 h[3], const float4 l[3],
                                                          int k) {
  float u[3], w[3], t[3];
  float eu, ew;
  if (k & 1) {
    eu = sdiff3(h[1], l[1], h[0], l[0], u);
    ew = sdiff3(h[2], l[2], h[0], l[0], w);
  } else {
    eu = sdiff3(h[2], l[2], h[0], l[0], u);
    ew = sdiff3(h[1], l[1], h[0], l[0], w);
  }
  float et = sdiff3(h[2], l[2], h[1], l[1], t);
  float n0 = __fmaf_rn(u[1], w[2], -__fmul_rn(u[2], w[1]));
  float n1 = __fmaf_rn(u[2], w[0], -__fmul_rn(u[0], w[2]));
  float n2 = __fmaf_rn(u[0], w[1], -__fmul_rn(u[1], w[0]));
  float au[3] = {fabsf(u[0]), fabsf(u[1]), fabsf(u[2])};
  float aw[3] = {fabsf(w[0]), fabsf(w[1]), fabsf(w[2])};
  float A0 = __fmaf_rn(au[1], aw[2], __fmul_rn(au[2], aw[1]));
  float A1 = __fmaf_rn(au[2], aw[0], __fmul_rn(au[0], aw[2]));
  float A2 = __fmaf_rn(au[0], aw[1], __fmul_rn(au[1], aw[0]));
  float cuw = __fadd_rn(__fadd_rn(A0, A1), A2);
  float nu = fmaxf(au[0], fmaxf(au[1], au[2]));
  float nw = fmaxf(aw[0], fmaxf(aw[1], aw[2]));
  float nt = fmaxf(fabsf(t[0]), fmaxf(fabsf(t[1]), fabsf(t[2])));
  float u1 = __fadd_rn(__fadd_rn(au[0], au[1]), au[2]);
  float w1 = __fadd_rn(__fadd_rn(aw[0], aw[1]), aw[2]);
  float K1 = __fmaf_rn(eu, w1, __fmul_rn(ew, u1));
  float E2a = __fmul_rn(eu, ew);
  float E2b = __fmaf_rn(eu, nw, __fmul_rn(ew, nu));
  float L = fmaxf(__fadd_rn(nu, eu), fmaxf(__fadd_rn(nw, ew), __fadd_rn(nt, et)));
  GramAcc G;
  G.add(u, eu);
  G.add(w, ew);
  G.add(t, et);
  TetFaceInv r;
  r.a = make_float4(n0, n1, n2, cuw);
  r.b = make_float4(A0, A1, A2, K1);
  r.c = make_float4(E2a, E2b, L, G.esq);
  r.d = make_float4(G.gxx, G.gyy, G.gzz, G.gxy);
  r.e = make_float4(G.gyz, G.gzx, G.hxy, G.hyz);
  r.f = make_float4(G.hzx, G.wx, G.wy, G.wz);
  return r;
}

// Interval of the double quality of the tet that puts p at the slot the
// invariants were made for (cubed: of its cube); hf/lf the face vertices in
// slot order, ma/mb the metric record of the new tet's maxdet vertex.
template <bool cubed>
__device__ __forceinline__ FIv tet_face_bounds(const TetFaceInv& f, const float4 hf[3],
                                               const float4 lf[3], float4 hp, float4 lp,
                                               float4 ma, float4 mb) {
  float d0[3], d1[3], d2[3];
  float e0 = sdiff3(hp, lp, hf[0], lf[0], d0);
  float e1 = sdiff3(hp, lp, hf[1], lf[1], d1);
  float e2 = sdiff3(hp, lp, hf[2], lf[2], d2);
  float T = __fmaf_rn(f.a.z, d0[2], __fmaf_rn(f.a.y, d0[1], __fmul_rn(f.a.x, d0[0])));
  float P = __fmaf_rn(fabsf(d0[2]), f.b.z, __fmaf_rn(fabsf(d0[1]), f.b.y,
                                                     __fmul_rn(fabsf(d0[0]), f.b.x)));
  float n_d = fmaxf(fabsf(d0[0]), fmaxf(fabsf(d0[1]), fabsf(d0[2])));
  float d_1 = __fadd_rn(__fadd_rn(fabsf(d0[0]), fabsf(d0[1])), fabsf(d0[2]));
  float first = __fmaf_rn(f.b.w, d_1, __fmul_rn(e0, f.a.w));
  float second = __fmul_rn(6.0f, __fmaf_rn(f.c.x, __fadd_rn(n_d, e0), __fmul_rn(e0, f.c.y)));
  float n1 = fmaxf(fabsf(d1[0]), fmaxf(fabsf(d1[1]), fabsf(d1[2])));
  float n2 = fmaxf(fabsf(d2[0]), fmaxf(fabsf(d2[1]), fabsf(d2[2])));
  float L = fmaxf(f.c.z, fmaxf(__fadd_rn(n_d, e0), fmaxf(__fadd_rn(n1, e1), __fadd_rn(n2, e2))));
  float dbl = __fmul_rn(0x1p-47f, __fmul_rn(L, __fmul_rn(L, L)));
  float eT = __fmaf_rn(5.1f * kU, P, __fadd_rn(__fadd_rn(__fadd_rn(first, second), dbl), kTiny));
  GramAcc G;
  G.gxx = f.d.x;
  G.gyy = f.d.y;
  G.gzz = f.d.z;
  G.gxy = f.d.w;
  G.gyz = f.e.x;
  G.gzx = f.e.y;
  G.hxy = f.e.z;
  G.hyz = f.e.w;
  G.hzx = f.f.x;
  G.wx = f.f.y;
  G.wy = f.f.z;
  G.wz = f.f.w;
  G.esq = f.c.w;
  G.add(d0, e0);
  G.add(d1, e1);
  G.add(d2, e2);
  return cubed ? tet_bounds_tail_cubed(T, eT, G, ma, mb) : tet_bounds_tail(T, eT, G, ma, mb);
}

template <bool cubed = false>
__device__ __forceinline__ FIv tet_quality_bounds(const ScreenView& s, const LO vv[4]) {
  int mi = maxdet_vertex(s, vv);
  float4 h[4], l[4];
  for (int i = 0; i < 4; ++i) {
    h[i] = s.xh[vv[i]];
    l[i] = s.xl[vv[i]];
  }
  return tet_quality_bounds_of<cubed>(h, l, s.ma[vv[mi]], s.mb[vv[mi]]);
}

// The double tet quality with sqrt(det M) and the maxdet choice taken from
// the per-vertex screening data: the same operations, in the same order, as
// tet_quality(p, metric of the maxdet vertex), since sqrt(det3(M)) of a
// vertex metric is the same double wherever it is computed.
__device__ __forceinline__ double tet_quality_exact(const ScreenView& s, View<const double> c,
                                                    View<const double> mt, const LO vv[4]) {
  int mi = maxdet_vertex(s, vv);
  V3 p[4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) p[i].x[j] = c[vv[i] * 3 + j];
  double sdet = s.sdet[vv[mi]];
  V3 b0 = sub3(p[1], p[0]), b1 = sub3(p[2], p[0]), b2 = sub3(p[3], p[0]);
  double rs = dot3(cross3(b0, b1), b2) / 6.0;
  double sz = rs * sdet;
  if (sz < 0) return sz;
  V3 nb1 = {{-b1.x[0], -b1.x[1], -b1.x[2]}};
  V3 ev[6] = {b0, sub3(p[2], p[1]), nb1, b2, sub3(p[3], p[1]), sub3(p[3], p[2])};
  double msl = 0;
  if (s.mc == 1) {
    double m = mt[vv[mi]];
    for (int i = 0; i < 6; ++i) msl += iso_product3(m, ev[i]);
  } else {
    M3 m = symm3(&mt[vv[mi] * 6]);
    for (int i = 0; i < 6; ++i) msl += metric_product3(m, ev[i]);
  }
  msl = msl / 6;
  double x = sz / kEquilateralTet;
  return cbrt_cr(x * x) / msl;
}

// ------------------------------------------------------------ 2D
// Per-vertex data of a 2D mesh: xh = (x_hi, y_hi, 0, max |hi|),
// xl = (x_lo, y_lo, 0, 0), ma = (xx, yy, yx, S0), mb = (0, 0, 0, sqrt(det M)).

// q = v^T M v for a 2D metric with A = |v|^T |M| |v| and S1 = 1^T |M| |v|
__device__ __forceinline__ float mprod2(float4 ma, const float v[2], float& A, float& S1) {
  float xx = ma.x, yy = ma.y, yx = ma.z;
  float y0 = __fmaf_rn(yx, v[1], __fmul_rn(xx, v[0]));
  float y1 = __fmaf_rn(yy, v[1], __fmul_rn(yx, v[0]));
  float q = __fmaf_rn(v[1], y1, __fmul_rn(v[0], y0));
  float a0 = fabsf(v[0]), a1 = fabsf(v[1]);
  float w0 = __fmaf_rn(fabsf(yx), a1, __fmul_rn(fabsf(xx), a0));
  float w1 = __fmaf_rn(fabsf(yy), a1, __fmul_rn(fabsf(yx), a0));
  S1 = __fadd_rn(w0, w1);
  A = __fmaf_rn(a1, w1, __fmul_rn(a0, w0));
  return q;
}
// error of a 2D v^T M v: at most 4 roundings per term in either evaluation
// plus the metric's conversion, and the input perturbation
__device__ __forceinline__ float mprod2_err(float A, float S1, float S0, float e) {
  float pert = __fmaf_rn(e, __fmaf_rn(2.0f, S1, __fmul_rn(e, S0)), 0.0f);
  return __fmaf_rn(5.1f * kU, A, __fmaf_rn(pert, 1.0f + kU, kTiny));
}
__device__ __forceinline__ float sdiff2(float4 h1, float4 l1, float4 h0, float4 l0, float v[2]) {
  v[0] = __fadd_rn(__fsub_rn(h1.x, h0.x), __fsub_rn(l1.x, l0.x));
  v[1] = __fadd_rn(__fsub_rn(h1.y, h0.y), __fsub_rn(l1.y, l0.y));
  float n = fmaxf(fabsf(v[0]), fabsf(v[1]));
  return __fmaf_rn(n, kC2, __fmaf_rn(__fadd_rn(h1.w, h0.w), 0x1p-44f, kTiny));
}

// the logarithmic-mean enclosure shared by both dimensions (see
// edge_len_bounds)
__device__ __forceinline__ FIv log_mean_bounds(const float l_lo[2], const float l_hi[2]) {
  float m[2];
  for (int c = 0; c < 2; ++c) {
    float x = c ? l_hi[0] : l_lo[0], y = c ? l_hi[1] : l_lo[1];
    float r = __fdiv_rn(x, y);
    float lm;
    if (r > 1.01f || r < 0.99f) {
      lm = __fdiv_rn(__fsub_rn(x, y), logf(r));
      lm = c ? __fmul_ru(lm, 1.0f + 0x1p-15f) : __fmul_rd(lm, 1.0f - 0x1p-15f);
    } else {
      lm = c ? __fmul_ru(__fmul_ru(__fadd_ru(x, y), 0.5f), 1.0f + 0x1p-20f)
             : __fmul_rd(__fsqrt_rd(__fmul_rd(x, y)), 1.0f - 0x1p-20f);
    }
    m[c] = lm;
  }
  float mx = fmaxf(l_hi[0], l_hi[1]);
  float d = __fmaf_ru(mx, 300.0f * 0x1p-50f, 0x1p-50f);
  FIv r = {__fmul_rd(m[0], 1.0f - d), __fmul_ru(m[1], 1.0f + d)};
  if (!finite_iv(r) || !(r.lo > 0.0f)) return widen_all();
  return r;
}

// Interval of the double 2D metric edge length (edge_length2)
__device__ __forceinline__ bool edge_q_bounds2(const ScreenView& s, LO a, LO b, float lo[2],
                                               float hi[2]) {
  float v[2];
  float e = sdiff2(s.xh[b], s.xl[b], s.xh[a], s.xl[a], v);
  LO vs[2] = {a, b};
  bool ok = true;
  for (int k = 0; k < 2; ++k) {
    float4 ma = s.ma[vs[k]];
    float A, S1;
    float q = mprod2(ma, v, A, S1);
    float qe = __fmul_rn(mprod2_err(A, S1, ma.w, e), kInflate);
    lo[k] = __fsub_rd(q, qe);
    hi[k] = __fadd_ru(q, qe);
    ok = ok && lo[k] > 0.0f && hi[k] <= FLT_MAX;
  }
  return ok;
}
__device__ __forceinline__ FIv edge_len_bounds2(const ScreenView& s, LO a, LO b) {
  float lo[2], hi[2];
  if (!edge_q_bounds2(s, a, b, lo, hi)) return widen_all();
  return len_from_q(lo, hi);
}

__device__ __forceinline__ int maxdet_vertex3(const ScreenView& s, const LO vv[3]) {
  int best = 0;
  long long bk = s.dkey[vv[0]];
  for (int i = 1; i < 3; ++i) {
    long long k = s.dkey[vv[i]];
    if (k > bk) {
      best = i;
      bk = k;
    }
  }
  return best;
}

constexpr float kInvEqTri = 2.3094010767585030f;  // float(1 / 0.4330127018922193)
constexpr float kInvEqTriUp = 2.3094013f;         // above 1 / 0.4330127018922193
constexpr float kThird = 1.0f / 3.0f;
constexpr float kThirdUp = 0.33333337f;

// Interval of the double triangle quality (tri_quality on the maxdet metric):
// x / msl with x = area * sqrt(det M) / s_eq, msl the mean v^T M v of the
// three edges; a negative size is returned as the size.
__device__ __forceinline__ FIv tri_quality_bounds_of(const float4 h[3], const float4 l[3],
                                                     float4 ma, float4 mb) {
  float sd = mb.w;
  float ev[3][2], ee[3];
  ee[0] = sdiff2(h[1], l[1], h[0], l[0], ev[0]);  // b0
  ee[1] = sdiff2(h[2], l[2], h[1], l[1], ev[1]);
  ee[2] = sdiff2(h[2], l[2], h[0], l[0], ev[2]);  // b1 (the third edge is -b1)
  const float* b0 = ev[0];
  const float* b1 = ev[2];
  float e0 = ee[0], e1 = ee[2];
  // T = b0 x b1 (rs = T / 2 is exact in both evaluations)
  float T = __fmaf_rn(b0[0], b1[1], -__fmul_rn(b0[1], b1[0]));
  float P = __fmaf_rn(fabsf(b0[0]), fabsf(b1[1]), __fmul_rn(fabsf(b0[1]), fabsf(b1[0])));
  float pert = __fmaf_rn(e0, __fadd_rn(fabsf(b1[0]), fabsf(b1[1])),
                         __fmaf_rn(e1, __fadd_rn(fabsf(b0[0]), fabsf(b0[1])),
                                   __fmul_rn(2.0f, __fmul_rn(e0, e1))));
  float eT = __fmaf_rn(3.1f * kU, P, __fadd_rn(pert, kTiny));
  float rs = __fmul_rn(T, 0.5f);
  float ers = __fmul_rn(eT, 0.5f);
  float sv = __fmul_rn(rs, sd);
  float es = __fmaf_rn(fabsf(sv), kC2, __fmul_rn(__fmul_rn(ers, fabsf(sd)), 1.0f + 0x1p-20f));
  es = __fmul_rn(es, kInflate);
  if (!(fabsf(sv) <= FLT_MAX) || !(es <= FLT_MAX)) return widen_all();
  if (__fadd_ru(sv, es) < 0.0f) return {__fsub_rd(sv, es), __fadd_ru(sv, es)};
  float s_lo = __fsub_rd(sv, es);
  float msum = 0.0f, emsum = 0.0f, asum = 0.0f;
  for (int i = 0; i < 3; ++i) {
    float A, S1;
    float q = mprod2(ma, ev[i], A, S1);
    msum = __fadd_rn(msum, q);
    asum = __fadd_rn(asum, A);
    emsum = __fadd_rn(emsum, mprod2_err(A, S1, ma.w, ee[i]));
  }
  float msl = __fmul_rn(msum, kThird);
  float emsl = __fmaf_rn(fabsf(msl), kC2, __fmul_rn(__fmaf_rn(2.1f * kU, asum, emsum), kThirdUp));
  emsl = __fmul_rn(emsl, kInflate);
  float msl_lo = __fsub_rd(msl, emsl), msl_hi = __fadd_ru(msl, emsl);
  if (!(msl_lo > 1e-30f) || !(msl_hi < 1e30f)) return widen_all();
  if (s_lo < 0.0f) return {s_lo, INFINITY};
  float x = __fmul_rn(sv, kInvEqTri);
  float ex = __fmaf_rn(fabsf(x), kC2, __fmul_rn(es, kInvEqTriUp));
  ex = __fmul_rn(ex, kInflate);
  float x_lo = fmaxf(__fsub_rd(x, ex), 0.0f), x_hi = __fadd_ru(x, ex);
  if (!(x_hi < 1e30f)) return widen_all();
  FIv q = {__fmul_rd(__fdividef(x_lo, msl_hi), 1.0f - 0x1p-21f),
           __fmul_ru(__fdividef(x_hi, msl_lo), 1.0f + 0x1p-21f)};
  if (!finite_iv(q)) return widen_all();
  return q;
}

__device__ __forceinline__ FIv tri_quality_bounds(const ScreenView& s, const LO vv[3]) {
  int mi = maxdet_vertex3(s, vv);
  float4 h[3], l[3];
  for (int i = 0; i < 3; ++i) {
    h[i] = s.xh[vv[i]];
    l[i] = s.xl[vv[i]];
  }
  return tri_quality_bounds_of(h, l, s.ma[vv[mi]], s.mb[vv[mi]]);
}

// The double triangle quality with sqrt(det M) and the maxdet choice taken
// from the per-vertex data: the operations of tri_quality on the maxdet
// vertex metric.
__device__ __forceinline__ double tri_quality_exact(const ScreenView& s, View<const double> c,
                                                    View<const double> mt, const LO vv[3]) {
  int mi = maxdet_vertex3(s, vv);
  double p[3][2];
  for (int i = 0; i < 3; ++i) {
    p[i][0] = c[vv[i] * 2];
    p[i][1] = c[vv[i] * 2 + 1];
  }
  double b00 = p[1][0] - p[0][0], b01 = p[1][1] - p[0][1];
  double b10 = p[2][0] - p[0][0], b11 = p[2][1] - p[0][1];
  double rs = (b00 * b11 - b01 * b10) / 2.0;
  double sz = rs * s.sdet[vv[mi]];
  if (sz < 0) return sz;
  double ev[3][2] = {{b00, b01}, {p[2][0] - p[1][0], p[2][1] - p[1][1]}, {-b10, -b11}};
  double msl = 0;
  if (s.mc == 1) {
    double mi_ = mt[vv[mi]];
    for (int i = 0; i < 3; ++i) msl += iso_product2(mi_, ev[i][0], ev[i][1]);
    msl = msl / 3;
    double x = sz / kEquilateralTri;
    return x / msl;
  }
  const double* m = &mt[vv[mi] * 3];
  for (int i = 0; i < 3; ++i) {
    double a0 = m[0] * ev[i][0], a1 = m[2] * ev[i][0];
    a0 = a0 + m[2] * ev[i][1];
    a1 = a1 + m[1] * ev[i][1];
    double d = ev[i][0] * a0;
    d = d + ev[i][1] * a1;
    msl += d;
  }
  msl = msl / 3;
  double x = sz / kEquilateralTri;
  return x / msl;
}

// dimension dispatch
__device__ __forceinline__ FIv elem_quality_bounds(int dim, const ScreenView& s, const LO* vv) {
  return dim == 3 ? tet_quality_bounds(s, vv) : tri_quality_bounds(s, vv);
}
__device__ __forceinline__ double elem_quality_exact(int dim, const ScreenView& s,
                                                     View<const double> c, View<const double> mt,
                                                     const LO* vv) {
  return dim == 3 ? tet_quality_exact(s, c, mt, vv) : tri_quality_exact(s, c, mt, vv);
}
__device__ __forceinline__ FIv edge_len_bounds_d(int dim, const ScreenView& s, LO a, LO b) {
  return dim == 3 ? edge_len_bounds(s, a, b) : edge_len_bounds2(s, a, b);
}
__device__ __forceinline__ bool edge_q_bounds_d(int dim, const ScreenView& s, LO a, LO b,
                                                float lo[2], float hi[2]) {
  return dim == 3 ? edge_q_bounds3(s, a, b, lo, hi) : edge_q_bounds2(s, a, b, lo, hi);
}

// edge_q_bounds3 / edge_q_bounds2 from the two ends' records (coordinate
// pairs and metric records, end a first): the same operations
template <int D>
__device__ __forceinline__ bool edge_q_bounds_rec(float4 ha, float4 la, float4 maa, float4 mba,
                                                  float4 hb, float4 lb, float4 mab, float4 mbb,
                                                  float lo[2], float hi[2]) {
  bool ok = true;
  if constexpr (D == 3) {
    float v[3];
    float e = sdiff3(hb, lb, ha, la, v);  // p1 - p0 with p0 = a
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float4 ma = k == 0 ? maa : mab, mb = k == 0 ? mba : mbb;
      float A, S1;
      float q = mprod(ma, mb, v, A, S1);
      float qe = __fmul_rn(mprod_err(A, S1, mb.z, e), kInflate);
      lo[k] = __fsub_rd(q, qe);
      hi[k] = __fadd_ru(q, qe);
      ok = ok && lo[k] > 0.0f && hi[k] <= FLT_MAX;
    }
  } else {
    float v[2];
    float e = sdiff2(hb, lb, ha, la, v);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float4 ma = k == 0 ? maa : mab;
      float A, S1;
      float q = mprod2(ma, v, A, S1);
      float qe = __fmul_rn(mprod2_err(A, S1, ma.w, e), kInflate);
      lo[k] = __fsub_rd(q, qe);
      hi[k] = __fadd_ru(q, qe);
      ok = ok && lo[k] > 0.0f && hi[k] <= FLT_MAX;
    }
  }
  return ok;
}

// builds the per-vertex screening data of a mesh of dimension dim
VertScreen build_vert_screen(const Arr<double>& coords, const Arr<double>& metric, LO nverts,
                             int dim = 3);
// the mesh's screening data, built on first use and kept with the mesh
struct Mesh;
const VertScreen& mesh_screen(Mesh& m);

}  // namespace ohg
