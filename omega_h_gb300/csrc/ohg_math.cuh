// Device (and host) math for the adapt pass: alignment codes and simplex
// templates (src/Omega_h_align.hpp, src/Omega_h_simplex.hpp), metric edge
// length (src/Omega_h_shape.hpp:112-134), metric mean-ratio quality
// (src/Omega_h_quality.hpp:8-36), maxdet metric (src/Omega_h_metric.hpp:170-182)
// and the log-Euclidean metric average built on the closed-form 3x3
// symmetric eigensolver (src/Omega_h_eigen.hpp:21-319,474-488).
//
// Every expression keeps the reference's association order and the library
// is compiled with -fmad=false, so +,-,*,/,sqrt round exactly as the
// reference's host build does.  cbrt, log, exp, acos and cos are correctly
// rounded (ohg_libm.cuh), so the results do not depend on a math library's
// last ulp.
#pragma once
#include <cstdint>

#include "ohg_libm.cuh"

#ifndef OHG_HD
#define OHG_HD __host__ __device__ __forceinline__
#endif

namespace ohg {

typedef std::int8_t I8i;

// ------------------------------------------------------------ alignment
OHG_HD bool code_is_flipped(I8i c) { return c & 1; }
OHG_HD int code_rotation(I8i c) { return (c >> 1) & 3; }
OHG_HD int code_which_down(I8i c) { return c >> 3; }
OHG_HD I8i make_code(bool f, int rot, int wd) { return I8i((wd << 3) | (rot << 1) | int(f)); }
OHG_HD int rotate_index(int n, int i, int r) { return (i + r) % n; }
OHG_HD int invert_rotation(int n, int r) { return (n - r) % n; }
OHG_HD int rotation_to_first(int n, int f) { return invert_rotation(n, f); }
OHG_HD int align_index(int n, int idim, int i, I8i c) {
  int r = rotate_index(n, i, code_rotation(c));
  if (!code_is_flipped(c)) return r;
  if (idim == 0) return r == 0 ? 0 : (1 + (n - 2 - (r - 1)));
  return n - 1 - r;
}
OHG_HD I8i invert_alignment(int n, I8i c) {
  return code_is_flipped(c) ? c : make_code(false, invert_rotation(n, code_rotation(c)), 0);
}

// ------------------------------------------------------------ templates
// simplex_down_template: vertex of boundary entity wb (dim bd) of a simplex
// of dim ed, as a simplex-local vertex index
OHG_HD int down_template(int ed, int bd, int wb, int wv) {
  if (bd == 0) return wb;
  if (ed == 3 && bd == 2) {
    // faces {0,2,1},{0,1,3},{1,2,3},{2,0,3}
    const int t = (0 << 0) | (2 << 2) | (1 << 4) | (0 << 6) | (1 << 8) | (3 << 10) |
                  (1 << 12) | (2 << 14) | (3 << 16) | (2 << 18) | (0 << 20) | (3 << 22);
    return (t >> (2 * (wb * 3 + wv))) & 3;
  }
  if (ed == 3 && bd == 1) {
    // edges {0,1},{1,2},{2,0},{0,3},{1,3},{2,3}
    const int t = (0 << 0) | (1 << 2) | (1 << 4) | (2 << 6) | (2 << 8) | (0 << 10) |
                  (0 << 12) | (3 << 14) | (1 << 16) | (3 << 18) | (2 << 20) | (3 << 22);
    return (t >> (2 * (wb * 2 + wv))) & 3;
  }
  // ed == 2, bd == 1: {0,1},{1,2},{2,0}
  return (wb + wv) % 3;
}
OHG_HD int opposite_template(int ed, int bd, int wb) {
  if (ed == 3 && bd == 0) return (0x1e >> (2 * wb)) & 3;    // {2,3,1,0}
  if (ed == 3 && bd == 1) return (8989 >> (3 * wb)) & 7;    // {5,3,4,1,2,0}
  if (ed == 3 && bd == 2) return (0x4b >> (2 * wb)) & 3;  // {3,2,0,1}
  if (ed == 2 && bd == 0) return (wb + 1) % 3;            // {1,2,0}
  if (ed == 2 && bd == 1) return (wb + 2) % 3;            // {2,0,1}
  return 1 - wb;
}
struct UpTemplate {
  int up, which_down;
  bool is_flipped;
};
// simplex_up_template(ed, bd, wb, 0): first upward entity of dim bd+1
OHG_HD UpTemplate up_template0(int ed, int bd, int wb) {
  if (ed == 3 && bd == 0) {
    const int up[4] = {0, 1, 2, 5};
    const int wd[4] = {0, 0, 0, 1};
    return {up[wb], wd[wb], false};
  }
  if (ed == 3 && bd == 1) {
    const int up[6] = {0, 0, 0, 1, 2, 3};
    const int wd[6] = {2, 1, 0, 2, 2, 2};
    return {up[wb], wd[wb], true};
  }
  // ed == 2, bd == 0
  return {wb, 0, false};
}

// ------------------------------------------------------------ math
struct V3 {
  double x[3];
};
struct M3 {
  V3 c[3];  // columns
};
OHG_HD V3 sub3(V3 a, V3 b) { return {{a.x[0] - b.x[0], a.x[1] - b.x[1], a.x[2] - b.x[2]}}; }
OHG_HD double dot3(V3 a, V3 b) {
  double o = a.x[0] * b.x[0];
  o = o + (a.x[1] * b.x[1]);
  o = o + (a.x[2] * b.x[2]);
  return o;
}
OHG_HD V3 cross3(V3 a, V3 b) {
  return {{a.x[1] * b.x[2] - a.x[2] * b.x[1], a.x[2] * b.x[0] - a.x[0] * b.x[2],
           a.x[0] * b.x[1] - a.x[1] * b.x[0]}};
}
OHG_HD V3 mv3(const M3& a, V3 b) {
  V3 c;
  for (int i = 0; i < 3; ++i) c.x[i] = a.c[0].x[i] * b.x[0];
  for (int j = 1; j < 3; ++j)
    for (int i = 0; i < 3; ++i) c.x[i] = c.x[i] + a.c[j].x[i] * b.x[j];
  return c;
}
OHG_HD M3 mm3(const M3& a, const M3& b) {
  M3 c;
  for (int j = 0; j < 3; ++j) c.c[j] = mv3(a, b.c[j]);
  return c;
}
OHG_HD M3 tr3(const M3& a) {
  M3 b;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) b.c[i].x[j] = a.c[j].x[i];
  return b;
}
OHG_HD double det3(const M3& m) {
  double a = m.c[0].x[0], b = m.c[1].x[0], c = m.c[2].x[0];
  double d = m.c[0].x[1], e = m.c[1].x[1], f = m.c[2].x[1];
  double g = m.c[0].x[2], h = m.c[1].x[2], i = m.c[2].x[2];
  return (a * e * i) + (b * f * g) + (c * d * h) - (c * e * g) - (b * d * i) - (a * f * h);
}
// packed (xx, yy, zz, yx, zy, zx)
OHG_HD M3 symm3(const double* v) {
  M3 s;
  s.c[0].x[0] = v[0];
  s.c[1].x[1] = v[1];
  s.c[2].x[2] = v[2];
  s.c[1].x[0] = v[3];
  s.c[2].x[1] = v[4];
  s.c[2].x[0] = v[5];
  s.c[0].x[1] = v[3];
  s.c[1].x[2] = v[4];
  s.c[0].x[2] = v[5];
  return s;
}
OHG_HD void unsymm3(const M3& s, double* v) {
  v[0] = s.c[0].x[0];
  v[1] = s.c[1].x[1];
  v[2] = s.c[2].x[2];
  v[3] = s.c[1].x[0];
  v[4] = s.c[2].x[1];
  v[5] = s.c[2].x[0];
}
OHG_HD double metric_product3(const M3& m, V3 v) { return dot3(v, mv3(m, v)); }

OHG_HD double aniso_length(double la, double lb) {
  if (fabs(la - lb) > 1e-3) return (la - lb) / (log_cr(la / lb));
  return (la + lb) / 2.;
}
OHG_HD double edge_length3(const double* p0, const double* p1, const double* m0,
                           const double* m1) {
  V3 v = {{p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]}};
  double la = sqrt(metric_product3(symm3(m0), v));
  double lb = sqrt(metric_product3(symm3(m1), v));
  return aniso_length(la, lb);
}
OHG_HD double edge_length2(const double* p0, const double* p1, const double* m0,
                           const double* m1) {
  double v0 = p1[0] - p0[0], v1 = p1[1] - p0[1];
  // m*v with m = [[m0 m2],[m2 m1]] accumulated column by column
  double a0 = m0[0] * v0, a1 = m0[2] * v0;
  a0 = a0 + m0[2] * v1;
  a1 = a1 + m0[1] * v1;
  double b0 = m1[0] * v0, b1 = m1[2] * v0;
  b0 = b0 + m1[2] * v1;
  b1 = b1 + m1[1] * v1;
  double da = v0 * a0;
  da = da + v1 * a1;
  double db = v0 * b0;
  db = db + v1 * b1;
  return aniso_length(sqrt(da), sqrt(db));
}

constexpr double kEquilateralTet = 0.1178511301977579;
constexpr double kEquilateralTri = 0.4330127018922193;

OHG_HD double tet_quality(const V3 p[4], const M3& m) {
  V3 b0 = sub3(p[1], p[0]), b1 = sub3(p[2], p[0]), b2 = sub3(p[3], p[0]);
  double rs = dot3(cross3(b0, b1), b2) / 6.0;
  double s = rs * sqrt(det3(m));
  if (s < 0) return s;
  V3 nb1 = {{-b1.x[0], -b1.x[1], -b1.x[2]}};
  V3 ev[6] = {b0, sub3(p[2], p[1]), nb1, b2, sub3(p[3], p[1]), sub3(p[3], p[2])};
  double msl = 0;
  for (int i = 0; i < 6; ++i) msl += metric_product3(m, ev[i]);
  msl = msl / 6;
  double x = s / kEquilateralTet;
  return cbrt_cr(x * x) / msl;
}
// maxdet over n metrics, first maximum wins ties
OHG_HD int maxdet_index3(const M3* ms, int n) {
  int best = 0;
  double maxdet = det3(ms[0]);
  for (int i = 1; i < n; ++i) {
    double d = det3(ms[i]);
    if (d > maxdet) {
      best = i;
      maxdet = d;
    }
  }
  return best;
}

// 2D triangle quality with a 2x2 metric packed (xx, yy, yx)
OHG_HD double det2p(const double* m) { return m[0] * m[1] - m[2] * m[2]; }
OHG_HD double tri_quality(const double p[3][2], const double* m) {
  double b00 = p[1][0] - p[0][0], b01 = p[1][1] - p[0][1];
  double b10 = p[2][0] - p[0][0], b11 = p[2][1] - p[0][1];
  double rs = (b00 * b11 - b01 * b10) / 2.0;
  double s = rs * sqrt(det2p(m));
  if (s < 0) return s;
  double ev[3][2] = {{b00, b01}, {p[2][0] - p[1][0], p[2][1] - p[1][1]}, {-b10, -b11}};
  double msl = 0;
  for (int i = 0; i < 3; ++i) {
    double a0 = m[0] * ev[i][0], a1 = m[2] * ev[i][0];
    a0 = a0 + m[2] * ev[i][1];
    a1 = a1 + m[1] * ev[i][1];
    double d = ev[i][0] * a0;
    d = d + ev[i][1] * a1;
    msl += d;
  }
  msl = msl / 3;
  double x = s / kEquilateralTri;
  return x / msl;
}

// ------------------------------------------------------------ isotropic metrics
// A metric of one component m per vertex (the reference's Tensor<1>): the
// product v^T (m v) scales each component first and sums left to right, the
// size factor is power<dim, 2>(m) (sqrt(m (m m)) in 3D, m in 2D), maxdet
// compares m itself, and the log-Euclidean mean of 1x1 tensors is
// exp(mean of logs), with the eigensolver's zero path (|x| <= 1e-10) kept
// (src/Omega_h_metric.hpp:10-23,126-150, src/Omega_h_shape.hpp:400-403,
// src/Omega_h_eigen.hpp:288-321).
OHG_HD double iso_product3(double m, V3 v) {
  double o = v.x[0] * (v.x[0] * m);
  o = o + v.x[1] * (v.x[1] * m);
  o = o + v.x[2] * (v.x[2] * m);
  return o;
}
OHG_HD double iso_product2(double m, double v0, double v1) {
  double o = v0 * (v0 * m);
  o = o + v1 * (v1 * m);
  return o;
}
OHG_HD double edge_length_iso3(const double* p0, const double* p1, double m0, double m1) {
  V3 v = {{p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]}};
  return aniso_length(sqrt(iso_product3(m0, v)), sqrt(iso_product3(m1, v)));
}
OHG_HD double edge_length_iso2(const double* p0, const double* p1, double m0, double m1) {
  double v0 = p1[0] - p0[0], v1 = p1[1] - p0[1];
  return aniso_length(sqrt(iso_product2(m0, v0, v1)), sqrt(iso_product2(m1, v0, v1)));
}
OHG_HD double iso_size_factor(int dim, double m) { return dim == 3 ? sqrt(m * (m * m)) : m; }
OHG_HD double tet_quality_iso(const V3 p[4], double m) {
  V3 b0 = sub3(p[1], p[0]), b1 = sub3(p[2], p[0]), b2 = sub3(p[3], p[0]);
  double rs = dot3(cross3(b0, b1), b2) / 6.0;
  double s = rs * iso_size_factor(3, m);
  if (s < 0) return s;
  V3 nb1 = {{-b1.x[0], -b1.x[1], -b1.x[2]}};
  V3 ev[6] = {b0, sub3(p[2], p[1]), nb1, b2, sub3(p[3], p[1]), sub3(p[3], p[2])};
  double msl = 0;
  for (int i = 0; i < 6; ++i) msl += iso_product3(m, ev[i]);
  msl = msl / 6;
  double x = s / kEquilateralTet;
  return cbrt_cr(x * x) / msl;
}
OHG_HD double tri_quality_iso(const double p[3][2], double m) {
  double b00 = p[1][0] - p[0][0], b01 = p[1][1] - p[0][1];
  double b10 = p[2][0] - p[0][0], b11 = p[2][1] - p[0][1];
  double rs = (b00 * b11 - b01 * b10) / 2.0;
  double s = rs * m;
  if (s < 0) return s;
  double ev[3][2] = {{b00, b01}, {p[2][0] - p[1][0], p[2][1] - p[1][1]}, {-b10, -b11}};
  double msl = 0;
  for (int i = 0; i < 3; ++i) msl += iso_product2(m, ev[i][0], ev[i][1]);
  msl = msl / 3;
  double x = s / kEquilateralTri;
  return x / msl;
}
OHG_HD double iso_log(double m) { return fabs(m) <= 1e-10 ? log_cr(0.0) : log_cr(m); }
OHG_HD double average_metric_iso(double a, double b) {
  double am = 0.0 + iso_log(a);
  am = am + iso_log(b);
  am = am / 2;
  return fabs(am) <= 1e-10 ? exp_cr(0.0) : exp_cr(am);
}

// the determinant the maxdet choice compares: the tensor's, or the scalar
OHG_HD double metric_det(int dim, int mc, const double* m) {
  return mc == 1 ? m[0] : dim == 3 ? det3(symm3(m)) : det2p(m);
}
// FP64 element quality with the maxdet metric among per-vertex metrics
// ms[0..dim] (mc components each; 1: isotropic); pts holds dim + 1 points
OHG_HD double elem_quality_ms(int dim, int mc, const double* pts, const double* const* ms) {
  int best = 0;
  double bd = metric_det(dim, mc, ms[0]);
  for (int i = 1; i <= dim; ++i) {
    double d = metric_det(dim, mc, ms[i]);
    if (d > bd) {
      best = i;
      bd = d;
    }
  }
  if (dim == 3) {
    V3 p[4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 3; ++j) p[i].x[j] = pts[i * 3 + j];
    return mc == 1 ? tet_quality_iso(p, ms[best][0]) : tet_quality(p, symm3(ms[best]));
  }
  double p[3][2];
  for (int i = 0; i < 3; ++i) {
    p[i][0] = pts[i * 2];
    p[i][1] = pts[i * 2 + 1];
  }
  return mc == 1 ? tri_quality_iso(p, ms[best][0]) : tri_quality(p, ms[best]);
}

// ------------------------------------------------------------ eigen (3x3)
OHG_HD double sq(double x) { return x * x; }
OHG_HD double cube(double x) { return x * (x * x); }
OHG_HD double max2d(double a, double b) { return (a < b) ? b : a; }
OHG_HD double min2d(double a, double b) { return (b < a) ? b : a; }

struct Eig3 {
  M3 q;
  V3 l;
  bool ok;
};
OHG_HD M3 ident3() {
  M3 a;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) a.c[j].x[i] = (i == j) ? 1.0 : 0.0;
  return a;
}
OHG_HD double norm3(V3 a) { return sqrt(dot3(a, a)); }
OHG_HD V3 single_eigvec3(const M3& m, double l, bool* ok) {
  M3 s = m;
  for (int i = 0; i < 3; ++i) s.c[i].x[i] -= l;
  s = tr3(s);
  V3 v = cross3(s.c[0], s.c[1]);
  double vn = norm3(v);
  V3 c = cross3(s.c[1], s.c[2]);
  double cn = norm3(c);
  if (cn > vn) {
    v = c;
    vn = cn;
  }
  c = cross3(s.c[0], s.c[2]);
  cn = norm3(c);
  if (cn > vn) {
    v = c;
    vn = cn;
  }
  if (!(vn > 1e-10)) *ok = false;
  return {{v.x[0] / vn, v.x[1] / vn, v.x[2] / vn}};
}
// find_polynomial_roots of x^3 + a_2 x^2 + a_1 x + a_0 with real roots
// (src/Omega_h_eigen.hpp:21-85): Cardano's formula when the discriminant D
// is >= 0, else the trigonometric form; roots closer than eps are merged,
// a pair first (into slots 1 and 2, averaged), then all three.  Returns the
// number of distinct roots; mult[] holds the multiplicities.
OHG_HD int cubic_roots(double a_0, double a_1, double a_2, double eps, double rt[3], int mult[3]) {
  const double PI = 3.14159265358979323;
  double p = (3. * a_1 - sq(a_2)) / 3.;
  double q = (9. * a_1 * a_2 - 27. * a_0 - 2. * cube(a_2)) / 27.;
  double Q = p / 3.;
  double R = q / 2.;
  double D = cube(Q) + sq(R);
  double shift = -a_2 / 3.;
  if (D >= 0.0) {
    double S = cbrt_cr(R + sqrt(D));
    double T = cbrt_cr(R - sqrt(D));
    double B = S + T;
    rt[0] = shift + B;
    rt[1] = rt[2] = shift - (1. / 2.) * B;
  } else {
    double ct = R / sqrt(-cube(Q));
    double theta = acos_cr(min2d(max2d(ct, -1.0), 1.0));
    double radius = 2. * sqrt(-Q);
    rt[0] = radius * cos_cr((theta) / 3.) + shift;
    rt[1] = radius * cos_cr((theta + 2. * PI) / 3.) + shift;
    rt[2] = radius * cos_cr((theta - 2. * PI) / 3.) + shift;
  }
  mult[0] = mult[1] = mult[2] = 1;
  if (fabs(rt[0] - rt[1]) < eps) {
    double t = rt[0];
    rt[0] = rt[2];
    rt[2] = t;
  } else if (fabs(rt[0] - rt[2]) < eps) {
    double t = rt[0];
    rt[0] = rt[1];
    rt[1] = t;
  } else if (!(fabs(rt[1] - rt[2]) < eps)) {
    return 3;
  }
  rt[1] = (rt[1] + rt[2]) / 2;
  mult[1] = 2;
  if (fabs(rt[0] - rt[1]) < eps) {
    rt[0] = (1. / 3.) * rt[0] + (2. / 3.) * rt[1];
    mult[0] = 3;
    return 1;
  }
  return 2;
}

OHG_HD Eig3 eigen3(M3 m) {
  Eig3 r;
  r.ok = true;
  double nm = 0.0;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) nm = max2d(nm, fabs(m.c[j].x[i]));
  if (nm <= 1e-10) {
    r.q = ident3();
    r.l = {{0, 0, 0}};
    return r;
  }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) m.c[j].x[i] = m.c[j].x[i] / nm;
  double tA = m.c[0].x[0];
  tA += m.c[1].x[1];
  tA += m.c[2].x[2];
  M3 m2 = mm3(m, m);
  double t2 = m2.c[0].x[0];
  t2 += m2.c[1].x[1];
  t2 += m2.c[2].x[2];
  double a_2 = -tA;
  double a_1 = (1. / 2.) * ((tA * tA) - t2);
  double a_0 = -det3(m);
  double rt[3];
  int mult[3];
  int nroots = cubic_roots(a_0, a_1, a_2, 5e-5, rt, mult);
  if (nroots == 3) {
    for (int i = 0; i < 3; ++i) {
      r.q.c[i] = single_eigvec3(m, rt[i], &r.ok);
      r.l.x[i] = rt[i];
    }
  } else if (nroots == 2) {
    r.q.c[0] = single_eigvec3(m, rt[0], &r.ok);
    r.l.x[0] = rt[0];
    // null space of (m - l I) is 2D: complete the unit row-space vector
    M3 s = m;
    for (int i = 0; i < 3; ++i) s.c[i].x[i] -= rt[1];
    M3 ta = tr3(s);
    int best = 0;
    double bn = norm3(ta.c[0]);
    for (int i = 1; i < 3; ++i) {
      double rn = norm3(ta.c[i]);
      if (rn > bn) {
        best = i;
        bn = rn;
      }
    }
    if (!(bn > 1e-10)) r.ok = false;
    V3 v = {{ta.c[best].x[0] / bn, ta.c[best].x[1] / bn, ta.c[best].x[2] / bn}};
    // Duff et al., "Building an orthonormal basis, revisited" (JCGT 2017)
    double sign = copysign(1.0, v.x[2]);
    const double a = -1.0 / (sign + v.x[2]);
    const double b = v.x[0] * v.x[1] * a;
    r.q.c[1] = {{1.0 + sign * v.x[0] * v.x[0] * a, sign * b, -sign * v.x[0]}};
    r.q.c[2] = {{b, sign + v.x[1] * v.x[1] * a, -v.x[1]}};
    r.l.x[1] = r.l.x[2] = rt[1];
  } else {
    r.l.x[0] = r.l.x[1] = r.l.x[2] = rt[0];
    r.q = ident3();
  }
  for (int i = 0; i < 3; ++i) r.l.x[i] = r.l.x[i] * nm;
  return r;
}
OHG_HD M3 compose_ortho3(const M3& q, V3 l) {
  M3 d;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) d.c[i].x[j] = 0.0;
  for (int i = 0; i < 3; ++i) d.c[i].x[i] = l.x[i];
  return mm3(mm3(q, d), tr3(q));
}
// log M of a packed metric (linearize_metric, src/Omega_h_metric.hpp:105-125)
// as the full 3x3 matrix, column by column; false if the eigendecomposition
// failed
OHG_HD bool log_metric3(const double* m, double* L9) {
  Eig3 e = eigen3(symm3(m));
  for (int i = 0; i < 3; ++i) e.l.x[i] = log_cr(e.l.x[i]);
  M3 L = compose_ortho3(e.q, e.l);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) L9[j * 3 + i] = L.c[j].x[i];
  return e.ok;
}
// exp(mean of two log metrics) (average_metric, src/Omega_h_metric.hpp:
// 127-150): the sum starts from zero and adds L0, then L1, as the reference
// accumulates it
OHG_HD bool average_log_metrics3(const double* L0, const double* L1, double* out) {
  M3 am;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) am.c[j].x[i] = 0.0;
  for (int k = 0; k < 2; ++k) {
    const double* L = k == 0 ? L0 : L1;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] + L[j * 3 + i];
  }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] / 2;
  Eig3 e = eigen3(am);
  for (int i = 0; i < 3; ++i) e.l.x[i] = exp_cr(e.l.x[i]);
  unsymm3(compose_ortho3(e.q, e.l), out);
  return e.ok;
}
// exp(mean(log M0, log M1)) for two packed metrics
OHG_HD bool average_metric3(const double* m0, const double* m1, double* out) {
  double L0[9], L1[9];
  bool ok0 = log_metric3(m0, L0);
  bool ok1 = log_metric3(m1, L1);
  bool ok2 = average_log_metrics3(L0, L1, out);
  return ok0 && ok1 && ok2;
}

// ------------------------------------------------------------ eigen (2x2)
// The 2x2 symmetric eigendecomposition of src/Omega_h_eigen.hpp (quadratic
// roots, a double root below 5e-5 taken as isotropic) and the 2D
// log-Euclidean metric average, in the reference's operation order.
struct V2 {
  double x[2];
};
struct M2 {
  V2 c[2];  // columns
};
OHG_HD V2 mv2(const M2& a, V2 b) {
  V2 c;
  for (int i = 0; i < 2; ++i) c.x[i] = a.c[0].x[i] * b.x[0];
  for (int i = 0; i < 2; ++i) c.x[i] = c.x[i] + a.c[1].x[i] * b.x[1];
  return c;
}
OHG_HD M2 mm2(const M2& a, const M2& b) {
  M2 c;
  for (int j = 0; j < 2; ++j) c.c[j] = mv2(a, b.c[j]);
  return c;
}
OHG_HD M2 tr2(const M2& a) {
  M2 b;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) b.c[i].x[j] = a.c[j].x[i];
  return b;
}
OHG_HD M2 ident2() {
  M2 a;
  a.c[0].x[0] = 1;
  a.c[0].x[1] = 0;
  a.c[1].x[0] = 0;
  a.c[1].x[1] = 1;
  return a;
}
OHG_HD double det2m(const M2& m) {
  double a = m.c[0].x[0], b = m.c[1].x[0], c = m.c[0].x[1], d = m.c[1].x[1];
  return a * d - b * c;
}
// packed (xx, yy, yx)
OHG_HD M2 symm2(const double* v) {
  M2 s;
  s.c[0].x[0] = v[0];
  s.c[1].x[1] = v[1];
  s.c[1].x[0] = v[2];
  s.c[0].x[1] = s.c[1].x[0];
  return s;
}
struct Eig2 {
  M2 q;
  V2 l;
  bool ok;
};
OHG_HD Eig2 eigen2(M2 m) {
  Eig2 r;
  r.ok = true;
  double nm = 0.0;
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) nm = max2d(nm, fabs(m.c[j].x[i]));
  if (nm <= 1e-10) {
    r.q = ident2();
    r.l.x[0] = r.l.x[1] = 0;
    return r;
  }
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) m.c[j].x[i] = m.c[j].x[i] / nm;
  double tr = m.c[0].x[0];
  tr += m.c[1].x[1];
  double a = -tr;
  double b = det2m(m);
  double disc = sq(a) - 4. * b;
  if (fabs(disc) < 5e-5) {
    double rt = -a / 2.;
    r.l.x[0] = r.l.x[1] = rt;
    r.q = ident2();
  } else {
    if (!(disc > 0.0)) r.ok = false;
    double roots[2] = {(-a + sqrt(disc)) / 2., (-a - sqrt(disc)) / 2.};
    for (int i = 0; i < 2; ++i) {
      M2 s = m;
      for (int k = 0; k < 2; ++k) s.c[k].x[k] = s.c[k].x[k] - roots[i];
      M2 ts = tr2(s);
      int best = 0;
      double bn = sqrt(ts.c[0].x[0] * ts.c[0].x[0] + ts.c[0].x[1] * ts.c[0].x[1]);
      double n1 = sqrt(ts.c[1].x[0] * ts.c[1].x[0] + ts.c[1].x[1] * ts.c[1].x[1]);
      if (n1 > bn) {
        best = 1;
        bn = n1;
      }
      if (!(bn > 1e-10)) r.ok = false;
      double r0 = ts.c[best].x[0] / bn, r1 = ts.c[best].x[1] / bn;
      r.q.c[i].x[0] = -r1;
      r.q.c[i].x[1] = r0;
      r.l.x[i] = roots[i];
    }
  }
  r.l.x[0] = r.l.x[0] * nm;
  r.l.x[1] = r.l.x[1] * nm;
  return r;
}
OHG_HD M2 compose_ortho2(const M2& q, V2 l) {
  M2 d;
  d.c[0].x[1] = d.c[1].x[0] = 0.0;
  d.c[0].x[0] = l.x[0];
  d.c[1].x[1] = l.x[1];
  return mm2(mm2(q, d), tr2(q));
}
// exp(mean(log M0, log M1)) for two packed 2D metrics
OHG_HD bool average_metric2(const double* m0, const double* m1, double* out) {
  M2 am;
  am.c[0].x[0] = am.c[0].x[1] = am.c[1].x[0] = am.c[1].x[1] = 0.0;
  bool ok = true;
  for (int k = 0; k < 2; ++k) {
    Eig2 e = eigen2(symm2(k == 0 ? m0 : m1));
    ok = ok && e.ok;
    for (int i = 0; i < 2; ++i) e.l.x[i] = log_cr(e.l.x[i]);
    M2 L = compose_ortho2(e.q, e.l);
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] + L.c[j].x[i];
  }
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] / 2;
  Eig2 e = eigen2(am);
  ok = ok && e.ok;
  for (int i = 0; i < 2; ++i) e.l.x[i] = exp_cr(e.l.x[i]);
  M2 r = compose_ortho2(e.q, e.l);
  out[0] = r.c[0].x[0];
  out[1] = r.c[1].x[1];
  out[2] = r.c[1].x[0];
  return ok;
}

}  // namespace ohg
