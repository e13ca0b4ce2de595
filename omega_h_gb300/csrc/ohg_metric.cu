// Metric tools: the producers of the vertex metric array that the adapt
// path consumes (src/Omega_h_metric.cpp, src/Omega_h_metric_input.cpp).
// Per-vertex and per-element kernels in FP64, each small dense operation
// (eigendecomposition, inverse, Householder QR, log/exp of an SPD tensor)
// in the reference's operation order, so that the discrete decisions inside
// them (the eigen solver's root merging, the clamps) come out the same:
//   intersect_metrics   Barral's simultaneous reduction and degenerate cases
//   clamp_metrics       eigenvalues clamped to [1/h_max^2, 1/h_min^2]
//   hessian_metrics     Alauzet-Frey: |eigenvalues| d^2 / (2 (d+1)^2 eps)
//   implied_metrics     each element's unit-edge metric, log-averaged to
//                       the vertices and scaled to a typical element size
//   limit_gradation     vertex-star sweeps until no value changes by tol
//   expected_nelems     sum over elements of volume * sqrt(det M) / typical
//                       unit simplex size, summed exactly in fixed point
//   generate_metrics    sources, isotropy, length clamps, smoothing,
//                       gradation and the element-count iteration
#include <cfloat>
#include <cmath>

#include "ohg_math.cuh"
#include "ohg_mesh.cuh"
#include "ohg_metric.cuh"

namespace ohg {

namespace {

constexpr double kEps = 1e-10;  // OMEGA_H_EPSILON

// ------------------------------------------------------------ dense algebra
OHG_HD M3 zero3() {
  M3 a;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) a.c[j].x[i] = 0.0;
  return a;
}
OHG_HD M3 diag3(V3 l) {
  M3 a = zero3();
  for (int i = 0; i < 3; ++i) a.c[i].x[i] = l.x[i];
  return a;
}
OHG_HD M3 scale3(const M3& a, double s) {
  M3 b;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) b.c[j].x[i] = a.c[j].x[i] * s;
  return b;
}
// invert (src/Omega_h_matrix.hpp:344-350): cross products of the columns,
// transposed, over the determinant
OHG_HD M3 inv3(const M3& a) {
  M3 b;
  b.c[0] = cross3(a.c[1], a.c[2]);
  b.c[1] = cross3(a.c[2], a.c[0]);
  b.c[2] = cross3(a.c[0], a.c[1]);
  M3 t = tr3(b);
  double d = det3(a);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) t.c[j].x[i] = t.c[j].x[i] / d;
  return t;
}
OHG_HD M3 log_spd3(const M3& m, bool* ok) {
  Eig3 e = eigen3(m);
  *ok = *ok && e.ok;
  for (int i = 0; i < 3; ++i) e.l.x[i] = log_cr(e.l.x[i]);
  return compose_ortho3(e.q, e.l);
}
OHG_HD M3 exp_spd3(const M3& m, bool* ok) {
  Eig3 e = eigen3(m);
  *ok = *ok && e.ok;
  for (int i = 0; i < 3; ++i) e.l.x[i] = exp_cr(e.l.x[i]);
  return compose_ortho3(e.q, e.l);
}
OHG_HD double max_norm3(const M3& a) {
  double x = 0.0;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) x = max2d(x, fabs(a.c[j].x[i]));
  return x;
}

OHG_HD M2 zero2() {
  M2 a;
  a.c[0].x[0] = a.c[0].x[1] = a.c[1].x[0] = a.c[1].x[1] = 0.0;
  return a;
}
OHG_HD M2 diag2(V2 l) {
  M2 a = zero2();
  a.c[0].x[0] = l.x[0];
  a.c[1].x[1] = l.x[1];
  return a;
}
OHG_HD M2 scale2(const M2& a, double s) {
  M2 b;
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) b.c[j].x[i] = a.c[j].x[i] * s;
  return b;
}
// invert (src/Omega_h_matrix.hpp:336-342)
OHG_HD M2 inv2(const M2& m) {
  double a = m.c[0].x[0], b = m.c[1].x[0], c = m.c[0].x[1], d = m.c[1].x[1];
  double det = a * d - b * c;
  M2 o;
  o.c[0].x[0] = d / det;
  o.c[0].x[1] = -c / det;
  o.c[1].x[0] = -b / det;
  o.c[1].x[1] = a / det;
  return o;
}
OHG_HD M2 log_spd2(const M2& m, bool* ok) {
  Eig2 e = eigen2(m);
  *ok = *ok && e.ok;
  for (int i = 0; i < 2; ++i) e.l.x[i] = log_cr(e.l.x[i]);
  return compose_ortho2(e.q, e.l);
}
OHG_HD M2 exp_spd2(const M2& m, bool* ok) {
  Eig2 e = eigen2(m);
  *ok = *ok && e.ok;
  for (int i = 0; i < 2; ++i) e.l.x[i] = exp_cr(e.l.x[i]);
  return compose_ortho2(e.q, e.l);
}
OHG_HD double max_norm2(const M2& a) {
  double x = 0.0;
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) x = max2d(x, fabs(a.c[j].x[i]));
  return x;
}
OHG_HD void unsymm2(const M2& s, double* v) {
  v[0] = s.c[0].x[0];
  v[1] = s.c[1].x[1];
  v[2] = s.c[1].x[0];
}

// ------------------------------------------------------------ intersection
// Metric intersection (src/Omega_h_metric_intersect.hpp:215-262): Barral's
// simultaneous reduction when the less degenerate metric has no eigenvalue
// below 1e-10, else the degenerate cases of Barral's dissertation, appendix
// A (src/Omega_h_metric_intersect.hpp:25-212): 2D case 5; 3D cases 2
// (both metrics rank 1), 3 (ranks 2 and 1) and 4 (both rank 2).  Products
// are taken in the reference's order, so the discrete choices (orthogonality
// tests, which eigenvector is which) fall the same way.
OHG_HD double dot2(V2 a, V2 b) {
  double o = a.x[0] * b.x[0];
  o = o + (a.x[1] * b.x[1]);
  return o;
}
OHG_HD M2 outer2(V2 a, V2 b) {
  M2 c;
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) c.c[j].x[i] = a.x[i] * b.x[j];
  return c;
}
OHG_HD M3 outer3(V3 a, V3 b) {
  M3 c;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) c.c[j].x[i] = a.x[i] * b.x[j];
  return c;
}
OHG_HD V3 normalize3(V3 v) {
  double n = sqrt(dot3(v, v));
  return {{v.x[0] / n, v.x[1] / n, v.x[2] / n}};
}
// transpose(P^-1) diag(l) P^-1
OHG_HD M3 congruent_diag3(const M3& p, V3 l) {
  M3 pi = inv3(p);
  return mm3(mm3(tr3(pi), diag3(l)), pi);
}

OHG_HD M2 intersect2(M2 m1, M2 m2, bool* ok);

// Two metrics of rank 2 in 3D reduced to the plane of the first one's
// non-degenerate eigenvectors u and v, intersected there and lifted back:
// P (3x2) = [u v]; P (intersect(P^T m1 P, P^T m2 P)) P^T (cases 3.a and 4.a)
OHG_HD M3 intersect_in_plane3(const M3& m1, const M3& m2, V3 u, V3 v, bool* ok) {
  V3 p[2] = {u, v};
  M2 mb[2];
  for (int k = 0; k < 2; ++k) {
    const M3& m = k == 0 ? m1 : m2;
    for (int j = 0; j < 2; ++j) {
      V3 x = mv3(m, p[j]);  // column j of m P
      // column j of P^T (m P): sum over the 3 columns of P^T
      V2 c;
      for (int i = 0; i < 2; ++i) c.x[i] = p[i].x[0] * x.x[0];
      for (int r = 1; r < 3; ++r)
        for (int i = 0; i < 2; ++i) c.x[i] = c.x[i] + p[i].x[r] * x.x[r];
      mb[k].c[j] = c;
    }
  }
  M2 mi = intersect2(mb[0], mb[1], ok);
  // Y (2x3) = mi P^T: column r = mi[0] P^T[r][0] + mi[1] P^T[r][1]
  V2 y[3];
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < 2; ++i)
      y[r].x[i] = mi.c[0].x[i] * p[0].x[r] + mi.c[1].x[i] * p[1].x[r];
  M3 out;
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < 3; ++i) out.c[r].x[i] = p[0].x[i] * y[r].x[0] + p[1].x[i] * y[r].x[1];
  return out;
}

// Barral's case 5: one eigenvalue of each 2D metric below 1e-10
OHG_HD M2 intersect_degen2(const M2& m1, const Eig2& d1, const int* g1, const M2& m2,
                           const Eig2& d2, const int* g2) {
  V2 u1 = {{0, 0}}, v1 = {{0, 0}}, v2 = {{0, 0}};
  double l1 = -1.0, l2 = -1.0;
  for (int i = 0; i < 2; ++i) {
    if (g1[i]) {
      v1 = d1.q.c[i];
    } else {
      u1 = d1.q.c[i];
      l1 = d1.l.x[i];
    }
    if (g2[i]) v2 = d2.q.c[i];
    else l2 = d2.l.x[i];
  }
  if (dot2(v1, v2) < kEps) return scale2(outer2(u1, u1), max2d(l1, l2));  // 5.a
  M2 p;  // 5.b
  p.c[0] = v1;
  p.c[1] = v2;
  M2 pi = inv2(p);
  V2 l;
  l.x[0] = dot2(v1, mv2(m2, v1));
  l.x[1] = dot2(v2, mv2(m1, v2));
  return mm2(mm2(tr2(pi), diag2(l)), pi);
}

// Barral's cases 2-4 in 3D; m1 is the less degenerate metric (n1 <= n2)
OHG_HD M3 intersect_degen3(const M3& m1, const Eig3& d1, const int* g1, int n1, const M3& m2,
                           const Eig3& d2, const int* g2, int n2, bool* ok) {
  const V3 z = {{0, 0, 0}};
  if (n1 == 2 && n2 == 2) {
    V3 u1 = z, u2 = z;
    double l1 = -1.0, l2 = -1.0;
    for (int i = 0; i < 3; ++i) {
      if (!g1[i]) {
        u1 = d1.q.c[i];
        l1 = d1.l.x[i];
      }
      if (!g2[i]) {
        u2 = d2.q.c[i];
        l2 = d2.l.x[i];
      }
    }
    V3 u = cross3(u1, u2);
    if (dot3(u, u) < kEps) return scale3(outer3(u1, u1), max2d(l1, l2));  // 2.a
    u = normalize3(u);  // 2.b
    V3 e1 = cross3(u1, u), e2 = cross3(u2, u);
    M3 p;
    p.c[0] = e1;
    p.c[1] = e2;
    p.c[2] = u;
    V3 l = {{dot3(e1, mv3(m2, e1)), dot3(e2, mv3(m1, e2)), 0.0}};
    return congruent_diag3(p, l);
  }
  if (n1 == 1 && n2 == 2) {
    V3 u1 = z, v1 = z, w1 = z, u2 = z, v2 = z, w2 = z;
    bool found_u1 = false, found_v2 = false;
    for (int i = 0; i < 3; ++i) {
      if (g1[i]) {
        w1 = d1.q.c[i];
      } else if (found_u1) {
        v1 = d1.q.c[i];
      } else {
        u1 = d1.q.c[i];
        found_u1 = true;
      }
      if (!g2[i]) {
        u2 = d2.q.c[i];
      } else if (found_v2) {
        w2 = d2.q.c[i];
      } else {
        v2 = d2.q.c[i];
        found_v2 = true;
      }
    }
    if (dot3(u2, w1) < kEps) return intersect_in_plane3(m1, m2, u1, v1, ok);  // 3.a
    M3 p;  // 3.b
    p.c[0] = v2;
    p.c[1] = w2;
    p.c[2] = w1;
    V3 l = {{dot3(p.c[0], mv3(m1, p.c[0])), dot3(p.c[1], mv3(m1, p.c[1])),
             dot3(p.c[2], mv3(m2, p.c[2]))}};
    return congruent_diag3(p, l);
  }
  if (n1 == 1 && n2 == 1) {
    V3 u1 = z, v1 = z, w1 = z, w2 = z;
    bool found_u1 = false;
    for (int i = 0; i < 3; ++i) {
      if (g1[i]) {
        w1 = d1.q.c[i];
      } else if (found_u1) {
        v1 = d1.q.c[i];
      } else {
        u1 = d1.q.c[i];
        found_u1 = true;
      }
      if (g2[i]) w2 = d2.q.c[i];
    }
    V3 w = cross3(w1, w2);
    if (dot3(w, w) < kEps) return intersect_in_plane3(m1, m2, u1, v1, ok);  // 4.a
    w = normalize3(w);  // 4.b
    M3 p;
    p.c[0] = w1;
    p.c[1] = w2;
    p.c[2] = w;
    V3 l = {{dot3(p.c[0], mv3(m2, p.c[0])), dot3(p.c[1], mv3(m1, p.c[1])),
             max2d(dot3(p.c[2], mv3(m1, p.c[2])), dot3(p.c[2], mv3(m2, p.c[2])))}};
    return congruent_diag3(p, l);
  }
  return m1;
}

OHG_HD M3 intersect3(M3 m1, M3 m2, bool* ok) {
  Eig3 d1 = eigen3(m1), d2 = eigen3(m2);
  *ok = *ok && d1.ok && d2.ok;
  int g1[3], g2[3], n1 = 0, n2 = 0;
  for (int i = 0; i < 3; ++i) {
    g1[i] = d1.l.x[i] < kEps;
    g2[i] = d2.l.x[i] < kEps;
    n1 += g1[i];
    n2 += g2[i];
  }
  if (n1 > n2) {
    M3 t = m1;
    m1 = m2;
    m2 = t;
    Eig3 te = d1;
    d1 = d2;
    d2 = te;
    for (int i = 0; i < 3; ++i) {
      int tg = g1[i];
      g1[i] = g2[i];
      g2[i] = tg;
    }
    int tn = n1;
    n1 = n2;
    n2 = tn;
  }
  if (n1 == 3) return zero3();
  if (n1 != 0) return intersect_degen3(m1, d1, g1, n1, m2, d2, g2, n2, ok);
  V3 s, is;
  for (int i = 0; i < 3; ++i) {
    s.x[i] = sqrt(d1.l.x[i]);
    is.x[i] = 1.0 / s.x[i];
  }
  M3 m1_sqrt = compose_ortho3(d1.q, s);
  M3 m1_isqrt = compose_ortho3(d1.q, is);
  M3 m2_bar = mm3(mm3(tr3(m1_isqrt), m2), m1_isqrt);
  Eig3 db = eigen3(m2_bar);
  *ok = *ok && db.ok;
  V3 l;
  for (int i = 0; i < 3; ++i) l.x[i] = max2d(db.l.x[i], 1.0);
  M3 mib = compose_ortho3(db.q, l);
  return mm3(mm3(tr3(m1_sqrt), mib), m1_sqrt);
}
OHG_HD M2 intersect2(M2 m1, M2 m2, bool* ok) {
  Eig2 d1 = eigen2(m1), d2 = eigen2(m2);
  *ok = *ok && d1.ok && d2.ok;
  int g1[2], g2[2], n1 = 0, n2 = 0;
  for (int i = 0; i < 2; ++i) {
    g1[i] = d1.l.x[i] < kEps;
    g2[i] = d2.l.x[i] < kEps;
    n1 += g1[i];
    n2 += g2[i];
  }
  if (n1 > n2) {
    M2 t = m1;
    m1 = m2;
    m2 = t;
    Eig2 te = d1;
    d1 = d2;
    d2 = te;
    for (int i = 0; i < 2; ++i) {
      int tg = g1[i];
      g1[i] = g2[i];
      g2[i] = tg;
    }
    int tn = n1;
    n1 = n2;
    n2 = tn;
  }
  if (n1 == 2) return zero2();
  if (n1 != 0) return intersect_degen2(m1, d1, g1, m2, d2, g2);
  V2 s, is;
  for (int i = 0; i < 2; ++i) {
    s.x[i] = sqrt(d1.l.x[i]);
    is.x[i] = 1.0 / s.x[i];
  }
  M2 m1_sqrt = compose_ortho2(d1.q, s);
  M2 m1_isqrt = compose_ortho2(d1.q, is);
  M2 m2_bar = mm2(mm2(tr2(m1_isqrt), m2), m1_isqrt);
  Eig2 db = eigen2(m2_bar);
  *ok = *ok && db.ok;
  V2 l;
  for (int i = 0; i < 2; ++i) l.x[i] = max2d(db.l.x[i], 1.0);
  M2 mib = compose_ortho2(db.q, l);
  return mm2(mm2(tr2(m1_sqrt), mib), m1_sqrt);
}

// Householder QR least squares (src/Omega_h_qr.hpp: Trefethen and Bau,
// algorithms 10.1, 10.2 and 11.2) for the 6x6 system of the 3D implied
// metric; a[j][i] is column j, row i
OHG_HD void solve_qr6(double a[6][6], double b[6], double x[6], bool* ok) {
  double v[6][6];
  for (int k = 0; k < 6; ++k) {
    double nx = 0.0;
    for (int i = k; i < 6; ++i) nx += a[k][i] * a[k][i];
    nx = sqrt(nx);
    if (!(nx > 0.0)) *ok = false;
    for (int i = k; i < 6; ++i) v[k][i] = a[k][i];
    v[k][k] += ((a[k][k] < 0.0) ? -1.0 : 1.0) * nx;
    double nv = 0.0;
    for (int i = k; i < 6; ++i) nv += v[k][i] * v[k][i];
    nv = sqrt(nv);
    for (int i = k; i < 6; ++i) v[k][i] /= nv;
    for (int j = k; j < 6; ++j) {
      double dot = 0.0;
      for (int i = k; i < 6; ++i) dot += a[j][i] * v[k][i];
      for (int i = k; i < 6; ++i) a[j][i] -= 2.0 * dot * v[k][i];
    }
  }
  for (int k = 0; k < 6; ++k) {
    double dot = 0.0;
    for (int i = k; i < 6; ++i) dot += v[k][i] * b[i];
    for (int i = k; i < 6; ++i) b[i] -= 2.0 * dot * v[k][i];
  }
  for (int ii = 0; ii < 6; ++ii) {
    int i = 5 - ii;
    x[i] = b[i];
    for (int j = i + 1; j < 6; ++j) x[i] -= a[j][i] * x[j];
    x[i] /= a[i][i];
  }
}

// element_implied_metric (src/Omega_h_shape.hpp:240-273): the metric in
// which every edge of the element has unit length
OHG_HD M3 implied_metric3(const V3 p[4], bool* ok) {
  V3 b0 = sub3(p[1], p[0]), b1 = sub3(p[2], p[0]), b2 = sub3(p[3], p[0]);
  V3 nb1 = {{-b1.x[0], -b1.x[1], -b1.x[2]}};
  V3 ev[6] = {b0, sub3(p[2], p[1]), nb1, b2, sub3(p[3], p[1]), sub3(p[3], p[2])};
  double a[6][6], rhs[6], x[6];
  for (int i = 0; i < 6; ++i) {
    a[0][i] = ev[i].x[0] * ev[i].x[0];
    a[1][i] = ev[i].x[1] * ev[i].x[1];
    a[2][i] = ev[i].x[2] * ev[i].x[2];
    a[3][i] = 2 * ev[i].x[0] * ev[i].x[1];
    a[4][i] = 2 * ev[i].x[1] * ev[i].x[2];
    a[5][i] = 2 * ev[i].x[0] * ev[i].x[2];
    rhs[i] = 1.0;
  }
  solve_qr6(a, rhs, x, ok);
  return symm3(x);
}
OHG_HD M2 implied_metric2(const V2 p[3]) {
  V2 b0 = {{p[1].x[0] - p[0].x[0], p[1].x[1] - p[0].x[1]}};
  V2 b1 = {{p[2].x[0] - p[0].x[0], p[2].x[1] - p[0].x[1]}};
  V2 ev[3] = {b0, {{p[2].x[0] - p[1].x[0], p[2].x[1] - p[1].x[1]}}, {{-b1.x[0], -b1.x[1]}}};
  M3 a;
  V3 rhs;
  for (int i = 0; i < 3; ++i) {
    a.c[0].x[i] = ev[i].x[0] * ev[i].x[0];
    a.c[1].x[i] = ev[i].x[1] * ev[i].x[1];
    a.c[2].x[i] = 2 * ev[i].x[0] * ev[i].x[1];
    rhs.x[i] = 1.0;
  }
  V3 x = mv3(inv3(a), rhs);
  double v[3] = {x.x[0], x.x[1], x.x[2]};
  return symm2(v);
}

}  // namespace

namespace {

// packed symmetric tensor <-> matrix, by dimension
OHG_HD int mcomps(int dim) { return dim == 3 ? 6 : 3; }

// log-Euclidean average of n packed metrics (average_metric with its
// contrib/finish steps, src/Omega_h_metric.hpp:126-150); degenerate
// (max_norm < 1e-10) metrics are skipped when has_degen
OHG_HD void average3(const double* const* ms, int n, bool has_degen, double* out, bool* ok) {
  M3 am = zero3();
  int ng = 0;
  for (int k = 0; k < n; ++k) {
    M3 m = symm3(ms[k]);
    if (has_degen && max_norm3(m) < kEps) continue;
    M3 l = log_spd3(m, ok);
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] + l.c[j].x[i];
    ++ng;
  }
  if (has_degen && ng == 0) {
    unsymm3(am, out);
    return;
  }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] / double(ng);
  unsymm3(exp_spd3(am, ok), out);
}
OHG_HD void average2(const double* const* ms, int n, bool has_degen, double* out, bool* ok) {
  M2 am = zero2();
  int ng = 0;
  for (int k = 0; k < n; ++k) {
    M2 m = symm2(ms[k]);
    if (has_degen && max_norm2(m) < kEps) continue;
    M2 l = log_spd2(m, ok);
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] + l.c[j].x[i];
    ++ng;
  }
  if (has_degen && ng == 0) {
    unsymm2(am, out);
    return;
  }
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] / double(ng);
  unsymm2(exp_spd2(am, ok), out);
}

// empirical volume of an element of a unit-edge mesh and the volume of the
// equilateral simplex (src/Omega_h_metric.cpp:288-294,
// src/Omega_h_shape.hpp:406-409)
double typical_unit_simplex_size(int dim) { return dim == 3 ? 0.0838934100219 : 0.377645136635; }
double equilateral_simplex_size(int dim) { return dim == 3 ? 0.1178511301977579 : 0.4330127018922193; }
// power(x, 2, dim) of src/Omega_h_scalar.hpp: x^(2/dim)
double power_2_over(double x, int dim) { return dim == 3 ? cbrt_cr(x * x) : x; }

// per-vertex metrics from per-element ones (project_metrics,
// src/Omega_h_metric.cpp:222-252): log-Euclidean mean over the elements of
// each vertex, degenerate ones skipped
Arr<double> project_metrics(Mesh& m, const Arr<double>& e2m) {
  int dim = m.dim, mc = mcomps(dim);
  const Adj& v2e = m.ask_up(0, dim);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto em = cview(e2m);
  Arr<double> out(m.nverts() * mc);
  auto o = view(out);
  int* st = ctx().d_status;
  pfor(m.nverts(), [=] __device__(LO v) {
    LO x0 = va[v], n = va[v + 1] - x0;
    bool ok = true;
    // the logs are summed in the row's (element) order
    if (dim == 3) {
      M3 am = zero3();
      int ng = 0;
      for (LO k = 0; k < n; ++k) {
        M3 mm = symm3(&em[vb[x0 + k] * 6]);
        if (max_norm3(mm) < kEps) continue;
        M3 l = log_spd3(mm, &ok);
        for (int j = 0; j < 3; ++j)
          for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] + l.c[j].x[i];
        ++ng;
      }
      if (ng) {
        for (int j = 0; j < 3; ++j)
          for (int i = 0; i < 3; ++i) am.c[j].x[i] = am.c[j].x[i] / double(ng);
        am = exp_spd3(am, &ok);
      }
      unsymm3(am, &o[v * 6]);
    } else {
      M2 am = zero2();
      int ng = 0;
      for (LO k = 0; k < n; ++k) {
        M2 mm = symm2(&em[vb[x0 + k] * 3]);
        if (max_norm2(mm) < kEps) continue;
        M2 l = log_spd2(mm, &ok);
        for (int j = 0; j < 2; ++j)
          for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] + l.c[j].x[i];
        ++ng;
      }
      if (ng) {
        for (int j = 0; j < 2; ++j)
          for (int i = 0; i < 2; ++i) am.c[j].x[i] = am.c[j].x[i] / double(ng);
        am = exp_spd2(am, &ok);
      }
      unsymm2(am, &o[v * 3]);
    }
    if (!ok) raise_status(st, ST_NUMERIC);
  });
  return out;
}

// element metrics as the mean of their vertices' (get_mident_metrics over
// elements, has_degen false)
Arr<double> element_mident_metrics(Mesh& m, const double* v2m_p) {
  int dim = m.dim, mc = mcomps(dim);
  auto ev = cview(m.ask_verts_of(dim));
  auto vm = cview(v2m_p, m.nverts() * mc);
  Arr<double> out(m.nelems() * mc);
  auto o = view(out);
  int* st = ctx().d_status;
  pfor(m.nelems(), [=] __device__(LO e) {
    bool ok = true;
    const double* ms[4];
    for (int k = 0; k <= dim; ++k) ms[k] = &vm[ev[e * (dim + 1) + k] * mc];
    if (dim == 3)
      average3(ms, 4, false, &o[e * 6], &ok);
    else
      average2(ms, 3, false, &o[e * 3], &ok);
    if (!ok) raise_status(st, ST_NUMERIC);
  });
  return out;
}

Arr<double> scale_each(const Arr<double>& a, double s) {
  Arr<double> out(a.size());
  auto i_ = cview(a);
  auto o = view(out);
  pfor(a.size(), [=] __device__(LO i) { o[i] = i_[i] * s; });
  return out;
}

// metrics_from_isos (src/Omega_h_metric.cpp:559-575)
Arr<double> metrics_from_isos(int dim, const Arr<double>& isos) {
  int mc = mcomps(dim);
  Arr<double> out(isos.size() * mc);
  auto s = cview(isos);
  auto o = view(out);
  pfor(isos.size(), [=] __device__(LO i) {
    for (int k = 0; k < mc; ++k) o[i * mc + k] = k < dim ? s[i] : 0.0;
  });
  return out;
}

// get_size_isos (src/Omega_h_metric.cpp:577-598): det(M)^(1/dim)
Arr<double> size_isos(int dim, LO n, const double* m_p) {
  Arr<double> out(n);
  auto mm = cview(m_p, n * mcomps(dim));
  auto o = view(out);
  pfor(n, [=] __device__(LO i) {
    if (dim == 3) {
      o[i] = cbrt_cr(det3(symm3(&mm[i * 6])));
    } else {
      M2 s = symm2(&mm[i * 3]);
      o[i] = sqrt(s.c[0].x[0] * s.c[1].x[1] - s.c[1].x[0] * s.c[0].x[1]);
    }
  });
  return out;
}

// exact sum of doubles (repro_sum, src/Omega_h_array_ops.cpp:496-545): every
// value truncated to an integer count of 2^(e - 52), e the largest binary
// exponent, and the integers summed exactly; the device adds the high and
// the low 32 bits of each count into two 64-bit integers
double exact_sum(const Arr<double>& a) {
  LO n = a.size();
  if (n == 0) return 0.0;
  Arr<long long> acc = fill<long long>(3, 0);
  Arr<int> ex = fill<int>(1, INT_MIN);
  auto v = cview(a);
  auto e = view(ex);
  pfor(n, [=] __device__(LO i) {
    if (v[i] == 0.0) return;
    int x;
    frexp(v[i], &x);
    atomicMax(&e[0], x);
  });
  std::vector<int> he = to_host(ex);
  if (he[0] == INT_MIN) return 0.0;
  double unit = std::exp2(double(he[0] - 52));
  auto ac = view(acc);
  pfor(n, [=] __device__(LO i) {
    long long t = (long long)(v[i] / unit);
    unsigned long long lo = (unsigned long long)t & 0xffffffffULL;
    long long hi = t >> 32;
    if (lo) atomicAdd(reinterpret_cast<unsigned long long*>(&ac[0]), lo);
    if (hi) atomicAdd(reinterpret_cast<unsigned long long*>(&ac[1]), (unsigned long long)hi);
  });
  std::vector<long long> h = to_host(acc);
  __int128 s = (__int128)h[1] * ((__int128)1 << 32) + (__int128)(unsigned long long)h[0];
  // Int128::to_double (src/Omega_h_int128.cpp:5-16)
  bool neg = s < 0;
  unsigned __int128 t = neg ? (unsigned __int128)(-s) : (unsigned __int128)s;
  while ((t >> 64) != 0) {
    t >>= 1;
    unit *= 2;
  }
  double x = double((unsigned long long)t);
  if (neg) x = -x;
  return x * unit;
}

}  // namespace

// ------------------------------------------------------------ entry points
// find_polynomial_roots of n monic cubics (coefficients a_0, a_1, a_2 each;
// src/Omega_h_eigen.hpp:21-85), one thread per cubic
void cubic_roots_batch(LO n, const double* coeffs_p, double eps, int* nroots_p, double* roots_p,
                       int* mults_p) {
  auto cf = cview(coeffs_p, n * 3);
  auto nr = view(nroots_p, n);
  auto rv = view(roots_p, n * 3);
  auto mu = view(mults_p, n * 3);
  pfor(n, [=] __device__(LO i) {
    double rt[3];
    int ml[3];
    nr[i] = cubic_roots(cf[i * 3], cf[i * 3 + 1], cf[i * 3 + 2], eps, rt, ml);
    for (int k = 0; k < 3; ++k) {
      rv[i * 3 + k] = rt[k];
      mu[i * 3 + k] = ml[k];
    }
  });
}

// decompose_eigen (src/Omega_h_eigen.hpp:278-293) of n dim x dim matrices
// stored by columns; q by columns (the eigenvectors), l the eigenvalues
void decompose_eigen_batch(int dim, LO n, const double* m_p, double* q_p, double* l_p) {
  int mm = dim * dim;
  auto a = cview(m_p, n * mm);
  auto q = view(q_p, n * mm);
  auto l = view(l_p, n * dim);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    bool ok;
    if (dim == 3) {
      M3 m;
      for (int j = 0; j < 3; ++j)
        for (int r = 0; r < 3; ++r) m.c[j].x[r] = a[i * 9 + j * 3 + r];
      Eig3 e = eigen3(m);
      ok = e.ok;
      for (int j = 0; j < 3; ++j) {
        for (int r = 0; r < 3; ++r) q[i * 9 + j * 3 + r] = e.q.c[j].x[r];
        l[i * 3 + j] = e.l.x[j];
      }
    } else {
      M2 m;
      for (int j = 0; j < 2; ++j)
        for (int r = 0; r < 2; ++r) m.c[j].x[r] = a[i * 4 + j * 2 + r];
      Eig2 e = eigen2(m);
      ok = e.ok;
      for (int j = 0; j < 2; ++j) {
        for (int r = 0; r < 2; ++r) q[i * 4 + j * 2 + r] = e.q.c[j].x[r];
        l[i * 2 + j] = e.l.x[j];
      }
    }
    if (!ok) raise_status(st, ST_NUMERIC);
  });
}

void intersect_metrics(int dim, LO n, const double* a_p, const double* b_p, double* out_p) {
  int mc = mcomps(dim);
  auto a = cview(a_p, n * mc);
  auto b = cview(b_p, n * mc);
  auto o = view(out_p, n * mc);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    bool ok = true;
    if (dim == 3)
      unsymm3(intersect3(symm3(&a[i * 6]), symm3(&b[i * 6]), &ok), &o[i * 6]);
    else
      unsymm2(intersect2(symm2(&a[i * 3]), symm2(&b[i * 3]), &ok), &o[i * 3]);
    if (!ok) raise_status(st, ST_NUMERIC);
  });
}

// clamp_metrics (src/Omega_h_metric.cpp:36-56, clamp_metric
// src/Omega_h_metric.hpp:153-160)
void clamp_metrics(int dim, LO n, const double* m_p, double h_min, double h_max, double* out_p) {
  int mc = mcomps(dim);
  auto mm = cview(m_p, n * mc);
  auto o = view(out_p, n * mc);
  double l_max = 1.0 / (h_min * h_min), l_min = 1.0 / (h_max * h_max);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    if (dim == 3) {
      Eig3 e = eigen3(symm3(&mm[i * 6]));
      for (int k = 0; k < 3; ++k) e.l.x[k] = min2d(max2d(e.l.x[k], l_min), l_max);
      unsymm3(compose_ortho3(e.q, e.l), &o[i * 6]);
      if (!e.ok) raise_status(st, ST_NUMERIC);
    } else {
      Eig2 e = eigen2(symm2(&mm[i * 3]));
      for (int k = 0; k < 2; ++k) e.l.x[k] = min2d(max2d(e.l.x[k], l_min), l_max);
      unsymm2(compose_ortho2(e.q, e.l), &o[i * 3]);
      if (!e.ok) raise_status(st, ST_NUMERIC);
    }
  });
}

// get_hessian_metrics (src/Omega_h_metric.cpp:332-368): eigenvalues
// d^2 |l| / (2 (d+1)^2 eps), recomposed with the inverse of the eigenvectors
void hessian_metrics(int dim, LO n, const double* h_p, double eps, double* out_p) {
  int mc = mcomps(dim);
  auto hh = cview(h_p, n * mc);
  auto o = view(out_p, n * mc);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    if (dim == 3) {
      Eig3 e = eigen3(symm3(&hh[i * 6]));
      V3 tl;
      for (int k = 0; k < 3; ++k) tl.x[k] = (9 * fabs(e.l.x[k])) / (32 * eps);
      unsymm3(mm3(mm3(e.q, diag3(tl)), inv3(e.q)), &o[i * 6]);
      if (!e.ok) raise_status(st, ST_NUMERIC);
    } else {
      Eig2 e = eigen2(symm2(&hh[i * 3]));
      V2 tl;
      for (int k = 0; k < 2; ++k) tl.x[k] = (4 * fabs(e.l.x[k])) / (18 * eps);
      unsymm2(mm2(mm2(e.q, diag2(tl)), inv2(e.q)), &o[i * 3]);
      if (!e.ok) raise_status(st, ST_NUMERIC);
    }
  });
}

// get_implied_metrics (src/Omega_h_metric.cpp:260-309): each element's
// unit-edge metric scaled from the equilateral to the typical element
// volume, then projected to the vertices
Arr<double> implied_metrics(Mesh& m) {
  int dim = m.dim, mc = mcomps(dim);
  auto ev = cview(m.ask_verts_of(dim));
  auto c = cview(m.coords);
  Arr<double> e2m(m.nelems() * mc);
  auto o = view(e2m);
  int* st = ctx().d_status;
  pfor(m.nelems(), [=] __device__(LO e) {
    bool ok = true;
    if (dim == 3) {
      V3 p[4];
      for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) p[k].x[j] = c[ev[e * 4 + k] * 3 + j];
      unsymm3(implied_metric3(p, &ok), &o[e * 6]);
    } else {
      V2 p[3];
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 2; ++j) p[k].x[j] = c[ev[e * 3 + k] * 2 + j];
      unsymm2(implied_metric2(p), &o[e * 3]);
    }
    if (!ok) raise_status(st, ST_NUMERIC);
  });
  double size_scalar = typical_unit_simplex_size(dim) / equilateral_simplex_size(dim);
  return project_metrics(m, scale_each(e2m, power_2_over(size_scalar, dim)));
}

// limit_metric_gradation (src/Omega_h_metric.cpp:156-220): each sweep
// intersects every vertex metric with its neighbours' metrics grown by
// (1 + rate * metric distance)^2 in length, until no value changes by more
// than tol relative (floor 1e-10)
Arr<double> limit_metric_gradation(Mesh& m, const Arr<double>& v2m, double max_rate, double tol,
                                   int* steps) {
  if (!(max_rate > 0.0)) throw Error(1, "limit_metric_gradation: max_rate must be positive");
  int dim = m.dim, mc = mcomps(dim);
  const Adj& v2e = m.ask_up(0, 1);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto vcd = cview(v2e.codes);
  auto ev = cview(m.ask_verts_of(1));
  auto c = cview(m.coords);
  int* st = ctx().d_status;
  Arr<double> cur = v2m;
  Arr<int> close = fill<int>(1, 1);
  int i = 0;
  constexpr int kMaxSweeps = 10000;  // a guard; the reference's loop is unbounded
  for (;;) {
    Arr<double> next(cur.size());
    auto in = cview(cur);
    auto o = view(next);
    pfor(m.nverts(), [=] __device__(LO v) {
      bool ok = true;
      if (dim == 3) {
        M3 mm = symm3(&in[v * 6]);
        V3 x = {{c[v * 3], c[v * 3 + 1], c[v * 3 + 2]}};
        for (LO k = va[v]; k < va[v + 1]; ++k) {
          LO e = vb[k];
          LO av = ev[e * 2 + (1 - code_which_down(vcd[k]))];
          M3 am = symm3(&in[av * 6]);
          V3 ax = {{c[av * 3], c[av * 3 + 1], c[av * 3 + 2]}};
          V3 vec = sub3(ax, x);
          double dist = sqrt(metric_product3(am, vec));
          double h = 1.0 + dist * max_rate;
          mm = intersect3(mm, scale3(am, 1.0 / (h * h)), &ok);
        }
        unsymm3(mm, &o[v * 6]);
      } else {
        M2 mm = symm2(&in[v * 3]);
        V2 x = {{c[v * 2], c[v * 2 + 1]}};
        for (LO k = va[v]; k < va[v + 1]; ++k) {
          LO e = vb[k];
          LO av = ev[e * 2 + (1 - code_which_down(vcd[k]))];
          M2 am = symm2(&in[av * 3]);
          V2 vec = {{c[av * 2] - x.x[0], c[av * 2 + 1] - x.x[1]}};
          V2 mv = mv2(am, vec);
          double dist = sqrt(vec.x[0] * mv.x[0] + vec.x[1] * mv.x[1]);
          double h = 1.0 + dist * max_rate;
          mm = intersect2(mm, scale2(am, 1.0 / (h * h)), &ok);
        }
        unsymm2(mm, &o[v * 3]);
      }
      if (!ok) raise_status(st, ST_NUMERIC);
    });
    ++i;
    // are_close over all values (rel_diff_with_floor, src/Omega_h_scalar.hpp:266-277)
    auto a = cview(cur);
    auto b = cview(next);
    auto cl = view(close);
    pfor(1, [=] __device__(LO) { cl[0] = 1; });
    pfor(cur.size(), [=] __device__(LO k) {
      double am = fabs(a[k]), bm = fabs(b[k]);
      if (am <= kEps && bm <= kEps) return;
      if (!(fabs(b[k] - a[k]) / max2d(am, bm) <= tol)) cl[0] = 0;
    });
    cur = next;
    if (to_host(close)[0]) break;
    if (i >= kMaxSweeps) throw Error(5, "limit_metric_gradation: no convergence");
  }
  (void)mc;
  if (steps) *steps = i;
  return cur;
}

// get_expected_nelems (src/Omega_h_metric.cpp:465-519): the exact sum over
// elements of volume * sqrt(det of the element's mean metric), over the
// typical unit simplex volume
double expected_nelems(Mesh& m, const double* v2m) {
  int dim = m.dim, mc = mcomps(dim);
  Arr<double> em = element_mident_metrics(m, v2m);
  auto ev = cview(m.ask_verts_of(dim));
  auto c = cview(m.coords);
  auto emv = cview(em);
  Arr<double> per(m.nelems());
  auto o = view(per);
  pfor(m.nelems(), [=] __device__(LO e) {
    if (dim == 3) {
      V3 p[4];
      for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) p[k].x[j] = c[ev[e * 4 + k] * 3 + j];
      V3 b0 = sub3(p[1], p[0]), b1 = sub3(p[2], p[0]), b2 = sub3(p[3], p[0]);
      double vol = dot3(cross3(b0, b1), b2) / 6.0;
      o[e] = vol * sqrt(det3(symm3(&emv[e * 6])));
    } else {
      double p[3][2];
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 2; ++j) p[k][j] = c[ev[e * 3 + k] * 2 + j];
      double b0x = p[1][0] - p[0][0], b0y = p[1][1] - p[0][1];
      double b1x = p[2][0] - p[0][0], b1y = p[2][1] - p[0][1];
      double area = (b0x * b1y - b0y * b1x) / 2.0;
      M2 s = symm2(&emv[e * 3]);
      o[e] = area * sqrt(s.c[0].x[0] * s.c[1].x[1] - s.c[1].x[0] * s.c[0].x[1]);
    }
  });
  (void)mc;
  return exact_sum(per) / typical_unit_simplex_size(dim);
}

// generate_metrics (src/Omega_h_metric_input.cpp:140-275) for the constant,
// given and implied sources
Arr<double> generate_metrics(Mesh& m, const MetricInput& in, int* niters_out) {
  int dim = m.dim, mc = mcomps(dim);
  LO n = m.nverts();
  if (in.sources.empty()) throw Error(1, "generate_metrics: no sources given");
  if (in.limit_lengths && !(in.min_length <= in.max_length))
    throw Error(1, "generate_metrics: min_length above max_length");
  std::vector<Arr<double>> orig;
  std::vector<bool> iso;
  int metric_dim = 1;
  for (const MetricSource& s : in.sources) {
    Arr<double> ms;
    bool is_iso = false;
    switch (s.type) {
      case MS_CONSTANT:
        ms = fill<double>(n, 1.0 / (s.knob * s.knob));
        is_iso = true;
        break;
      case MS_GIVEN: {
        if (!s.given) throw Error(1, "generate_metrics: given source without metrics");
        ms = Arr<double>(n * mc);
        OHG_CUDA(cudaMemcpyAsync(ms.data(), s.given, sizeof(double) * size_t(n) * mc,
                                 cudaMemcpyDeviceToDevice, ctx().stream));
        if (s.knob != 1.0) ms = scale_each(ms, 1.0 / (s.knob * s.knob));
        break;
      }
      case MS_IMPLIED:
        ms = implied_metrics(m);
        if (s.knob != 1.0) ms = scale_each(ms, 1.0 / (s.knob * s.knob));
        break;
      default:
        throw Error(1, "generate_metrics: variation, derivative and curvature sources are not built");
    }
    if (!is_iso) {
      if (s.isotropy == MI_ISO_SIZE) {
        ms = size_isos(dim, n, ms.data());
        is_iso = true;
      } else if (s.isotropy == MI_ISO_LENGTH) {
        throw Error(1, "generate_metrics: the iso-length isotropy is not built");
      }
    }
    if (!is_iso) metric_dim = dim;
    orig.push_back(ms);
    iso.push_back(is_iso);
  }
  if (metric_dim != dim)
    throw Error(1, "generate_metrics: all sources isotropic (scalar metrics are not built)");
  double scalar = 1.0;
  Arr<double> metrics;
  int niters;
  for (niters = 0;; ++niters) {
    if (niters == 100) throw Error(5, "generate_metrics: too many element count iterations");
    for (size_t i = 0; i < in.sources.size(); ++i) {
      Arr<double> cur = iso[i] ? metrics_from_isos(dim, orig[i]) : orig[i];
      if (in.sources[i].scales == MSC_SCALES) cur = scale_each(cur, scalar);
      if (in.limit_lengths) {
        Arr<double> cl(cur.size());
        clamp_metrics(dim, n, cur.data(), in.min_length, in.max_length, cl.data());
        cur = cl;
      }
      if (i) {
        Arr<double> x(cur.size());
        intersect_metrics(dim, n, metrics.data(), cur.data(), x.data());
        metrics = x;
      } else {
        metrics = cur;
      }
    }
    for (int k = 0; k < in.nsmoothing_steps; ++k)
      metrics = project_metrics(m, element_mident_metrics(m, metrics.data()));
    if (in.limit_gradation)
      metrics = limit_metric_gradation(m, metrics, in.max_gradation_rate, in.gradation_tol, nullptr);
    if (!in.limit_element_count) break;
    double ne = expected_nelems(m, metrics.data());
    if (ne > in.max_element_count) {
      scalar *= power_2_over(in.max_element_count / ne, dim);
      scalar /= in.element_count_over_relaxation;
    } else if (ne < in.min_element_count) {
      scalar *= power_2_over(in.min_element_count / ne, dim);
      scalar *= in.element_count_over_relaxation;
    } else {
      break;
    }
  }
  if (niters_out) *niters_out = niters;
  return metrics;
}

}  // namespace ohg
