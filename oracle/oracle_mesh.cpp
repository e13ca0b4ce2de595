// ORACLE — test infrastructure only (see oracle_core.hpp).
// Eigen/metric math, adjacency derivation, box construction, Hilbert order,
// classification and measurement.
#include <algorithm>
#include <cfloat>
#include <numeric>

#include "oracle_core.hpp"

namespace orc {

static const double PI = 3.14159265358979323;
static const double EPSILON = 1e-10;

static inline double square(double x) { return x * x; }
static inline double cube(double x) { return x * (x * x); }
static inline double max2(double a, double b) { return (a < b) ? b : a; }
static inline double min2(double a, double b) { return (b < a) ? b : a; }
static inline double clampd(double x, double lo, double hi) {
  return min2(max2(x, lo), hi);
}

// ------------------------------------------------------------ eigen (3x3)
// find_polynomial_roots for a monic cubic (src/Omega_h_eigen.hpp:21-85)
struct Roots3 {
  int n;
  double r[3];
  int mult[3];
};
static Roots3 cubic_roots(double a_0, double a_1, double a_2, double eps) {
  double roots[3] = {0, 0, 0};
  int mults[3];
  double p = (3. * a_1 - square(a_2)) / 3.;
  double q = (9. * a_1 * a_2 - 27. * a_0 - 2. * cube(a_2)) / 27.;
  double Q = p / 3.;
  double R = q / 2.;
  double D = cube(Q) + square(R);
  double shift = -a_2 / 3.;
  if (D >= 0.0) {
    double S = orc_cbrt(R + std::sqrt(D));
    double T = orc_cbrt(R - std::sqrt(D));
    double B = S + T;
    double z_1 = shift + B;
    double z_23_real = shift - (1. / 2.) * B;
    roots[0] = z_1;
    roots[1] = roots[2] = z_23_real;
  } else {
    double cos_theta = R / std::sqrt(-cube(Q));
    double theta = orc_acos(clampd(cos_theta, -1.0, 1.0));
    double radius = 2. * std::sqrt(-Q);
    roots[0] = radius * orc_cos((theta) / 3.) + shift;
    roots[1] = radius * orc_cos((theta + 2. * PI) / 3.) + shift;
    roots[2] = radius * orc_cos((theta - 2. * PI) / 3.) + shift;
  }
  mults[0] = mults[1] = mults[2] = 1;
  if (std::abs(roots[0] - roots[1]) < eps) {
    std::swap(roots[0], roots[2]);
  } else if (std::abs(roots[0] - roots[2]) < eps) {
    std::swap(roots[0], roots[1]);
  } else if (std::abs(roots[1] - roots[2]) < eps) {
  } else {
    return {3, {roots[0], roots[1], roots[2]}, {1, 1, 1}};
  }
  roots[1] = (roots[1] + roots[2]) / 2;
  mults[1] = 2;
  if (std::abs(roots[0] - roots[1]) < eps) {
    roots[0] = (1. / 3.) * roots[0] + (2. / 3.) * roots[1];
    mults[0] = 3;
    return {1, {roots[0], roots[1], roots[2]}, {mults[0], mults[1], mults[2]}};
  }
  return {2, {roots[0], roots[1], roots[2]}, {mults[0], mults[1], mults[2]}};
}

static Mat3 identity3() {
  Mat3 a;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) a[j][i] = (i == j);
  return a;
}
static double trace3(const Mat3& a) {
  double t = a[0][0];
  for (int i = 1; i < 3; ++i) t += a[i][i];
  return t;
}
static double max_norm3(const Mat3& a) {
  double x = 0.0;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) x = max2(x, std::abs(a[j][i]));
  return x;
}
static Mat3 subtract_from_diag3(Mat3 a, double mu) {
  for (int i = 0; i < 3; ++i) a[i][i] -= mu;
  return a;
}
static Vec3 single_eigenvector3(const Mat3& m, double l) {
  Mat3 s = transpose3(subtract_from_diag3(m, l));
  Vec3 v = cross3(s[0], s[1]);
  double v_norm = norm3(v);
  Vec3 c = cross3(s[1], s[2]);
  double c_norm = norm3(c);
  if (c_norm > v_norm) {
    v = c;
    v_norm = c_norm;
  }
  c = cross3(s[0], s[2]);
  c_norm = norm3(c);
  if (c_norm > v_norm) {
    v = c;
    v_norm = c_norm;
  }
  OCHECK(v_norm > EPSILON);
  return vdiv(v, v_norm);
}
static Vec3 row_space_1d3(const Mat3& a) {
  Mat3 ta = transpose3(a);
  int best = 0;
  double best_norm = norm3(ta[0]);
  for (int i = 1; i < 3; ++i) {
    double rn = norm3(ta[i]);
    if (rn > best_norm) {
      best = i;
      best_norm = rn;
    }
  }
  OCHECK(best_norm > EPSILON);
  return vdiv(ta[best], best_norm);
}
// Duff et al. 2017 orthonormal basis (src/Omega_h_matrix.hpp:567-576)
static Mat3 ortho_basis3(Vec3 v) {
  Mat3 A;
  A[0] = v;
  double sign = std::copysign(1.0, v[2]);
  const double a = -1.0 / (sign + v[2]);
  const double b = v[0] * v[1] * a;
  A[1] = {{1.0 + sign * v[0] * v[0] * a, sign * b, -sign * v[0]}};
  A[2] = {{b, sign + v[1] * v[1] * a, -v[1]}};
  return A;
}
struct Decomp3 {
  Mat3 q;
  Vec3 l;
};
static Decomp3 decompose_eigen3(Mat3 m) {
  double nm = max_norm3(m);
  if (nm <= EPSILON) return {identity3(), {{0, 0, 0}}};
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) m[j][i] = m[j][i] / nm;
  double tA = trace3(m);
  double c2 = -tA;
  double c1 = (1. / 2.) * ((tA * tA) - trace3(mm3(m, m)));
  double c0 = -det3(m);
  Roots3 r = cubic_roots(c0, c1, c2, 5e-5);
  Mat3 q;
  Vec3 l;
  if (r.n == 3) {
    for (int i = 0; i < 3; ++i) {
      q[i] = single_eigenvector3(m, r.r[i]);
      l[i] = r.r[i];
    }
  } else if (r.n == 2 && r.mult[1] == 2) {
    q[0] = single_eigenvector3(m, r.r[0]);
    l[0] = r.r[0];
    Vec3 n = row_space_1d3(subtract_from_diag3(m, r.r[1]));
    Mat3 b = ortho_basis3(n);
    q[1] = b[1];
    q[2] = b[2];
    l[1] = l[2] = r.r[1];
  } else {
    OCHECK(r.n == 1 && r.mult[0] == 3);
    l[0] = l[1] = l[2] = r.r[0];
    q = identity3();
  }
  return {q, vscale(l, nm)};
}
static Mat3 compose_ortho3(const Mat3& q, Vec3 l) {
  Mat3 d;
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j) d[i][j] = d[j][i] = 0.0;
  for (int i = 0; i < 3; ++i) d[i][i] = l[i];
  return mm3(mm3(q, d), transpose3(q));
}
Mat3 log_spd3(Mat3 m) {
  Decomp3 d = decompose_eigen3(m);
  for (int i = 0; i < 3; ++i) d.l[i] = orc_log(d.l[i]);
  return compose_ortho3(d.q, d.l);
}
Mat3 exp_spd3(Mat3 m) {
  Decomp3 d = decompose_eigen3(m);
  for (int i = 0; i < 3; ++i) d.l[i] = orc_exp(d.l[i]);
  return compose_ortho3(d.q, d.l);
}
// average_metric of two metrics, has_degen = false (src/Omega_h_metric.hpp:120-150)
void average_metric3(const double* m0, const double* m1, double* out) {
  Mat3 am;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) am[j][i] = 0.0;
  const double* ms[2] = {m0, m1};
  int n = 0;
  for (int k = 0; k < 2; ++k) {
    Mat3 L = log_spd3(symm3(ms[k]));
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) am[j][i] = am[j][i] + L[j][i];
    n++;
  }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) am[j][i] = am[j][i] / n;
  unsymm3(exp_spd3(am), out);
}

// ------------------------------------------------------------ eigen (2x2)
static Mat2 identity2() {
  Mat2 a;
  a[0][0] = 1;
  a[0][1] = 0;
  a[1][0] = 0;
  a[1][1] = 1;
  return a;
}
static Mat2 mm2(const Mat2& a, const Mat2& b) {
  Mat2 c;
  for (int j = 0; j < 2; ++j) c[j] = mv2(a, b[j]);
  return c;
}
static Mat2 transpose2(const Mat2& a) {
  Mat2 b;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) b[i][j] = a[j][i];
  return b;
}
struct Decomp2 {
  Mat2 q;
  Vec2 l;
};
static Decomp2 decompose_eigen2(Mat2 m) {
  double nm = 0.0;
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) nm = max2(nm, std::abs(m[j][i]));
  if (nm <= EPSILON) return {identity2(), {{0, 0}}};
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) m[j][i] = m[j][i] / nm;
  double tr = m[0][0];
  tr += m[1][1];
  double a = -tr;
  double b = det2(m);
  double disc = square(a) - 4. * b;
  Decomp2 d;
  if (std::abs(disc) < 5e-5) {
    double r = -a / 2.;
    d.l[0] = d.l[1] = r;
    d.q = identity2();
  } else {
    OCHECK(disc > 0.0);
    double roots[2] = {(-a + std::sqrt(disc)) / 2., (-a - std::sqrt(disc)) / 2.};
    for (int i = 0; i < 2; ++i) {
      Mat2 s = m;
      for (int k = 0; k < 2; ++k) s[k][k] -= roots[i];
      Mat2 ts = transpose2(s);
      int best = 0;
      double bn = std::sqrt(dotn<2>(ts[0].v, ts[0].v));
      double n1 = std::sqrt(dotn<2>(ts[1].v, ts[1].v));
      if (n1 > bn) {
        best = 1;
        bn = n1;
      }
      OCHECK(bn > EPSILON);
      Vec2 r = {{ts[best][0] / bn, ts[best][1] / bn}};
      d.q[i] = {{-r[1], r[0]}};
      d.l[i] = roots[i];
    }
  }
  d.l[0] = d.l[0] * nm;
  d.l[1] = d.l[1] * nm;
  return d;
}
static Mat2 compose_ortho2(const Mat2& q, Vec2 l) {
  Mat2 d;
  d[0][1] = d[1][0] = 0.0;
  d[0][0] = l[0];
  d[1][1] = l[1];
  return mm2(mm2(q, d), transpose2(q));
}
Mat2 log_spd2(Mat2 m) {
  Decomp2 d = decompose_eigen2(m);
  for (int i = 0; i < 2; ++i) d.l[i] = orc_log(d.l[i]);
  return compose_ortho2(d.q, d.l);
}
Mat2 exp_spd2(Mat2 m) {
  Decomp2 d = decompose_eigen2(m);
  for (int i = 0; i < 2; ++i) d.l[i] = orc_exp(d.l[i]);
  return compose_ortho2(d.q, d.l);
}
void average_metric2(const double* m0, const double* m1, double* out) {
  Mat2 am;
  am[0][0] = am[0][1] = am[1][0] = am[1][1] = 0.0;
  const double* ms[2] = {m0, m1};
  int n = 0;
  for (int k = 0; k < 2; ++k) {
    Mat2 L = log_spd2(symm2(ms[k]));
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) am[j][i] = am[j][i] + L[j][i];
    n++;
  }
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) am[j][i] = am[j][i] / n;
  Mat2 e = exp_spd2(am);
  out[0] = e[0][0];
  out[1] = e[1][1];
  out[2] = e[1][0];
}

// ------------------------------------------------------------ adjacency
// invert_adj (src/Omega_h_adj.cpp:231-263).  A sequential counting fill in
// increasing high-use order yields rows already sorted by high index, which
// is the order the reference reaches with sort_by_high_index.
Adj invert_adj(const Adj& down, int k, LO nlows) {
  const V<LO>& hl2l = down.ab2b;
  LO nhl = LO(hl2l.size());
  Adj up;
  up.a2ab.assign((size_t)(nlows) + 1, 0);
  for (LO hl = 0; hl < nhl; ++hl) up.a2ab[(size_t)(hl2l[hl]) + 1]++;
  for (LO l = 0; l < nlows; ++l) up.a2ab[l + 1] += up.a2ab[l];
  up.ab2b.resize((size_t)(nhl));
  up.codes.resize((size_t)(nhl));
  V<LO> pos(up.a2ab.begin(), up.a2ab.end() - 1);
  for (LO hl = 0; hl < nhl; ++hl) {
    LO l = hl2l[hl];
    LO lh = pos[l]++;
    up.ab2b[lh] = hl / k;
    int wd = hl % k;
    if (!down.codes.empty()) {
      I8 dc = down.codes[hl];
      up.codes[lh] = make_code(code_is_flipped(dc), code_rotation(dc), wd);
    } else {
      up.codes[lh] = make_code(false, 0, wd);
    }
  }
  return up;
}

V<LO> form_uses(const V<LO>& hv2v, int hd, int ld) {
  int nvh = hd + 1, nvl = ld + 1, nlh = simplex_degree(hd, ld);
  LO nh = LO(hv2v.size() / (size_t)(nvh));
  V<LO> uv2v((size_t)(nh) * nlh * nvl);
  for (LO h = 0; h < nh; ++h)
    for (int u = 0; u < nlh; ++u)
      for (int uv = 0; uv < nvl; ++uv)
        uv2v[((size_t)(h) * nlh + u) * nvl + uv] =
            hv2v[(size_t)(h) * nvh + down_template(hd, ld, u, uv)];
  return uv2v;
}

// reflect_down / find_matches (src/Omega_h_adj.cpp:297-441)
Adj reflect_down(const V<LO>& hv2v, const V<LO>& lv2v, const Adj& v2l, int hd,
                 int ld) {
  V<LO> uv2v = form_uses(hv2v, hd, ld);
  int deg = ld + 1;
  LO na = LO(uv2v.size() / (size_t)(deg));
  Adj out;
  out.ab2b.resize((size_t)(na));
  out.codes.resize((size_t)(na));
  ORC_PARALLEL_FOR
  for (LO a = 0; a < na; ++a) {
    const LO* av = &uv2v[(size_t)(a) * deg];
    LO fv = av[0];
    bool found = false;
    for (LO vb = v2l.a2ab[fv]; vb < v2l.a2ab[fv + 1]; ++vb) {
      LO b = v2l.ab2b[vb];
      int wd = code_which_down(v2l.codes[vb]);
      const LO* bv = &lv2v[(size_t)(b) * deg];
      I8 mc = 0;
      bool match = false;
      if (deg == 2) {
        if (av[1] == bv[1 - wd]) {
          mc = make_code(false, wd, 0);
          match = true;
        }
      } else {
        if (av[1] == bv[(wd + 1) % 3] && av[2] == bv[(wd + 2) % 3]) {
          mc = make_code(false, rotation_to_first(3, wd), 0);
          match = true;
        } else if (av[1] == bv[(wd + 2) % 3] && av[2] == bv[(wd + 1) % 3]) {
          mc = make_code(true, rotation_to_first(3, wd), 0);
          match = true;
        }
      }
      if (match) {
        OCHECK(!found);
        out.ab2b[a] = b;
        out.codes[a] = mc;
        found = true;
      }
    }
    OCHECK(found);
  }
  if (ld == 0) out.codes.clear();
  return out;
}

// transit (src/Omega_h_adj.cpp:443-510)
Adj transit(const Adj& h2m, const Adj& m2l, int hd, int ld) {
  int md = ld + 1;
  int nmh = simplex_degree(hd, md), nlm = simplex_degree(md, ld),
      nlh = simplex_degree(hd, ld);
  LO nh = LO(h2m.ab2b.size() / (size_t)(nmh));
  Adj out;
  out.ab2b.resize((size_t)(nh) * nlh);
  if (ld == 1) out.codes.resize((size_t)(nh) * nlh);
  ORC_PARALLEL_FOR
  for (LO h = 0; h < nh; ++h) {
    for (int hl = 0; hl < nlh; ++hl) {
      UpT ut = up_template(hd, ld, hl, 0);
      int hm = ut.up, hml = ut.which_down;
      LO m = h2m.ab2b[(size_t)(h) * nmh + hm];
      I8 m2hm_code = h2m.codes[(size_t)(h) * nmh + hm];
      I8 hm2m_code = invert_alignment(nlm, m2hm_code);
      int ml = align_index(nlm, ld, hml, hm2m_code);
      LO l = m2l.ab2b[(size_t)(m) * nlm + ml];
      out.ab2b[(size_t)(h) * nlh + hl] = l;
      if (ld == 1) {
        I8 fe_code = m2l.codes[(size_t)(m) * nlm + ml];
        bool ref = code_is_flipped(hm2m_code) ^ (code_rotation(fe_code) == 1) ^
                   ut.is_flipped;
        out.codes[(size_t)(h) * nlh + hl] = make_code(false, ref, 0);
      }
    }
  }
  return out;
}

// stars and dual (src/Omega_h_adj.cpp:512-657, src/Omega_h_graph.cpp:14-40)
static Adj verts_across_edges(const Adj& e2v, const Adj& v2e) {
  Adj g;
  g.a2ab = v2e.a2ab;
  g.ab2b.resize(v2e.ab2b.size());
  for (size_t ve = 0; ve < v2e.ab2b.size(); ++ve) {
    LO e = v2e.ab2b[ve];
    int eev = code_which_down(v2e.codes[ve]);
    g.ab2b[ve] = e2v.ab2b[(size_t)(e) * 2 + (1 - eev)];
  }
  return g;
}
static Adj edges_across_tris(const Adj& f2e, const Adj& e2f) {
  LO ne = LO(e2f.a2ab.size() - 1);
  Adj g;
  g.a2ab.assign((size_t)(ne) + 1, 0);
  for (LO e = 0; e < ne; ++e) g.a2ab[e + 1] = g.a2ab[e] + 2 * (e2f.a2ab[e + 1] - e2f.a2ab[e]);
  g.ab2b.resize((size_t)(g.a2ab[ne]));
  for (LO e = 0; e < ne; ++e) {
    LO k = g.a2ab[e];
    for (LO ef = e2f.a2ab[e]; ef < e2f.a2ab[e + 1]; ++ef) {
      LO f = e2f.ab2b[ef];
      int ffe = code_which_down(e2f.codes[ef]);
      g.ab2b[k++] = f2e.ab2b[(size_t)(f) * 3 + (ffe + 1) % 3];
      g.ab2b[k++] = f2e.ab2b[(size_t)(f) * 3 + (ffe + 2) % 3];
    }
  }
  return g;
}
static Adj edges_across_tets(const Adj& r2e, const Adj& e2r) {
  Adj g;
  g.a2ab = e2r.a2ab;
  g.ab2b.resize(e2r.ab2b.size());
  for (size_t er = 0; er < e2r.ab2b.size(); ++er) {
    LO r = e2r.ab2b[er];
    int rre = code_which_down(e2r.codes[er]);
    g.ab2b[er] = r2e.ab2b[(size_t)(r) * 6 + opposite_template(3, 1, rre)];
  }
  return g;
}
static Adj add_edges(const Adj& g1, const Adj& g2) {
  LO nv = LO(g1.a2ab.size() - 1);
  Adj g;
  g.a2ab.assign((size_t)(nv) + 1, 0);
  for (LO v = 0; v < nv; ++v)
    g.a2ab[v + 1] = g.a2ab[v] + (g1.a2ab[v + 1] - g1.a2ab[v]) + (g2.a2ab[v + 1] - g2.a2ab[v]);
  g.ab2b.resize((size_t)(g.a2ab[nv]));
  for (LO v = 0; v < nv; ++v) {
    LO k = g.a2ab[v];
    for (LO j = g1.a2ab[v]; j < g1.a2ab[v + 1]; ++j) g.ab2b[k++] = g1.ab2b[j];
    for (LO j = g2.a2ab[v]; j < g2.a2ab[v + 1]; ++j) g.ab2b[k++] = g2.ab2b[j];
  }
  return g;
}
static Adj elements_across_sides(int dim, const Adj& e2s, const Adj& s2e,
                                 const V<I8>& exposed) {
  int nse = dim + 1;
  LO ne = LO(e2s.ab2b.size() / (size_t)(nse));
  Adj g;
  g.a2ab.assign((size_t)(ne) + 1, 0);
  for (LO e = 0; e < ne; ++e) {
    int n = 0;
    for (int k = 0; k < nse; ++k)
      if (!exposed[e2s.ab2b[(size_t)(e) * nse + k]]) ++n;
    g.a2ab[e + 1] = g.a2ab[e] + n;
  }
  g.ab2b.resize((size_t)(g.a2ab[ne]));
  for (LO e = 0; e < ne; ++e) {
    LO k = g.a2ab[e];
    for (int j = 0; j < nse; ++j) {
      LO s = e2s.ab2b[(size_t)(e) * nse + j];
      if (!exposed[s]) {
        LO se = s2e.a2ab[s];
        if (s2e.ab2b[se] == e) ++se;
        g.ab2b[k++] = s2e.ab2b[se];
      }
    }
  }
  return g;
}

// Mesh::derive_adj (src/Omega_h_mesh.cpp:307-345)
const Adj& Mesh::ask_adj(int from, int to) {
  auto it = adj.find({from, to});
  if (it != adj.end()) return it->second;
  Adj d;
  if (from < to) {
    d = invert_adj(ask_adj(to, from), simplex_degree(to, from), nents[from]);
  } else if (to < from) {
    OCHECK(to + 1 < from);
    const Adj& h2m = ask_adj(from, to + 1);
    const Adj& m2l = ask_adj(to + 1, to);
    d = transit(h2m, m2l, from, to);
  } else if (from == dim) {
    const Adj& s2e = ask_adj(dim - 1, dim);
    V<I8> exposed((size_t)(nents[dim - 1]));
    for (LO s = 0; s < nents[dim - 1]; ++s)
      exposed[s] = (s2e.a2ab[s + 1] - s2e.a2ab[s]) < 2;
    d = elements_across_sides(dim, ask_adj(dim, dim - 1), s2e, exposed);
  } else if (from == VERT) {
    d = verts_across_edges(ask_adj(EDGE, VERT), ask_adj(VERT, EDGE));
  } else {
    OCHECK(from == EDGE);
    d = edges_across_tris(ask_adj(FACE, EDGE), ask_adj(EDGE, FACE));
    if (dim == 3) d = add_edges(d, edges_across_tets(ask_adj(REGION, EDGE), ask_adj(EDGE, REGION)));
  }
  return adj[{from, to}] = std::move(d);
}

// ------------------------------------------------------------ sort / unique
template <class T>
static V<LO> sort_keys_t(const V<T>& keys, int w) {
  LO n = LO(keys.size() / (size_t)(w));
  V<LO> perm((size_t)(n));
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](LO a, LO b) {
    for (int i = 0; i < w; ++i) {
      T x = keys[(size_t)(a) * w + i], y = keys[(size_t)(b) * w + i];
      if (x != y) return x < y;
    }
    return false;
  });
  return perm;
}
V<LO> sort_by_keys(const V<LO>& keys, int w) { return sort_keys_t(keys, w); }
V<LO> sort_by_keys64(const V<GO>& keys, int w) { return sort_keys_t(keys, w); }

// find_unique (src/Omega_h_adj.cpp:68-153): the last use of each run of
// equal canonical vertex tuples is kept, in its own (non-canonical) order
V<LO> find_unique(const V<LO>& hv2v, int hd, int ld) {
  V<LO> uv2v = form_uses(hv2v, hd, ld);
  int deg = ld + 1;
  LO nu = LO(uv2v.size() / (size_t)(deg));
  V<LO> canon(uv2v.size());
  for (LO u = 0; u < nu; ++u) {
    const LO* in = &uv2v[(size_t)(u) * deg];
    int min_j = 0;
    LO min_v = in[0];
    for (int j = 1; j < deg; ++j)
      if (in[j] < min_v) {
        min_j = j;
        min_v = in[j];
      }
    int rot = rotation_to_first(deg, min_j);
    LO tmp[4];
    for (int j = 0; j < deg; ++j) tmp[rotate_index(deg, j, rot)] = in[j];
    bool flipped = (deg == 3) ? (tmp[2] < tmp[1]) : false;
    // align_adj: rotate, then flip
    LO* out = &canon[(size_t)(u) * deg];
    for (int j = 0; j < deg; ++j) out[rotate_index(deg, j, rot)] = in[j];
    if (flipped && deg == 3) std::swap(out[1], out[2]);
  }
  V<LO> sorted2u = sort_by_keys(canon, deg);
  V<I8> jumps((size_t)(nu), 0);
  for (LO s = 0; s + 1 < nu; ++s) {
    LO e0 = sorted2u[s], e1 = sorted2u[s + 1];
    for (int j = 0; j < deg; ++j)
      if (canon[(size_t)(e0) * deg + j] != canon[(size_t)(e1) * deg + j]) {
        jumps[s] = 1;
        break;
      }
  }
  if (nu) jumps[nu - 1] = 1;
  V<LO> out;
  for (LO s = 0; s < nu; ++s)
    if (jumps[s])
      for (int j = 0; j < deg; ++j) out.push_back(uv2v[(size_t)(sorted2u[s]) * deg + j]);
  return out;
}

static void add_ents2verts(Mesh& m, int d, const V<LO>& ev2v) {
  if (d == 1) {
    Adj a;
    a.ab2b = ev2v;
    m.set_ents(1, std::move(a));
  } else {
    const V<LO>& lv2v = m.ask_verts_of(d - 1);
    const Adj& v2l = m.ask_up(0, d - 1);
    m.set_ents(d, reflect_down(ev2v, lv2v, v2l, d, d - 1));
  }
}

Mesh build_from_elems2verts(int dim, const V<LO>& ev2v, LO nverts) {
  Mesh m;
  m.dim = dim;
  m.nents[0] = nverts;
  for (int md = 1; md < dim; ++md) add_ents2verts(m, md, find_unique(ev2v, dim, md));
  add_ents2verts(m, dim, ev2v);
  return m;
}

// ------------------------------------------------------------ Hilbert
// Skilling's transform (src/Omega_h_hilbert.hpp:39-107)
typedef std::uint64_t coord_t;
static void axes_to_transpose(coord_t* X, int b, int n) {
  coord_t M = coord_t(1) << (b - 1), P, Q, t;
  for (Q = M; Q > 1; Q >>= 1) {
    P = Q - 1;
    for (int i = 0; i < n; i++) {
      if (X[i] & Q)
        X[0] ^= P;
      else {
        t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < n; i++) X[i] ^= X[i - 1];
  t = 0;
  for (Q = M; Q > 1; Q >>= 1)
    if (X[n - 1] & Q) t ^= Q - 1;
  for (int i = 0; i < n; i++) X[i] ^= t;
}
static void untranspose(const coord_t* in, coord_t* out, int b, int n) {
  for (int i = 0; i < n; ++i) out[i] = 0;
  for (int i = 0; i < (b * n); ++i)
    out[i / b] |= (((in[i % n] >> (b - 1 - (i / n))) & 1) << (b - 1 - (i % b)));
}

V<GO> hilbert_keys(const V<double>& coords, int dim) {
  LO n = LO(coords.size() / (size_t)(dim));
  double mn[3], mx[3];
  for (int j = 0; j < dim; ++j) {
    mn[j] = DBL_MAX;
    mx[j] = -DBL_MAX;
  }
  for (LO i = 0; i < n; ++i)
    for (int j = 0; j < dim; ++j) {
      double x = coords[(size_t)(i) * dim + j];
      mn[j] = min2(mn[j], x);
      mx[j] = max2(mx[j], x);
    }
  double maxl = mx[0] - mn[0];
  for (int j = 1; j < dim; ++j) maxl = max2(maxl, mx[j] - mn[j]);
  double s[3], t[3];
  for (int j = 0; j < dim; ++j) {
    mx[j] = mn[j] + maxl;
    s[j] = 1.0 / (mx[j] - mn[j]);
  }
  for (int j = 0; j < dim; ++j) t[j] = -(s[j] * mn[j]);
  const int nbits = 52;
  V<GO> keys((size_t)(n) * dim);
  for (LO i = 0; i < n; ++i) {
    coord_t X[3], Y[3];
    for (int j = 0; j < dim; ++j) {
      double u = s[j] * coords[(size_t)(i) * dim + j];
      u = u + t[j];
      double z = clampd(u, 0.0, 1.0) * std::exp2(double(nbits));
      X[j] = coord_t(z);
      if (X[j] >= (coord_t(1) << nbits)) X[j] = (coord_t(1) << nbits) - 1;
    }
    axes_to_transpose(X, nbits, dim);
    untranspose(X, Y, nbits, dim);
    for (int j = 0; j < dim; ++j) keys[(size_t)(i) * dim + j] = GO(Y[j]);
  }
  return keys;
}
V<LO> hilbert_sort(const V<double>& coords, int dim) {
  return sort_by_keys64(hilbert_keys(coords, dim), dim);
}

// reorder_by_hilbert + unmap_mesh (src/Omega_h_reorder.cpp:19-64,
// src/Omega_h_unmap_mesh.cpp:108-136)
void reorder_by_hilbert(Mesh& m) {
  int dim = m.dim;
  LO nv = m.nverts();
  V<LO> new2old[4];
  new2old[0] = hilbert_sort(m.coords, dim);
  for (int d = 1; d <= dim; ++d) {
    const V<LO>& ev2v = m.ask_verts_of(d);
    int deg = d + 1;
    LO ne = m.nents[d];
    V<LO> e2fv((size_t)(ne));
    for (LO e = 0; e < ne; ++e) e2fv[e] = ev2v[(size_t)(e) * deg];
    // invert_map_by_sorting: entities of each first vertex in index order
    V<LO> perm = sort_by_keys(e2fv, 1);
    V<LO> fv2e_off((size_t)(nv) + 1, 0);
    for (LO e = 0; e < ne; ++e) fv2e_off[e2fv[e] + 1]++;
    for (LO v = 0; v < nv; ++v) fv2e_off[v + 1] += fv2e_off[v];
    for (LO nvi = 0; nvi < nv; ++nvi) {
      LO ov = new2old[0][nvi];
      for (LO k = fv2e_off[ov]; k < fv2e_off[ov + 1]; ++k) new2old[d].push_back(perm[k]);
    }
  }
  Mesh nm;
  nm.dim = dim;
  nm.nents[0] = nv;
  V<LO> old2new_low((size_t)(nv));
  for (LO i = 0; i < nv; ++i) old2new_low[new2old[0][i]] = i;
  nm.coords.resize(m.coords.size());
  for (LO i = 0; i < nv; ++i)
    for (int j = 0; j < dim; ++j)
      nm.coords[(size_t)(i) * dim + j] = m.coords[(size_t)(new2old[0][i]) * dim + j];
  for (int d = 1; d <= dim; ++d) {
    const Adj& od = m.ask_down(d, d - 1);
    int deg = simplex_degree(d, d - 1);
    LO ne = m.nents[d];
    Adj nd;
    nd.ab2b.resize((size_t)(ne) * deg);
    if (!od.codes.empty()) nd.codes.resize((size_t)(ne) * deg);
    for (LO e = 0; e < ne; ++e)
      for (int k = 0; k < deg; ++k) {
        nd.ab2b[(size_t)(e) * deg + k] = old2new_low[od.ab2b[(size_t)(new2old[d][e]) * deg + k]];
        if (!od.codes.empty()) nd.codes[(size_t)(e) * deg + k] = od.codes[(size_t)(new2old[d][e]) * deg + k];
      }
    nm.set_ents(d, std::move(nd));
    V<LO> o2n((size_t)(ne));
    for (LO i = 0; i < ne; ++i) o2n[new2old[d][i]] = i;
    old2new_low = std::move(o2n);
  }
  m = std::move(nm);
}

// classify_box (src/Omega_h_box.cpp:105-160)
void classify_box(Mesh& m, int n) {
  int dim = m.dim;
  double dist = 1.0 / double(n * 32);
  for (int d = 0; d <= dim; ++d) {
    LO ne = m.nents[d];
    V<double> cen((size_t)(ne) * dim);
    if (d == 0) {
      cen = m.coords;
    } else {
      const V<LO>& ev2v = m.ask_verts_of(d);
      int deg = d + 1;
      for (LO e = 0; e < ne; ++e)
        for (int j = 0; j < dim; ++j) {
          double comp = 0;
          for (int k = 0; k < deg; ++k) comp += m.coords[(size_t)(ev2v[(size_t)(e) * deg + k]) * dim + j];
          comp /= deg;
          cen[(size_t)(e) * dim + j] = comp;
        }
    }
    m.class_id[d].resize((size_t)(ne));
    m.class_dim[d].resize((size_t)(ne));
    for (LO i = 0; i < ne; ++i) {
      int id = 0, cd = 0;
      for (int j = dim - 1; j >= 0; --j) {
        id *= 3;
        double x = cen[(size_t)(i) * dim + j];
        if (x > (1.0 - dist)) {
          id += 2;
        } else if (x > dist) {
          id += 1;
          ++cd;
        }
      }
      m.class_id[d][i] = id;
      m.class_dim[d][i] = I8(cd);
    }
  }
}

// tets_from_hexes, case analysis of Dompierre et al. (src/Omega_h_simplify.cpp:20-230)
static const int htv2hhv_0[5][4] = {{0, 1, 2, 5}, {0, 2, 7, 5}, {0, 2, 3, 7}, {0, 5, 7, 4}, {2, 7, 5, 6}};
static const int htv2hhv_1[6][4] = {{0, 5, 7, 4}, {0, 1, 7, 5}, {1, 6, 7, 5}, {0, 7, 2, 3}, {0, 7, 1, 2}, {1, 7, 6, 2}};
static const int htv2hhv_2[6][4] = {{0, 4, 5, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 1, 2, 5}, {0, 3, 6, 2}, {0, 6, 5, 2}};
static const int htv2hhv_3[6][4] = {{0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 5, 6, 4}, {1, 5, 6, 0}, {1, 6, 2, 0}};
static const int hex_flip_pairs[4][2] = {{0, 4}, {3, 5}, {1, 7}, {2, 6}};
static const int hex_bur_faces[3][4] = {{6, 5, 1, 2}, {6, 2, 3, 7}, {6, 7, 4, 5}};
static const int hex_bur_ring[6] = {1, 2, 3, 7, 5, 4};
// the reference's rot() shifts forward in place (each slot copies its
// predecessor's already-updated value); kept as is
static void rot_once(LO* v, int n) {
  LO tmp = v[n - 1];
  for (int i = 0; i < n - 1; ++i) v[i + 1] = v[i];
  v[0] = tmp;
}
static void rot_ntimes(LO* v, int n, int k) {
  for (int i = 0; i < k; ++i) rot_once(v, n);
}
static void rot_to_first(LO* v, int n, int first) { rot_ntimes(v, n, (n - first) % n); }
static bool lt4(LO a, LO b, LO c, LO d) { return std::min(a, b) < std::min(c, d); }

static V<LO> tets_from_hexes(const V<LO>& hv2v) {
  LO nh = LO(hv2v.size() / 8);
  V<LO> tv2v;
  tv2v.reserve((size_t)(nh) * 24);
  for (LO h = 0; h < nh; ++h) {
    LO hh[8];
    for (int i = 0; i < 8; ++i) hh[i] = hv2v[(size_t)(h) * 8 + i];
    int min_i = 0;
    for (int i = 1; i < 8; ++i)
      if (hh[i] < hh[min_i]) min_i = i;
    rot_to_first(hh + 0, 4, min_i % 4);
    rot_to_first(hh + 4, 4, min_i % 4);
    if (min_i >= 4)
      for (int i = 0; i < 4; ++i) std::swap(hh[hex_flip_pairs[i][0]], hh[hex_flip_pairs[i][1]]);
    int di[3];
    for (int i = 0; i < 3; ++i)
      di[i] = lt4(hh[hex_bur_faces[i][0]], hh[hex_bur_faces[i][2]], hh[hex_bur_faces[i][1]],
                  hh[hex_bur_faces[i][3]]);
    int nd = di[0] + di[1] + di[2];
    const int(*tmpl)[4] = htv2hhv_0;
    int nt = 5;
    if (nd > 0) {
      int face = -1;
      if (nd == 1) {
        for (int i = 0; i < 3; ++i)
          if (di[i]) face = i;
        tmpl = htv2hhv_1;
      } else if (nd == 2) {
        for (int i = 0; i < 3; ++i)
          if (!di[i]) face = i;
        tmpl = htv2hhv_2;
      } else {
        tmpl = htv2hhv_3;
      }
      nt = 6;
      if (face >= 0) {
        LO tmp[6];
        for (int i = 0; i < 6; ++i) tmp[i] = hh[hex_bur_ring[i]];
        rot_ntimes(tmp, 6, ((3 - face) % 3) * 2);
        for (int i = 0; i < 6; ++i) hh[hex_bur_ring[i]] = tmp[i];
      }
    }
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < 4; ++j) tv2v.push_back(hh[tmpl[i][j]]);
  }
  return tv2v;
}

// build_box (src/Omega_h_build.cpp:136-149) on the unit square/cube
Mesh build_box(int dim, int n) {
  V<LO> ev2v;
  V<double> coords;
  LO nv;
  if (dim == 3) {
    LO nvx = n + 1, nvxy = nvx * nvx;
    nv = nvxy * nvx;
    double dx = 1.0 / n;
    coords.resize((size_t)(nv) * 3);
    for (LO v = 0; v < nv; ++v) {
      LO ij = v % nvxy, k = v / nvxy, i = ij % nvx, j = ij / nvx;
      coords[(size_t)(v) * 3 + 0] = i * dx;
      coords[(size_t)(v) * 3 + 1] = j * dx;
      coords[(size_t)(v) * 3 + 2] = k * dx;
    }
    LO nxy = n * n, nhex = nxy * n;
    V<LO> hv2v((size_t)(nhex) * 8);
    for (LO h = 0; h < nhex; ++h) {
      LO ij = h % nxy, k = h / nxy, i = ij % n, j = ij / n;
      LO* o = &hv2v[(size_t)(h) * 8];
      o[0] = (k + 0) * nvxy + (j + 0) * nvx + (i + 0);
      o[1] = (k + 0) * nvxy + (j + 0) * nvx + (i + 1);
      o[2] = (k + 0) * nvxy + (j + 1) * nvx + (i + 1);
      o[3] = (k + 0) * nvxy + (j + 1) * nvx + (i + 0);
      o[4] = (k + 1) * nvxy + (j + 0) * nvx + (i + 0);
      o[5] = (k + 1) * nvxy + (j + 0) * nvx + (i + 1);
      o[6] = (k + 1) * nvxy + (j + 1) * nvx + (i + 1);
      o[7] = (k + 1) * nvxy + (j + 1) * nvx + (i + 0);
    }
    ev2v = tets_from_hexes(hv2v);
  } else {
    // make_2d_box + tris_from_quads (src/Omega_h_box.cpp:25-54,
    // src/Omega_h_simplify.cpp:121-142)
    LO nvx = n + 1;
    nv = nvx * nvx;
    double dx = 1.0 / n;
    coords.resize((size_t)(nv) * 2);
    for (LO v = 0; v < nv; ++v) {
      LO i = v % nvx, j = v / nvx;
      coords[(size_t)(v) * 2 + 0] = i * dx;
      coords[(size_t)(v) * 2 + 1] = j * dx;
    }
    LO nq = n * n;
    for (LO q = 0; q < nq; ++q) {
      LO i = q % n, j = q / n;
      LO qq[4] = {(j + 0) * nvx + (i + 0), (j + 0) * nvx + (i + 1),
                  (j + 1) * nvx + (i + 1), (j + 1) * nvx + (i + 0)};
      int min_i = 0;
      for (int k = 1; k < 4; ++k)
        if (qq[k] < qq[min_i]) min_i = k;
      rot_to_first(qq, 4, min_i);
      static const int qt[2][3] = {{0, 1, 2}, {2, 3, 0}};
      for (int t = 0; t < 2; ++t)
        for (int k = 0; k < 3; ++k) ev2v.push_back(qq[qt[t][k]]);
    }
  }
  Mesh m = build_from_elems2verts(dim, ev2v, nv);
  m.coords = coords;
  reorder_by_hilbert(m);
  classify_box(m, n);
  return m;
}

// ------------------------------------------------------------ measurement
const V<double>& Mesh::ask_lengths() {
  if (!has_length) {
    V<LO> all((size_t)(nedges()));
    std::iota(all.begin(), all.end(), 0);
    length = measure_edges_metric(*this, all);
    has_length = true;
  }
  return length;
}
const V<double>& Mesh::ask_qualities() {
  if (!has_quality) {
    V<LO> all((size_t)(nelems()));
    std::iota(all.begin(), all.end(), 0);
    quality = measure_qualities(*this, all);
    has_quality = true;
  }
  return quality;
}

V<double> measure_edges_metric(Mesh& m, const V<LO>& a2e) {
  const V<LO>& ev2v = m.ask_verts_of(1);
  int dim = m.dim, mc = m.mcomp();
  V<double> out(a2e.size());
  ORC_PARALLEL_FOR
  for (size_t a = 0; a < a2e.size(); ++a) {
    LO e = a2e[a];
    LO v0 = ev2v[(size_t)(e) * 2], v1 = ev2v[(size_t)(e) * 2 + 1];
    const double* p0 = &m.coords[(size_t)(v0) * dim];
    const double* p1 = &m.coords[(size_t)(v1) * dim];
    const double* m0 = &m.metric[(size_t)(v0) * mc];
    const double* m1 = &m.metric[(size_t)(v1) * mc];
    out[a] = dim == 3 ? edge_length3(p0, p1, m0, m1) : edge_length2(p0, p1, m0, m1);
  }
  return out;
}

double elem_quality(Mesh& m, const LO* v) {
  if (m.dim == 3) {
    Vec3 p[4];
    Mat3 ms[4];
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j < 3; ++j) p[i][j] = m.coords[(size_t)(v[i]) * 3 + j];
      ms[i] = symm3(&m.metric[(size_t)(v[i]) * 6]);
    }
    return tet_quality(p, maxdet3(ms, 4));
  }
  Vec2 p[3];
  Mat2 ms[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 2; ++j) p[i][j] = m.coords[(size_t)(v[i]) * 2 + j];
    ms[i] = symm2(&m.metric[(size_t)(v[i]) * 3]);
  }
  return tri_quality(p, maxdet2(ms, 3));
}

V<double> measure_qualities(Mesh& m, const V<LO>& a2e) {
  const V<LO>& ev2v = m.ask_verts_of(m.dim);
  int deg = m.dim + 1;
  V<double> out(a2e.size());
  ORC_PARALLEL_FOR
  for (size_t a = 0; a < a2e.size(); ++a) out[a] = elem_quality(m, &ev2v[(size_t)(a2e[a]) * deg]);
  return out;
}

V<double> get_mident_metrics(Mesh& m, const V<LO>& edges) {
  const V<LO>& ev2v = m.ask_verts_of(1);
  int mc = m.mcomp();
  V<double> out(edges.size() * (size_t)(mc));
  ORC_PARALLEL_FOR
  for (size_t a = 0; a < edges.size(); ++a) {
    LO e = edges[a];
    const double* m0 = &m.metric[(size_t)(ev2v[(size_t)(e) * 2]) * mc];
    const double* m1 = &m.metric[(size_t)(ev2v[(size_t)(e) * 2 + 1]) * mc];
    if (m.dim == 3)
      average_metric3(m0, m1, &out[a * mc]);
    else
      average_metric2(m0, m1, &out[a * mc]);
  }
  return out;
}

AdaptOpts::AdaptOpts(int dim) {
  min_length_desired = 1.0 / std::sqrt(2.0);
  max_length_desired = std::sqrt(2.0);
  max_length_allowed = max_length_desired * 2.0;
  if (dim == 3) {
    min_quality_allowed = 0.20;
    min_quality_desired = 0.30;
  } else {
    min_quality_allowed = 0.30;
    min_quality_desired = 0.40;
  }
  nsliver_layers = 4;
}

}  // namespace orc
