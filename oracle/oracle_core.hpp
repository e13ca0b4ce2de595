// ORACLE — test infrastructure only.  A serial CPU restatement of the
// reference (sandialabs/omega_h v9.34.13) algorithms on the per-pass adapt
// path.  Used by tests/ as the checker and by bench.py as the CPU baseline;
// never linked into, or called by, the GPU product.
//
// Floating-point expressions keep the reference's evaluation order so that,
// compiled with -ffp-contract=off, every +,-,*,/,sqrt result is identical to
// the reference's; only libm (log, exp, cbrt, acos, cos) may differ by an ulp
// between platforms.
#pragma once
#include <cstdint>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../omega_h_gb300/csrc/ohg_libm.cuh"

// Independent per-entity loops run on all host threads when built with
// OpenMP, as the reference's parallel_for does in its OpenMP build; every
// iteration writes only its own outputs, so results do not depend on the
// thread count.  Lazily derived adjacencies are asked for before each loop.
#ifdef _OPENMP
#define ORC_PARALLEL_FOR _Pragma("omp parallel for schedule(dynamic, 512)")
#else
#define ORC_PARALLEL_FOR
#endif

namespace orc {

// The libm functions on the path.  Built with -DORC_CR_LIBM=<mask> (bits:
// 1 cbrt, 2 acos, 4 cos, 8 log, 16 exp) the selected ones are replaced by the
// library's correctly rounded functions (ohg_libm.cuh, the functions the GPU
// path calls).  Test infrastructure: with all five (mask 31) it is the
// reference's algorithm with the GPU path's elementary functions; with some
// of them it measures how the reference's results depend on the last ulp of
// each function.
#ifndef ORC_CR_LIBM
#define ORC_CR_LIBM 0
#endif
inline double orc_cbrt(double x) { return (ORC_CR_LIBM & 1) ? ohg::cbrt_cr(x) : std::cbrt(x); }
inline double orc_acos(double x) { return (ORC_CR_LIBM & 2) ? ohg::acos_cr(x) : std::acos(x); }
inline double orc_cos(double x) { return (ORC_CR_LIBM & 4) ? ohg::cos_cr(x) : std::cos(x); }
inline double orc_log(double x) { return (ORC_CR_LIBM & 8) ? ohg::log_cr(x) : std::log(x); }
inline double orc_exp(double x) { return (ORC_CR_LIBM & 16) ? ohg::exp_cr(x) : std::exp(x); }

typedef std::int32_t LO;
typedef std::int64_t GO;
typedef std::int8_t I8;
template <class T>
using V = std::vector<T>;

struct OracleError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
#define OCHECK(c)                                                          \
  do {                                                                     \
    if (!(c))                                                              \
      throw ::orc::OracleError(std::string("oracle check failed: ") + #c + \
                               " at " __FILE__ ":" + std::to_string(__LINE__)); \
  } while (0)

enum { VERT = 0, EDGE = 1, FACE = 2, REGION = 3 };

// ---------------------------------------------------------------- alignment
// src/Omega_h_align.hpp:44-110
inline bool code_is_flipped(I8 c) { return c & 1; }
inline int code_rotation(I8 c) { return (c >> 1) & 3; }
inline int code_which_down(I8 c) { return c >> 3; }
inline I8 make_code(bool f, int rot, int wd) {
  return I8((wd << 3) | (rot << 1) | int(f));
}
inline int rotate_index(int n, int i, int r) { return (i + r) % n; }
inline int invert_rotation(int n, int r) { return (n - r) % n; }
inline int reverse_index(int n, int i) { return n - 1 - i; }
inline int flip_vert_index(int n, int i) {
  return i == 0 ? 0 : (1 + reverse_index(n - 1, i - 1));
}
inline int align_vert_index(int n, int i, I8 c) {
  return code_is_flipped(c)
             ? flip_vert_index(n, rotate_index(n, i, code_rotation(c)))
             : rotate_index(n, i, code_rotation(c));
}
inline int align_edge_index(int n, int i, I8 c) {
  return code_is_flipped(c)
             ? reverse_index(n, rotate_index(n, i, code_rotation(c)))
             : rotate_index(n, i, code_rotation(c));
}
inline int align_index(int n, int idim, int i, I8 c) {
  return idim == 0 ? align_vert_index(n, i, c) : align_edge_index(n, i, c);
}
inline int rotation_to_first(int n, int f) { return invert_rotation(n, f); }
inline I8 invert_alignment(int n, I8 c) {
  return code_is_flipped(c) ? c
                            : make_code(false, invert_rotation(n, code_rotation(c)), 0);
}

// ---------------------------------------------------------------- templates
// src/Omega_h_simplex.hpp:23-300
inline int down_template(int ed, int bd, int wb, int wv) {
  static const int t32[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
  static const int t31[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  static const int t21[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  if (bd == 0) return wb;
  if (ed == 3 && bd == 2) return t32[wb][wv];
  if (ed == 3 && bd == 1) return t31[wb][wv];
  if (ed == 2 && bd == 1) return t21[wb][wv];
  return -1;
}
struct UpT {
  int up, which_down;
  bool is_flipped;
};
inline UpT up_template(int ed, int bd, int wb, int wu) {
  static const UpT t30[4][3] = {{{0, 0, 0}, {2, 1, 0}, {3, 0, 0}},
                                {{1, 0, 0}, {0, 1, 0}, {4, 0, 0}},
                                {{2, 0, 0}, {1, 1, 0}, {5, 0, 0}},
                                {{5, 1, 0}, {4, 1, 0}, {3, 1, 0}}};
  static const UpT t31[6][2] = {{{0, 2, 1}, {1, 0, 0}}, {{0, 1, 1}, {2, 0, 0}},
                                {{0, 0, 1}, {3, 0, 0}}, {{1, 2, 1}, {3, 1, 0}},
                                {{2, 2, 1}, {1, 1, 0}}, {{3, 2, 1}, {2, 1, 0}}};
  static const UpT t20[3][2] = {{{0, 0, 0}, {2, 1, 0}},
                                {{1, 0, 0}, {0, 1, 0}},
                                {{2, 0, 0}, {1, 1, 0}}};
  if (ed == 3 && bd == 0) return t30[wb][wu];
  if (ed == 3 && bd == 1) return t31[wb][wu];
  if (ed == 2 && bd == 0) return t20[wb][wu];
  return {-1, -1, false};
}
inline int opposite_template(int ed, int bd, int wb) {
  static const int t30[4] = {2, 3, 1, 0};
  static const int t31[6] = {5, 3, 4, 1, 2, 0};
  static const int t32[4] = {3, 2, 0, 1};
  static const int t20[3] = {1, 2, 0};
  static const int t21[3] = {2, 0, 1};
  if (ed == 3 && bd == 0) return t30[wb];
  if (ed == 3 && bd == 1) return t31[wb];
  if (ed == 3 && bd == 2) return t32[wb];
  if (ed == 2 && bd == 0) return t20[wb];
  if (ed == 2 && bd == 1) return t21[wb];
  if (ed == 1 && bd == 0) return 1 - wb;
  return -1;
}
inline int simplex_degree(int from, int to) {
  static const int t[4][4] = {{1, -1, -1, -1}, {2, 1, -1, -1}, {3, 3, 1, -1},
                              {4, 6, 4, 1}};
  return t[from][to];
}

// ---------------------------------------------------------------- math
// Vectors and column-major matrices with the reference's operation order
// (src/Omega_h_vector.hpp, src/Omega_h_matrix.hpp, src/Omega_h_few.hpp:138).
struct Vec3 {
  double v[3];
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
struct Mat3 {
  Vec3 c[3];  // columns
  Vec3& operator[](int j) { return c[j]; }
  const Vec3& operator[](int j) const { return c[j]; }
};
template <int n>
inline double dotn(const double* a, const double* b) {
  double out = a[0] * b[0];
  for (int i = 1; i < n; ++i) out = out + (a[i] * b[i]);
  return out;
}
inline Vec3 vsub(Vec3 a, Vec3 b) { return {{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
inline Vec3 vadd(Vec3 a, Vec3 b) { return {{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
inline Vec3 vscale(Vec3 a, double s) { return {{a[0] * s, a[1] * s, a[2] * s}}; }
inline Vec3 vdiv(Vec3 a, double s) { return {{a[0] / s, a[1] / s, a[2] / s}}; }
inline Vec3 vneg(Vec3 a) { return {{-a[0], -a[1], -a[2]}}; }
inline double dot3(Vec3 a, Vec3 b) { return dotn<3>(a.v, b.v); }
inline Vec3 cross3(Vec3 a, Vec3 b) {
  return {{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
           a[0] * b[1] - a[1] * b[0]}};
}
inline double norm3(Vec3 a) { return std::sqrt(dot3(a, a)); }
// matrix * vector: c = a[0]*b[0]; c = c + a[j]*b[j]  (src/Omega_h_matrix.hpp:89-94)
template <int n>
inline void matvec(const double* cols, const double* b, double* c) {
  for (int i = 0; i < n; ++i) c[i] = cols[0 * n + i] * b[0];
  for (int j = 1; j < n; ++j)
    for (int i = 0; i < n; ++i) c[i] = c[i] + cols[j * n + i] * b[j];
}
inline Vec3 mv3(const Mat3& a, Vec3 b) {
  Vec3 c;
  matvec<3>(&a.c[0].v[0], b.v, c.v);
  return c;
}
inline Mat3 mm3(const Mat3& a, const Mat3& b) {
  Mat3 c;
  for (int j = 0; j < 3; ++j) c[j] = mv3(a, b[j]);
  return c;
}
inline Mat3 transpose3(const Mat3& a) {
  Mat3 b;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) b[i][j] = a[j][i];
  return b;
}
inline double det3(const Mat3& m) {
  double a = m[0][0], b = m[1][0], c = m[2][0];
  double d = m[0][1], e = m[1][1], f = m[2][1];
  double g = m[0][2], h = m[1][2], i = m[2][2];
  return (a * e * i) + (b * f * g) + (c * d * h) - (c * e * g) - (b * d * i) -
         (a * f * h);
}
inline Mat3 symm3(const double* v) {
  Mat3 s;
  s[0][0] = v[0];
  s[1][1] = v[1];
  s[2][2] = v[2];
  s[1][0] = v[3];
  s[2][1] = v[4];
  s[2][0] = v[5];
  s[0][1] = s[1][0];
  s[1][2] = s[2][1];
  s[0][2] = s[2][0];
  return s;
}
inline void unsymm3(const Mat3& s, double* v) {
  v[0] = s[0][0];
  v[1] = s[1][1];
  v[2] = s[2][2];
  v[3] = s[1][0];
  v[4] = s[2][1];
  v[5] = s[2][0];
}
// metric_product(m, v) = v * (m * v)   (src/Omega_h_metric.hpp:8-11)
inline double metric_product3(const Mat3& m, Vec3 v) { return dot3(v, mv3(m, v)); }

// 2D versions
struct Vec2 {
  double v[2];
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
struct Mat2 {
  Vec2 c[2];
  Vec2& operator[](int j) { return c[j]; }
  const Vec2& operator[](int j) const { return c[j]; }
};
inline Vec2 mv2(const Mat2& a, Vec2 b) {
  Vec2 c;
  matvec<2>(&a.c[0].v[0], b.v, c.v);
  return c;
}
inline double det2(const Mat2& m) {
  double a = m[0][0], b = m[1][0], c = m[0][1], d = m[1][1];
  return a * d - b * c;
}
inline Mat2 symm2(const double* v) {
  Mat2 s;
  s[0][0] = v[0];
  s[1][1] = v[1];
  s[1][0] = v[2];
  s[0][1] = s[1][0];
  return s;
}

// quality / length (src/Omega_h_quality.hpp:8-36, src/Omega_h_shape.hpp:112-134)
const double EQUILATERAL_TET = 0.1178511301977579;
const double EQUILATERAL_TRI = 0.4330127018922193;

inline double anisotropic_edge_length(double la, double lb) {
  if (std::abs(la - lb) > 1e-3) return (la - lb) / (orc_log(la / lb));
  return (la + lb) / 2.;
}
inline double edge_length3(const double* p0, const double* p1, const double* m0,
                           const double* m1) {
  Vec3 v = {{p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]}};
  double la = std::sqrt(metric_product3(symm3(m0), v));
  double lb = std::sqrt(metric_product3(symm3(m1), v));
  return anisotropic_edge_length(la, lb);
}
inline double edge_length2(const double* p0, const double* p1, const double* m0,
                           const double* m1) {
  Vec2 v = {{p1[0] - p0[0], p1[1] - p0[1]}};
  Mat2 a = symm2(m0), b = symm2(m1);
  Vec2 av = mv2(a, v), bv = mv2(b, v);
  double la = std::sqrt(dotn<2>(v.v, av.v));
  double lb = std::sqrt(dotn<2>(v.v, bv.v));
  return anisotropic_edge_length(la, lb);
}
// metric_element_quality<3> with a full 3x3 metric
inline double tet_quality(const Vec3 p[4], const Mat3& m) {
  Vec3 b0 = vsub(p[1], p[0]), b1 = vsub(p[2], p[0]), b2 = vsub(p[3], p[0]);
  double rs = dot3(cross3(b0, b1), b2) / 6.0;
  double s = rs * std::sqrt(det3(m));
  if (s < 0) return s;
  Vec3 ev[6] = {b0, vsub(p[2], p[1]), vneg(b1), b2, vsub(p[3], p[1]),
                vsub(p[3], p[2])};
  double msl = 0;
  for (int i = 0; i < 6; ++i) msl += metric_product3(m, ev[i]);
  msl = msl / 6;
  double x = s / EQUILATERAL_TET;
  return orc_cbrt(x * x) / msl;
}
inline double tri_quality(const Vec2 p[3], const Mat2& m) {
  Vec2 b0 = {{p[1][0] - p[0][0], p[1][1] - p[0][1]}};
  Vec2 b1 = {{p[2][0] - p[0][0], p[2][1] - p[0][1]}};
  double rs = (b0[0] * b1[1] - b0[1] * b1[0]) / 2.0;
  // metric_size<2,2> = rs * power<2,4>(det) = rs * sqrt(det)
  double s = rs * std::sqrt(det2(m));
  if (s < 0) return s;
  Vec2 ev[3] = {b0, {{p[2][0] - p[1][0], p[2][1] - p[1][1]}}, {{-b1[0], -b1[1]}}};
  double msl = 0;
  for (int i = 0; i < 3; ++i) {
    Vec2 mv = mv2(m, ev[i]);
    msl += dotn<2>(ev[i].v, mv.v);
  }
  msl = msl / 3;
  double x = s / EQUILATERAL_TRI;
  // power<2,2>(x) = x
  return x / msl;
}
// maxdet_metric (src/Omega_h_metric.hpp:170-182): first max wins ties
inline Mat3 maxdet3(const Mat3* ms, int n) {
  Mat3 m = ms[0];
  double maxdet = det3(m);
  for (int i = 1; i < n; ++i) {
    double d = det3(ms[i]);
    if (d > maxdet) {
      m = ms[i];
      maxdet = d;
    }
  }
  return m;
}
inline Mat2 maxdet2(const Mat2* ms, int n) {
  Mat2 m = ms[0];
  double maxdet = det2(m);
  for (int i = 1; i < n; ++i) {
    double d = det2(ms[i]);
    if (d > maxdet) {
      m = ms[i];
      maxdet = d;
    }
  }
  return m;
}

// eigen decomposition and log/exp of SPD tensors (src/Omega_h_eigen.hpp)
Mat3 log_spd3(Mat3 m);
Mat3 exp_spd3(Mat3 m);
Mat2 log_spd2(Mat2 m);
Mat2 exp_spd2(Mat2 m);
void average_metric3(const double* m0, const double* m1, double* out);
void average_metric2(const double* m0, const double* m1, double* out);

// ---------------------------------------------------------------- mesh
struct Adj {
  V<LO> a2ab, ab2b;
  V<I8> codes;
};

struct Mesh {
  int dim = 3;
  LO nents[4] = {0, 0, 0, 0};
  V<double> coords;
  V<double> metric;  // symm_ncomps(dim) per vertex
  V<I8> class_dim[4];
  V<LO> class_id[4];
  bool has_length = false, has_quality = false;
  V<double> length, quality;
  std::map<std::pair<int, int>, Adj> adj;  // stored down adjacencies + cache

  int mcomp() const { return dim == 3 ? 6 : 3; }
  LO nverts() const { return nents[0]; }
  LO nedges() const { return nents[1]; }
  LO nelems() const { return nents[dim]; }
  void set_ents(int d, Adj down) {
    nents[d] = LO(down.ab2b.size() / size_t(simplex_degree(d, d - 1)));
    adj[{d, d - 1}] = std::move(down);
  }
  const Adj& ask_adj(int from, int to);
  const Adj& ask_down(int from, int to) { return ask_adj(from, to); }
  const Adj& ask_up(int from, int to) { return ask_adj(from, to); }
  const V<LO>& ask_verts_of(int d) { return ask_adj(d, 0).ab2b; }
  const V<double>& ask_lengths();
  const V<double>& ask_qualities();
};

struct AdaptOpts {
  double min_length_desired, max_length_desired, max_length_allowed;
  double min_quality_allowed, min_quality_desired;
  int nsliver_layers = 4;
  explicit AdaptOpts(int dim);
};

// adjacency (src/Omega_h_adj.cpp)
Adj invert_adj(const Adj& down, int nlows_per_high, LO nlows);
Adj reflect_down(const V<LO>& hv2v, const V<LO>& lv2v, const Adj& v2l,
                 int high_dim, int low_dim);
Adj transit(const Adj& h2m, const Adj& m2l, int high_dim, int low_dim);
V<LO> form_uses(const V<LO>& hv2v, int high_dim, int low_dim);
V<LO> find_unique(const V<LO>& hv2v, int high_dim, int low_dim);
V<LO> sort_by_keys(const V<LO>& keys, int width);
V<LO> sort_by_keys64(const V<GO>& keys, int width);

// mesh construction (src/Omega_h_build.cpp:107-149, src/Omega_h_box.cpp,
// src/Omega_h_simplify.cpp, src/Omega_h_reorder.cpp, src/Omega_h_hilbert.*)
Mesh build_from_elems2verts(int dim, const V<LO>& ev2v, LO nverts);
V<GO> hilbert_keys(const V<double>& coords, int dim);
V<LO> hilbert_sort(const V<double>& coords, int dim);
void reorder_by_hilbert(Mesh& m);
void classify_box(Mesh& m, int n);
Mesh build_box(int dim, int n);

// measurement (src/Omega_h_shape.cpp, src/Omega_h_quality.cpp,
// src/Omega_h_metric.cpp:56-104)
V<double> measure_edges_metric(Mesh& m, const V<LO>& a2e);
V<double> measure_qualities(Mesh& m, const V<LO>& a2e);
V<double> get_mident_metrics(Mesh& m, const V<LO>& edges);
double elem_quality(Mesh& m, const LO* v);

// primitives (src/Omega_h_map.cpp, src/Omega_h_int_scan.cpp)
template <class T>
V<LO> collect_marked(const V<T>& marks) {
  V<LO> out;
  for (size_t i = 0; i < marks.size(); ++i)
    if (marks[i]) out.push_back(LO(i));
  return out;
}
template <class T>
V<LO> offset_scan(const V<T>& a) {
  V<LO> out(a.size() + 1);
  out[0] = 0;
  for (size_t i = 0; i < a.size(); ++i) out[i + 1] = out[i] + LO(a[i]);
  return out;
}

// selection (src/Omega_h_indset.cpp, src/Omega_h_indset_inline.hpp)
V<I8> find_indset(const Adj& graph, const V<double>& quality,
                  const V<I8>& candidates, int* nrounds = nullptr);
V<I8> find_indset(Mesh& m, int ent_dim, const V<double>& quality,
                  const V<I8>& candidates);

// operators
V<double> refine_qualities(Mesh& m, const V<LO>& cands2edges);
bool refine_by_size(Mesh& m, const AdaptOpts& o);
bool coarsen_by_size(Mesh& m, const AdaptOpts& o);
bool swap_edges(Mesh& m, const AdaptOpts& o);
V<LO> get_rep2md_order_adapt(Mesh& m, int key_dim, int rep_dim,
                             const V<I8>& kds_are_keys);

// coarsen pieces (src/Omega_h_check_collapse.cpp, _overshoot, _qualities,
// src/Omega_h_collapse_rail.cpp)
V<I8> check_collapse_class(Mesh& m, const V<LO>& c2e, const V<I8>& codes);
V<I8> check_collapse_exposure(Mesh& m, const V<LO>& c2e, const V<I8>& codes);
V<I8> prevent_coarsen_overshoot(Mesh& m, double max_length, const V<LO>& c2e,
                                const V<I8>& codes);
V<double> coarsen_qualities(Mesh& m, const V<LO>& c2e, const V<I8>& codes);
void choose_rails(Mesh& m, const V<LO>& c2e, const V<I8>& codes,
                  const V<double>& quals, V<I8>* vc, V<double>* vq, V<GO>* vr);

void find_rails(Mesh& m, const V<LO>& k2v, const V<GO>& vr, V<LO>* r2e, V<I8>* rdir);
void mark_dead_ents(Mesh& m, const V<LO>& r2e, const V<I8>& rdir, V<I8>* dead);

// swap pieces
V<I8> mark_sliver_layers(Mesh& m, double qual_ceil, int nlayers);
void swap3d_qualities(Mesh& m, const AdaptOpts& o, const V<LO>& c2e,
                      V<double>* quals, V<I8>* configs);
V<I8> filter_swap_improve(Mesh& m, const V<LO>& c2e, const V<double>& quals);
V<double> swap2d_qualities(Mesh& m, const AdaptOpts& o, const V<LO>& c2e);

// the whole pass: refine -> coarsen -> swap (if min quality < desired)
struct PassResult {
  bool did_refine = false, did_coarsen = false, did_swap = false;
};
PassResult adapt_pass(Mesh& m, const AdaptOpts& o);

// coarsen_slivers and the full adapt() loop
bool coarsen_slivers(Mesh& m, const AdaptOpts& o);
struct AdaptResult {
  bool did = false, quality_satisfied = false;
  int refines = 0, coarsens = 0, swaps = 0, sliver_coarsens = 0, length_rounds = 0;
};
AdaptResult adapt(Mesh& m, const AdaptOpts& o);

// swap3d tables (same content as src/Omega_h_swap3d_tables.hpp, own layout)
namespace swap3d {
int mesh_count(int loop);
int mesh_size(int loop);
const int* triangle(int loop, int uniq_tri);
int mesh_tri(int loop, int mesh, int t);
int nedges(int loop);
const int* unique_edge(int loop, int ue);
int edge2unique(int loop, int mesh, int e);
}  // namespace swap3d

}  // namespace orc
