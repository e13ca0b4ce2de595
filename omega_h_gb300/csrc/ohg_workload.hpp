// Synthetic adapt-pass workloads: seeded vertex jitter and analytic metric
// fields on box meshes.  Header-only plain C++ (no CUDA), so the same
// definition drives the GPU library's input builder and any host program
// that must construct bit-identical inputs.
//
// Metric storage follows the reference's symmetric packing
// (src/Omega_h_matrix.hpp:408-432): 3D (xx, yy, zz, yx, zy, zx),
// 2D (xx, yy, yx).
#pragma once
#include <cmath>
#include <cstdint>

namespace ohg {
namespace workload {

enum MetricKind : int {
  METRIC_ISO_LINEAR = 0,  // h = 0.05 + 0.1*|x0 - 0.5|, M = I/h^2
  METRIC_SHOCK = 1,       // anisotropic shock across a rotated plane
  METRIC_BOUNDARY = 2,    // boundary layer at y = 0
  METRIC_ISO_SINE = 3,    // h = h0*(1 + a*sin(2*pi*k.x)), M = I/h^2
};

// kind + kScalarKind: an isotropic field stored as one scalar per vertex,
// as the reference stores an isotropic metric (a tag of one component);
// only for the isotropic kinds
constexpr int kScalarKind = 10;
inline bool scalar_kind(int kind) { return kind >= kScalarKind; }
inline int base_kind(int kind) { return kind >= kScalarKind ? kind - kScalarKind : kind; }

struct MetricParams {
  int kind = METRIC_ISO_LINEAR;
  // shock: unit normal of the rotated plane through (0.5,0.5,0.5)
  double normal[3] = {0.0, 0.0, 1.0};
  // iso sine
  double h0 = 0.1, amp = 0.0;
  double k[3] = {1.0, 1.0, 1.0};
};

// splitmix64 finaliser: a bijective 64-bit mixer (Steele, Lea, Flood 2014).
inline std::uint64_t mix64(std::uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// uniform double in [0,1) from (seed, stream, index), 53 random bits
inline double uniform01(std::uint64_t seed, std::uint64_t stream,
                        std::uint64_t index) {
  std::uint64_t z = mix64(seed ^ mix64(stream * 0x632be59bd9b4e019ull + index));
  return double(z >> 11) * (1.0 / 9007199254740992.0);
}

// Jitter of one coordinate of an interior vertex: uniform in
// [-amp, +amp) where amp = 0.15 / n (n = subdivisions per axis).
inline double jitter(std::uint64_t seed, std::int64_t vert, int axis,
                     int dim, int n) {
  double u = uniform01(seed, 1, std::uint64_t(vert) * std::uint64_t(dim) +
                                    std::uint64_t(axis));
  double amp = 0.15 / double(n);
  return (2.0 * u - 1.0) * amp;
}

// Shock-plane normal: (1,1,1)/sqrt(3) rotated by an angle uniform in
// [0, 0.2] rad about a seeded unit axis (Rodrigues' formula).
inline void shock_normal(std::uint64_t seed, double out[3]) {
  const double s3 = 1.0 / std::sqrt(3.0);
  double n[3] = {s3, s3, s3};
  double theta = 0.2 * uniform01(seed, 2, 0);
  double z = 2.0 * uniform01(seed, 2, 1) - 1.0;
  double phi = 2.0 * 3.14159265358979323846 * uniform01(seed, 2, 2);
  double r = std::sqrt(1.0 - z * z);
  double a[3] = {r * std::cos(phi), r * std::sin(phi), z};
  double c = std::cos(theta), s = std::sin(theta);
  double axn[3] = {a[1] * n[2] - a[2] * n[1], a[2] * n[0] - a[0] * n[2],
                   a[0] * n[1] - a[1] * n[0]};
  double adn = a[0] * n[0] + a[1] * n[1] + a[2] * n[2];
  double len2 = 0.0;
  for (int i = 0; i < 3; ++i) {
    out[i] = n[i] * c + axn[i] * s + a[i] * adn * (1.0 - c);
    len2 += out[i] * out[i];
  }
  double inv = 1.0 / std::sqrt(len2);
  for (int i = 0; i < 3; ++i) out[i] *= inv;
}

// Parameters of a metric family from a seed: the shock normal, and for the
// isotropic sine field h0 uniform in [0.02, 0.2], a uniform in [0, 0.5] and
// k with integer components uniform in 1..4.
inline MetricParams make_params(int kind, std::uint64_t seed) {
  MetricParams p;
  p.kind = kind;
  if (kind == METRIC_SHOCK) shock_normal(seed, p.normal);
  if (kind == METRIC_ISO_SINE) {
    p.h0 = 0.02 + 0.18 * uniform01(seed, 3, 0);
    p.amp = 0.5 * uniform01(seed, 3, 1);
    for (int i = 0; i < 3; ++i) p.k[i] = 1.0 + std::floor(4.0 * uniform01(seed, 3, 2 + i));
  }
  return p;
}

// Writes the packed metric of one vertex at point x (dim components).
inline void metric_at(const MetricParams& p, int dim, const double* x,
                      double* m) {
  const int nc = dim == 3 ? 6 : 3;
  for (int i = 0; i < nc; ++i) m[i] = 0.0;
  if (p.kind == METRIC_ISO_LINEAR || p.kind == METRIC_ISO_SINE) {
    double h;
    if (p.kind == METRIC_ISO_LINEAR) {
      h = 0.05 + 0.1 * std::fabs(x[0] - 0.5);
    } else {
      double kx = 0.0;
      for (int i = 0; i < dim; ++i) kx += p.k[i] * x[i];
      h = p.h0 * (1.0 + p.amp * std::sin(2.0 * 3.14159265358979323846 * kx));
    }
    double l = 1.0 / (h * h);
    for (int i = 0; i < dim; ++i) m[i] = l;
    return;
  }
  if (p.kind == METRIC_SHOCK) {
    double d = 0.0;
    for (int i = 0; i < dim; ++i) d += p.normal[i] * (x[i] - 0.5);
    double hn = 0.002 + 0.198 * (1.0 - std::exp(-std::fabs(d) / 0.05));
    double ht = 0.05;
    double lt = 1.0 / (ht * ht);
    double ln = 1.0 / (hn * hn);
    double dl = ln - lt;
    const double* n = p.normal;
    if (dim == 3) {
      m[0] = lt + dl * n[0] * n[0];
      m[1] = lt + dl * n[1] * n[1];
      m[2] = lt + dl * n[2] * n[2];
      m[3] = dl * n[1] * n[0];
      m[4] = dl * n[2] * n[1];
      m[5] = dl * n[2] * n[0];
    } else {
      m[0] = lt + dl * n[0] * n[0];
      m[1] = lt + dl * n[1] * n[1];
      m[2] = dl * n[1] * n[0];
    }
    return;
  }
  // boundary layer: h_y = 1e-4 + 0.1*(1 - exp(-y/0.02)), h_x = h_z = 0.1
  double hy = 1e-4 + 0.1 * (1.0 - std::exp(-x[1] / 0.02));
  double hx = 0.1;
  m[0] = 1.0 / (hx * hx);
  m[1] = 1.0 / (hy * hy);
  if (dim == 3) m[2] = 1.0 / (hx * hx);
}

}  // namespace workload
}  // namespace ohg
