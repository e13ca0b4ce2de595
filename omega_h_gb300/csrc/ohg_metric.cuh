// Metric tools (src/Omega_h_metric.cpp, src/Omega_h_metric_input.cpp):
// device arrays in, device arrays out.  Metrics are packed symmetric
// tensors, (xx, yy, zz, yx, zy, zx) in 3D and (xx, yy, yx) in 2D.
#pragma once
#include <vector>

#include "ohg_mesh.cuh"

namespace ohg {

// Omega_h_Source, Omega_h_Isotropy, Omega_h_Scales (src/Omega_h_defines.hpp)
enum MetricSourceType { MS_CONSTANT = 0, MS_VARIATION, MS_DERIVATIVE, MS_GIVEN, MS_IMPLIED,
                        MS_CURVATURE };
enum MetricIsotropy { MI_ANISOTROPIC = 0, MI_ISO_LENGTH, MI_ISO_SIZE };
enum MetricScales { MSC_ABSOLUTE = 0, MSC_SCALES };

struct MetricSource {
  int type = MS_CONSTANT;
  double knob = 1.0;
  int isotropy = MI_ANISOTROPIC;
  int scales = MSC_SCALES;
  const double* given = nullptr;  // MS_GIVEN: device array of packed metrics
};

// MetricInput (src/Omega_h_metric_input.cpp:23-35 defaults)
struct MetricInput {
  std::vector<MetricSource> sources;
  bool limit_lengths = false;
  double min_length = 0.0, max_length = 0.0;
  bool limit_gradation = false;
  double max_gradation_rate = 1.0, gradation_tol = 1e-3;
  bool limit_element_count = false;
  double max_element_count = 1e6, min_element_count = 1.0, element_count_over_relaxation = 1.1;
  int nsmoothing_steps = 0;
};

void cubic_roots_batch(LO n, const double* coeffs, double eps, int* nroots, double* roots,
                       int* mults);
void decompose_eigen_batch(int dim, LO n, const double* m, double* q, double* l);
void intersect_metrics(int dim, LO n, const double* a, const double* b, double* out);
void clamp_metrics(int dim, LO n, const double* m, double h_min, double h_max, double* out);
void hessian_metrics(int dim, LO n, const double* hessians, double eps, double* out);
Arr<double> implied_metrics(Mesh& m);
Arr<double> limit_metric_gradation(Mesh& m, const Arr<double>& v2m, double max_rate, double tol,
                                   int* steps);
double expected_nelems(Mesh& m, const double* v2m);
Arr<double> generate_metrics(Mesh& m, const MetricInput& in, int* niters);

}  // namespace ohg
