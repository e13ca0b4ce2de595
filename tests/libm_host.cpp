// The library's correctly rounded elementary functions (ohg_libm.cuh)
// compiled for the host, with glibc's for comparison, over arrays: built and
// called by tests/test_libm_cr.py.
#include <cmath>

#include "../omega_h_gb300/csrc/ohg_libm.cuh"

#define OHG_LIBM_HOST_N(name, expr)                                              \
  extern "C" void name(const double* x, double* y, long n) {                    \
    for (long i = 0; i < n; ++i) y[i] = expr(x[i]);                             \
  }
OHG_LIBM_HOST_N(cbrt_cr_n, ohg::cbrt_cr)
OHG_LIBM_HOST_N(log_cr_n, ohg::log_cr)
OHG_LIBM_HOST_N(exp_cr_n, ohg::exp_cr)
OHG_LIBM_HOST_N(cos_cr_n, ohg::cos_cr)
OHG_LIBM_HOST_N(acos_cr_n, ohg::acos_cr)
OHG_LIBM_HOST_N(cbrt_glibc_n, std::cbrt)
OHG_LIBM_HOST_N(log_glibc_n, std::log)
OHG_LIBM_HOST_N(exp_glibc_n, std::exp)
OHG_LIBM_HOST_N(cos_glibc_n, std::cos)
OHG_LIBM_HOST_N(acos_glibc_n, std::acos)
