// Array primitives on device arrays: scans, compaction, reductions, stable
// radix sorts and gathers/scatters (the roles of src/Omega_h_int_scan.cpp,
// src/Omega_h_map.cpp, src/Omega_h_sort.cpp and src/Omega_h_reduce.hpp).
#pragma once
#include <cstring>
#include "ohg_common.cuh"

namespace ohg {

// exclusive prefix sum of counts, n+1 outputs (offset_scan,
// src/Omega_h_int_scan.cpp:10-20)
Arr<LO> offset_scan(const Arr<LO>& counts);
Arr<LO> offset_scan(const Arr<I8>& counts);
// same, into caller memory of n+1 entries
void offset_scan_into(const LO* counts, LO n, LO* out);
void offset_scan_into(const I8* counts, LO n, LO* out);
// same, with the scan's scratch in a fixed device array instead of pool
// memory: allocates nothing, at most offset_scan_fixed_limit() counts, and
// calls in flight on one device at once race on the shared scratch
void offset_scan_fixed_scratch(const LO* counts, LO n, LO* out);
LO offset_scan_fixed_limit();

// the single-pass scan with its first tile withheld, so that the other
// tiles' bounded waits run out and raise ST_STALL (a test of the limit)
void scan_wait_limit_selftest(const LO* counts, LO n, LO* out);

// indices of nonzero marks (collect_marked, src/Omega_h_map.cpp:174-185)
Arr<LO> collect_marked(const Arr<I8>& marks, const char* file = __builtin_FILE(),
                       int line = __builtin_LINE());
// the same, with *extra_host = *extra_dev read in the same wait
Arr<LO> collect_marked(const Arr<I8>& marks, const int* extra_dev, int* extra_host,
                       const char* file = __builtin_FILE(), int line = __builtin_LINE());
LO count_marked(const Arr<I8>& marks, const char* file = __builtin_FILE(),
                int line = __builtin_LINE());

LO last(const Arr<LO>& a, const char* file = __builtin_FILE(), int line = __builtin_LINE());
// FP64 fused multiply-add throughput of the device (GFLOP/s, best of reps)
double fp64_peak_gflops(int reps);
// the last element of each array (at most 16) with one host wait
// (status, if given, receives the device status word read in the same wait;
// it is not cleared)
void read_lasts(const std::vector<const Arr<LO>*>& arrs, LO* out, int* status = nullptr,
                const char* file = __builtin_FILE(), int line = __builtin_LINE());
// indices of nonzero marks given offset_scan of the 0/1 marks and its total
Arr<LO> collect_marked_offs(const Arr<I8>& marks, const Arr<LO>& offs, LO cnt);

// reductions (synchronise the stream)
I8 max_i8(const Arr<I8>& a);
double min_f64(const Arr<double>& a);
Arr<double> min_f64_dev(const Arr<double>& a);  // no host wait
double max_f64(const Arr<double>& a);
LO max_lo(const Arr<LO>& a);

// stable permutation sort of n tuples of width w, lexicographic
// (sort_by_keys, src/Omega_h_sort.cpp:71-92); LSD radix sort
Arr<LO> sort_by_keys(const Arr<LO>& keys, int width);
Arr<LO> sort_by_keys64(const Arr<GO>& keys, int width);

template <class T>
Arr<T> fill(LO n, T v) {
  Arr<T> a(n);
  if (n <= 0) return a;
  // a value whose bytes are all equal (0, -1, 0.0) is a memset
  unsigned char b[sizeof(T)];
  std::memcpy(b, &v, sizeof(T));
  bool same = true;
  for (size_t k = 1; k < sizeof(T); ++k) same = same && b[k] == b[0];
  if (same) {
    OHG_CUDA(cudaMemsetAsync(a.data(), b[0], sizeof(T) * size_t(n), ctx().stream));
    return a;
  }
  auto p = view(a);
  pfor(n, [=] __device__(LO i) { p[i] = v; });
  return a;
}
inline Arr<LO> iota(LO n) {
  Arr<LO> a(n);
  auto p = view(a);
  pfor(n, [=] __device__(LO i) { p[i] = i; });
  return a;
}
// a[i*w+j] = b[a2b[i]*w+j]  (unmap)
template <class T>
Arr<T> unmap(const Arr<LO>& a2b, const Arr<T>& b, int w) {
  Arr<T> a(a2b.size() * w);
  auto m = cview(a2b);
  auto src = cview(b);
  auto dst = view(a);
  pfor(a2b.size(), [=] __device__(LO i) {
    LO k = m[i];
    for (int j = 0; j < w; ++j) dst[i * w + j] = src[k * w + j];
  });
  return a;
}
// b[a2b[i]*w+j] = a[i*w+j]  (map_into)
template <class T>
void map_into(const Arr<T>& a, const Arr<LO>& a2b, Arr<T>& b, int w) {
  auto m = cview(a2b);
  auto src = cview(a);
  auto dst = view(b);
  pfor(a2b.size(), [=] __device__(LO i) {
    LO k = m[i];
    for (int j = 0; j < w; ++j) dst[k * w + j] = src[i * w + j];
  });
}
template <class T>
Arr<T> map_onto(const Arr<T>& a, const Arr<LO>& a2b, LO nb, T init, int w) {
  Arr<T> b = fill<T>(nb * w, init);
  map_into(a, a2b, b, w);
  return b;
}
inline Arr<I8> mark_image(const Arr<LO>& a2b, LO nb) {
  Arr<I8> out = fill<I8>(nb, 0);
  auto m = cview(a2b);
  auto o = view(out);
  pfor(a2b.size(), [=] __device__(LO i) { o[m[i]] = 1; });
  return out;
}

}  // namespace ohg
