// A compiled C++ caller of include/ohg.h alone, as a host program that owns
// its mesh in plain host arrays would call it: upload (ohg_mesh_from_arrays
// from pageable host memory), one adapt pass (ohg_adapt_pass), read-back of
// every array with one ohg_mesh_get_arrays call.  Built and run by
// tests/test_gpu_capi_caller.py.
//
//   capi_caller IN_DIR OUT_DIR
//
// IN_DIR holds meta.txt ("dim nverts nedges nfaces nregions
// min_quality_allowed") and raw arrays down_<d>.bin (int32), downcodes_<d>.bin
// (int8, d >= 2), class_dim_<d>.bin (int8), class_id_<d>.bin (int32),
// coords.bin and metric.bin (float64).  OUT_DIR receives out_<name>.bin
// for every mesh array, pass_flags.bin, and manifest.txt
// ("name dtype count" per line).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ohg.h"

static std::vector<char> read_file(const std::string& path) {
  std::vector<char> b;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  b.resize(size_t(n));
  if (n && std::fread(b.data(), 1, size_t(n), f) != size_t(n)) std::exit(2);
  std::fclose(f);
  return b;
}

static void check(int rc, const char* what) {
  if (rc != OHG_OK) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, ohg_last_error());
    std::exit(1);
  }
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s IN_DIR OUT_DIR\n", argv[0]);
    return 2;
  }
  std::string in = argv[1], out = argv[2];
  int dim = 0, nents[4] = {0, 0, 0, 0};
  double mqa = 0.0;
  {
    FILE* f = std::fopen((in + "/meta.txt").c_str(), "r");
    if (!f || std::fscanf(f, "%d %d %d %d %d %lf", &dim, &nents[0], &nents[1], &nents[2],
                          &nents[3], &mqa) != 6)
      return 2;
    std::fclose(f);
  }
  std::vector<std::vector<char>> keep;
  const int* down[4] = {nullptr, nullptr, nullptr, nullptr};
  const signed char* codes[4] = {nullptr, nullptr, nullptr, nullptr};
  const signed char* cdim[4] = {nullptr, nullptr, nullptr, nullptr};
  const int* cid[4] = {nullptr, nullptr, nullptr, nullptr};
  keep.reserve(16);
  for (int d = 0; d <= dim; ++d) {
    std::string s = std::to_string(d);
    if (d > 0) {
      keep.push_back(read_file(in + "/down_" + s + ".bin"));
      down[d] = reinterpret_cast<const int*>(keep.back().data());
      if (d > 1) {
        keep.push_back(read_file(in + "/downcodes_" + s + ".bin"));
        codes[d] = reinterpret_cast<const signed char*>(keep.back().data());
      }
    }
    keep.push_back(read_file(in + "/class_dim_" + s + ".bin"));
    cdim[d] = reinterpret_cast<const signed char*>(keep.back().data());
    keep.push_back(read_file(in + "/class_id_" + s + ".bin"));
    cid[d] = reinterpret_cast<const int*>(keep.back().data());
  }
  std::vector<char> coords = read_file(in + "/coords.bin");
  std::vector<char> metric = read_file(in + "/metric.bin");

  ohg_context* ctx = nullptr;
  check(ohg_context_create(0, &ctx), "ohg_context_create");
  ohg_mesh* m = nullptr;
  check(ohg_mesh_from_arrays(ctx, dim, nents, down, codes, cdim, cid,
                             reinterpret_cast<const double*>(coords.data()),
                             reinterpret_cast<const double*>(metric.data()), &m),
        "ohg_mesh_from_arrays");
  ohg_adapt_opts o;
  check(ohg_adapt_opts_default(dim, &o), "ohg_adapt_opts_default");
  o.min_quality_allowed = mqa;
  ohg_pass_stats st;
  std::memset(&st, 0, sizeof(st));
  check(ohg_adapt_pass(m, &o, &st), "ohg_adapt_pass");

  // every mesh array of the result, read back with one call
  struct Arr {
    std::string name, dtype;
    int width;
  };
  std::vector<Arr> arrs = {{"coords", "<f8", 8}, {"metric", "<f8", 8}, {"length", "<f8", 8},
                           {"quality", "<f8", 8}};
  for (int d = 0; d <= dim; ++d) {
    std::string s = std::to_string(d);
    arrs.push_back({"class_dim_" + s, "|i1", 1});
    arrs.push_back({"class_id_" + s, "<i4", 4});
    if (d > 0) arrs.push_back({"down_" + s, "<i4", 4});
    if (d > 1) {
      arrs.push_back({"downcodes_" + s, "|i1", 1});
      arrs.push_back({"ev2v_" + s, "<i4", 4});
    }
  }
  std::vector<std::vector<char>> bufs(arrs.size());
  std::vector<const char*> names;
  std::vector<void*> dsts;
  std::vector<long long> caps;
  for (size_t i = 0; i < arrs.size(); ++i) {
    long long nb = 0;
    check(ohg_mesh_array_bytes(m, arrs[i].name.c_str(), &nb), "ohg_mesh_array_bytes");
    bufs[i].resize(size_t(nb) + 1);
    names.push_back(arrs[i].name.c_str());
    dsts.push_back(bufs[i].data());
    caps.push_back(nb);
  }
  check(ohg_mesh_get_arrays(m, int(names.size()), names.data(), dsts.data(), caps.data()),
        "ohg_mesh_get_arrays");
  FILE* man = std::fopen((out + "/manifest.txt").c_str(), "w");
  for (size_t i = 0; i < arrs.size(); ++i) {
    std::string key = "out_" + arrs[i].name;
    FILE* f = std::fopen((out + "/" + key + ".bin").c_str(), "wb");
    size_t nb = bufs[i].size() - 1;
    if (nb) std::fwrite(bufs[i].data(), 1, nb, f);
    std::fclose(f);
    std::fprintf(man, "%s %s %zu\n", key.c_str(), arrs[i].dtype.c_str(),
                 nb / size_t(arrs[i].width));
  }
  int flags[3] = {st.did_refine, st.did_coarsen, st.did_swap};
  FILE* f = std::fopen((out + "/pass_flags.bin").c_str(), "wb");
  std::fwrite(flags, sizeof(int), 3, f);
  std::fclose(f);
  std::fprintf(man, "pass_flags <i4 3\n");
  std::fclose(man);
  check(ohg_mesh_destroy(m), "ohg_mesh_destroy");
  check(ohg_context_destroy(ctx), "ohg_context_destroy");
  std::printf("pass flags %d %d %d, %d -> %d elements\n", flags[0], flags[1], flags[2],
              st.nelems_in, st.nelems_out);
  return 0;
}
