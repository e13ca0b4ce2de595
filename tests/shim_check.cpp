// Exercises the Omega_h::Mesh side of the GPU adapt pass without a GPU: the
// checks that refuse a mesh the pass would lose data from, and the upload's
// handling of a library error.  Built and run by tests/test_shim.py against
// the reference's own library (compiled from its sources), whose failures
// print their message and abort: each case runs in its own process.
//   shim_check no_metric | user_field | null_context
#include <Omega_h_build.hpp>
#include <Omega_h_library.hpp>

#include <cstdio>
#include <string>

#include "omega_h_adapt_gb300.hpp"

using namespace Omega_h;

int main(int argc, char** argv) {
  std::string what = argc > 1 ? argv[1] : "";
  auto lib = Library(&argc, &argv);
  auto mesh = build_box(lib.world(), OMEGA_H_SIMPLEX, 1., 1., 1., 2, 2, 2);
  if (what != "no_metric") mesh.add_tag(VERT, "metric", 6, Reals(mesh.nverts() * 6, 0.0));
  if (what == "user_field") mesh.add_tag(VERT, "user_field", 1, Reals(mesh.nverts(), 1.0));
  // a carriable mesh reaches the C ABI, which refuses the null context
  AdaptOpts opts(&mesh);
  adapt_pass_gb300(nullptr, &mesh, opts);
  std::printf("not refused\n");
  return 0;
}
