// The Omega_h::Mesh side of the GB300 adapt pass: lift the mesh's arrays
// into the C ABI, run the pass there, and rebuild the Mesh from the result.
#include "omega_h_adapt_gb300.hpp"

#include <Omega_h_fail.hpp>
#include <Omega_h_mesh.hpp>

#include <cstring>
#include <string>
#include <vector>

namespace Omega_h {

namespace {

// the tags the GPU pass produces again after every rebuild
const char* const kCarriedTags[] = {"coordinates", "metric", "class_dim", "class_id",
                                    "global", "length", "quality"};

void check_ohg(int rc, const char* what) {
  if (rc != OHG_OK) Omega_h_fail("%s failed (%d): %s\n", what, rc, ohg_last_error());
}

// Everything that would make the GPU pass lose data is refused before any
// call into the library.
void check_carriable(Mesh* mesh) {
  if (mesh->family() != OMEGA_H_SIMPLEX)
    Omega_h_fail("adapt on the GPU: only simplex meshes are supported\n");
  if (mesh->dim() != 2 && mesh->dim() != 3)
    Omega_h_fail("adapt on the GPU: only 2D and 3D meshes are supported\n");
  if (mesh->comm()->size() != 1)
    Omega_h_fail("adapt on the GPU: the mesh must live on one rank\n");
  if (!mesh->has_tag(VERT, "metric"))
    Omega_h_fail("adapt on the GPU: the mesh has no \"metric\" tag\n");
  for (Int d = 0; d <= mesh->dim(); ++d) {
    for (Int i = 0; i < mesh->ntags(d); ++i) {
      std::string const& name = mesh->get_tag(d, i)->name();
      bool carried = false;
      for (const char* c : kCarriedTags) carried = carried || name == c;
      if (!carried)
        Omega_h_fail(
            "adapt on the GPU: tag \"%s\" on dimension %d would not be transferred; the GPU "
            "pass carries coordinates, metric, class_dim, class_id, global, length and "
            "quality only\n",
            name.c_str(), int(d));
    }
  }
}

ohg_mesh* upload(ohg_context* ctx, Mesh* mesh) {
  Int dim = mesh->dim();
  int nents[4] = {0, 0, 0, 0};
  const int* down[4] = {nullptr, nullptr, nullptr, nullptr};
  const signed char* codes[4] = {nullptr, nullptr, nullptr, nullptr};
  const signed char* class_dim[4] = {nullptr, nullptr, nullptr, nullptr};
  const int* class_id[4] = {nullptr, nullptr, nullptr, nullptr};
  // the Read<T> handles keep the arrays alive until the copies are done
  std::vector<LOs> keep_lo;
  std::vector<Read<I8>> keep_i8;
  for (Int d = 0; d <= dim; ++d) {
    nents[d] = mesh->nents(d);
    if (d > 0) {
      Adj a = mesh->ask_down(d, d - 1);
      keep_lo.push_back(a.ab2b);
      down[d] = a.ab2b.data();
      if (d > 1) {
        keep_i8.push_back(a.codes);
        codes[d] = reinterpret_cast<const signed char*>(a.codes.data());
      }
    }
    auto cd = mesh->get_array<I8>(d, "class_dim");
    auto ci = mesh->get_array<ClassId>(d, "class_id");
    keep_i8.push_back(cd);
    keep_lo.push_back(ci);
    class_dim[d] = reinterpret_cast<const signed char*>(cd.data());
    class_id[d] = ci.data();
  }
  Reals coords = mesh->coords();
  Reals metric = mesh->get_array<Real>(VERT, "metric");
  Int ncomps = mesh->get_tagbase(VERT, "metric")->ncomps();
  Int packed = symm_ncomps(dim);
  if (ncomps != 1 && ncomps != packed)
    Omega_h_fail("adapt on the GPU: a metric of %d components\n", int(ncomps));
  ohg_mesh* m = nullptr;
  if (ncomps == packed) {
    check_ohg(ohg_mesh_from_arrays(ctx, int(dim), nents, down, codes, class_dim, class_id,
                                   coords.data(), metric.data(), &m),
              "ohg_mesh_from_arrays");
  } else {
    // an isotropic metric tag (one value per vertex): the mesh is made with a
    // placeholder tensor, then given the scalar field, which the library
    // evaluates with the reference's scalar formulas
    std::vector<double> zero(size_t(nents[0]) * size_t(packed), 0.0);
    check_ohg(ohg_mesh_from_arrays(ctx, int(dim), nents, down, codes, class_dim, class_id,
                                   coords.data(), zero.data(), &m),
              "ohg_mesh_from_arrays");
    int rc = ohg_mesh_set_array(m, "metric", metric.data(), 8LL * nents[0]);
    if (rc != OHG_OK) {
      ohg_mesh_destroy(m);
      check_ohg(rc, "ohg_mesh_set_array(metric)");
    }
  }
  return m;
}

ohg_adapt_opts to_ohg(Int dim, AdaptOpts const& opts) {
  ohg_adapt_opts o;
  check_ohg(ohg_adapt_opts_default(int(dim), &o), "ohg_adapt_opts_default");
  o.min_length_desired = opts.min_length_desired;
  o.max_length_desired = opts.max_length_desired;
  o.max_length_allowed = opts.max_length_allowed;
  o.min_quality_allowed = opts.min_quality_allowed;
  o.min_quality_desired = opts.min_quality_desired;
  o.nsliver_layers = int(opts.nsliver_layers);
  return o;
}

long long array_bytes(ohg_mesh* m, std::string const& name) {
  long long b = 0;
  check_ohg(ohg_mesh_array_bytes(m, name.c_str(), &b), ("ohg_mesh_array_bytes(" + name + ")").c_str());
  return b;
}

// Reads every array of the pass's result with one ohg_mesh_get_arrays call
// into Write<T> arrays (device memory in a CUDA build of the reference, host
// memory otherwise) and rebuilds *mesh from them.
void download(ohg_mesh* m, Mesh* mesh) {
  Int dim = mesh->dim();
  LO nents[4] = {0, 0, 0, 0};
  for (Int d = 0; d <= dim; ++d) {
    int n = 0;
    check_ohg(ohg_mesh_nents(m, int(d), &n), "ohg_mesh_nents");
    nents[d] = n;
  }
  Write<Real> coords(LO(array_bytes(m, "coords") / 8));
  Write<Real> metric(LO(array_bytes(m, "metric") / 8));
  Write<Real> length(LO(array_bytes(m, "length") / 8));
  Write<Real> quality(LO(array_bytes(m, "quality") / 8));
  std::vector<Write<LO>> down(size_t(dim + 1)), class_id(size_t(dim + 1));
  std::vector<Write<I8>> codes(size_t(dim + 1)), class_dim(size_t(dim + 1));
  std::vector<std::string> names = {"coords", "metric", "length", "quality"};
  std::vector<void*> dsts = {coords.data(), metric.data(), length.data(), quality.data()};
  std::vector<long long> caps = {8LL * coords.size(), 8LL * metric.size(), 8LL * length.size(),
                                 8LL * quality.size()};
  for (Int d = 0; d <= dim; ++d) {
    std::string s = std::to_string(d);
    class_dim[size_t(d)] = Write<I8>(nents[d]);
    class_id[size_t(d)] = Write<LO>(nents[d]);
    names.push_back("class_dim_" + s);
    dsts.push_back(class_dim[size_t(d)].data());
    caps.push_back(nents[d]);
    names.push_back("class_id_" + s);
    dsts.push_back(class_id[size_t(d)].data());
    caps.push_back(4LL * nents[d]);
    if (d > 0) {
      LO deg = d + 1;
      down[size_t(d)] = Write<LO>(nents[d] * deg);
      names.push_back("down_" + s);
      dsts.push_back(down[size_t(d)].data());
      caps.push_back(4LL * nents[d] * deg);
      if (d > 1) {
        codes[size_t(d)] = Write<I8>(nents[d] * deg);
        names.push_back("downcodes_" + s);
        dsts.push_back(codes[size_t(d)].data());
        caps.push_back(1LL * nents[d] * deg);
      }
    }
  }
  std::vector<const char*> cnames;
  for (auto& n : names) cnames.push_back(n.c_str());
  check_ohg(ohg_mesh_get_arrays(m, int(names.size()), cnames.data(), dsts.data(), caps.data()),
            "ohg_mesh_get_arrays");
  // the rebuild, as the reference's operators make their new mesh
  Mesh out = mesh->copy_meta();
  out.set_verts(nents[0]);
  for (Int d = 1; d <= dim; ++d) {
    if (d > 1)
      out.set_ents(d, Adj(LOs(down[size_t(d)]), Read<I8>(codes[size_t(d)])));
    else
      out.set_ents(d, Adj(LOs(down[size_t(d)])));
  }
  out.add_tag<Real>(VERT, "coordinates", dim, Reals(coords));
  out.add_tag<Real>(VERT, "metric", Int(metric.size() / nents[0]), Reals(metric));
  for (Int d = 0; d <= dim; ++d) {
    out.add_tag<I8>(d, "class_dim", 1, Read<I8>(class_dim[size_t(d)]));
    out.add_tag<ClassId>(d, "class_id", 1, LOs(class_id[size_t(d)]));
    // one rank: global numbers are the local ones
    out.add_tag<GO>(d, "global", 1, GOs(nents[d], 0, 1));
  }
  out.add_tag<Real>(EDGE, "length", 1, Reals(length));
  out.add_tag<Real>(dim, "quality", 1, Reals(quality));
  *mesh = out;
}

}  // namespace

bool adapt_pass_gb300(ohg_context* ctx, Mesh* mesh, AdaptOpts const& opts) {
  check_carriable(mesh);
  ohg_mesh* m = upload(ctx, mesh);
  ohg_adapt_opts o = to_ohg(mesh->dim(), opts);
  ohg_pass_stats st;
  std::memset(&st, 0, sizeof(st));
  int rc = ohg_adapt_pass(m, &o, &st);
  if (rc == OHG_OK) {
    try {
      download(m, mesh);
    } catch (...) {
      ohg_mesh_destroy(m);
      throw;
    }
  }
  ohg_mesh_destroy(m);
  check_ohg(rc, "ohg_adapt_pass");
  return st.did_refine || st.did_coarsen || st.did_swap;
}

bool adapt_gb300(ohg_context* ctx, Mesh* mesh, AdaptOpts const& opts) {
  check_carriable(mesh);
  ohg_mesh* m = upload(ctx, mesh);
  ohg_adapt_opts o = to_ohg(mesh->dim(), opts);
  ohg_adapt_result r;
  std::memset(&r, 0, sizeof(r));
  int rc = ohg_adapt(m, &o, &r);
  if (rc == OHG_OK) {
    try {
      download(m, mesh);
    } catch (...) {
      ohg_mesh_destroy(m);
      throw;
    }
  }
  ohg_mesh_destroy(m);
  check_ohg(rc, "ohg_adapt");
  return r.did != 0;
}

}  // namespace Omega_h
