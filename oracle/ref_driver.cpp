// Dump driver for the reference Omega_h build (oracle/_ref).  Builds a
// seeded box workload with the reference's own build_box, runs one adapt
// pass (refine_by_size -> coarsen_by_size -> swap_edges when the minimum
// quality is below min_quality_desired, as src/Omega_h_adapt.cpp:173-210
// sequences them) and writes every per-stage intermediate array plus the
// mesh after each operator as raw little-endian files with a manifest.
//
// This is test infrastructure: it produces golden fixtures and is never
// linked into the product.
//
//   ref_driver DIM N METRIC SEED MIN_QUAL_ALLOWED OUTDIR
#include <Omega_h_adapt.hpp>
#include <Omega_h_adj.hpp>
#include <Omega_h_array_ops.hpp>
#include <Omega_h_build.hpp>
#include <Omega_h_coarsen.hpp>
#include <Omega_h_collapse.hpp>
#include <Omega_h_file.hpp>
#include <Omega_h_hilbert.hpp>
#include <Omega_h_indset.hpp>
#include <Omega_h_library.hpp>
#include <Omega_h_map.hpp>
#include <Omega_h_mark.hpp>
#include <Omega_h_mesh.hpp>
#include <Omega_h_metric.hpp>
#include <Omega_h_metric_intersect.hpp>
#include <Omega_h_modify.hpp>
#include <Omega_h_quality.hpp>
#include <Omega_h_refine.hpp>
#include <Omega_h_refine_qualities.hpp>
#include <Omega_h_shape.hpp>
#include <Omega_h_swap.hpp>
#include <Omega_h_swap2d.hpp>
#include <Omega_h_swap3d.hpp>
#include <Omega_h_swap3d_loop.hpp>
#include <Omega_h_swap3d_tables.hpp>
#include <Omega_h_timer.hpp>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "ohg_workload.hpp"

using namespace Omega_h;

static std::string g_out;
static FILE* g_manifest = nullptr;

template <typename T>
static const char* dtype_name();
template <>
const char* dtype_name<I8>() { return "i1"; }
template <>
const char* dtype_name<I32>() { return "i4"; }
template <>
const char* dtype_name<I64>() { return "i8"; }
template <>
const char* dtype_name<Real>() { return "f8"; }

template <typename T>
static void dump(std::string const& name, Read<T> a) {
  HostRead<T> h(a);
  std::string path = g_out + "/" + name + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (h.size()) std::fwrite(h.data(), sizeof(T), size_t(h.size()), f);
  std::fclose(f);
  std::fprintf(g_manifest, "%s %s %d\n", name.c_str(), dtype_name<T>(),
      int(h.size()));
}

static void dump_scalar(std::string const& name, double v) {
  dump(name, Reals({v}));
}

static void dump_mesh(Mesh* mesh, std::string const& p) {
  int dim = mesh->dim();
  dump_scalar(p + "nents", mesh->nverts());
  for (int d = 1; d <= dim; ++d) {
    dump(p + "ev2v_" + std::to_string(d), mesh->ask_verts_of(d));
    auto down = mesh->ask_down(d, d - 1);
    dump(p + "down_" + std::to_string(d), down.ab2b);
    if (d > 1) dump(p + "downcodes_" + std::to_string(d), down.codes);
  }
  for (int d = 0; d <= dim; ++d) {
    auto s = std::to_string(d);
    dump(p + "global_" + s, mesh->globals(d));
    dump(p + "class_dim_" + s, mesh->get_array<I8>(d, "class_dim"));
    dump(p + "class_id_" + s, mesh->get_array<I32>(d, "class_id"));
  }
  dump(p + "coords", mesh->coords());
  dump(p + "metric", mesh->get_array<Real>(VERT, "metric"));
  if (mesh->has_tag(EDGE, "length"))
    dump(p + "length", mesh->get_array<Real>(EDGE, "length"));
  if (mesh->has_tag(dim, "quality"))
    dump(p + "quality", mesh->get_array<Real>(dim, "quality"));
}

static void dump_adjacency(Mesh* mesh, std::string const& p) {
  int dim = mesh->dim();
  for (int lo = 0; lo < dim; ++lo) {
    for (int hi = lo + 1; hi <= dim; ++hi) {
      auto s = std::to_string(lo) + std::to_string(hi);
      auto up = mesh->ask_up(lo, hi);
      dump(p + "up_a2ab_" + s, up.a2ab);
      dump(p + "up_ab2b_" + s, up.ab2b);
      dump(p + "up_codes_" + s, up.codes);
    }
  }
  if (dim == 3) {
    auto t2e = mesh->ask_down(3, 1);
    dump(p + "down31", t2e.ab2b);
    dump(p + "downcodes31", t2e.codes);
  }
  for (int d = 0; d <= 1; ++d) {
    auto star = mesh->ask_star(d);
    dump(p + "star_a2ab_" + std::to_string(d), star.a2ab);
    dump(p + "star_ab2b_" + std::to_string(d), star.ab2b);
  }
  auto dual = mesh->ask_dual();
  dump(p + "dual_a2ab", dual.a2ab);
  dump(p + "dual_ab2b", dual.ab2b);
}

static double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
      .count();
}

// refine stage intermediates, following refine_by_size/refine_ghosted
// (src/Omega_h_refine.cpp:17-41,92-100)
static void dump_refine_stage(Mesh* mesh, AdaptOpts const& opts) {
  auto lengths = mesh->ask_lengths();
  auto cands = each_gt(lengths, opts.max_length_desired);
  dump("r_cands", cands);
  if (get_max(cands) != 1) return;
  auto cands2edges = collect_marked(cands);
  dump("r_cands2edges", cands2edges);
  dump("r_midmetrics", get_mident_metrics(mesh, EDGE, cands2edges,
                           mesh->get_array<Real>(VERT, "metric")));
  auto cand_quals = refine_qualities(mesh, cands2edges);
  dump("r_cand_quals", cand_quals);
  auto good = each_geq_to(cand_quals, opts.min_quality_allowed);
  if (get_max(good) != 1) return;
  auto nedges = mesh->nedges();
  auto initial = map_onto(good, cands2edges, nedges, I8(0), 1);
  auto edge_quals = map_onto(cand_quals, cands2edges, nedges, 0.0, 1);
  auto keys = find_indset(mesh, EDGE, edge_quals, initial);
  dump("r_keys", keys);
  dump("r_rep2md", get_rep2md_order_adapt(mesh, EDGE, VERT, keys));
}

// coarsen stage intermediates, following coarsen_by_size, coarsen_verts,
// coarsen_element_based1 and coarsen_ghosted (src/Omega_h_coarsen.cpp:29-104,
// 174-208)
static void dump_coarsen_stage(Mesh* mesh, AdaptOpts const& opts) {
  auto lengths = mesh->ask_lengths();
  auto edge_is_cand = each_lt(lengths, opts.min_length_desired);
  dump("c_edge_is_cand", edge_is_cand);
  if (get_max(edge_is_cand) != 1) return;
  auto vert_marks = mark_down(mesh, EDGE, VERT, edge_is_cand);
  dump("c_vert_marks", vert_marks);
  auto ev2v = mesh->ask_verts_of(EDGE);
  auto nedges = mesh->nedges();
  HostRead<LO> hev2v(ev2v);
  HostRead<I8> hvm(vert_marks);
  HostWrite<I8> hcodes(nedges);
  for (LO e = 0; e < nedges; ++e) {
    I8 code = DONT_COLLAPSE;
    for (Int eev = 0; eev < 2; ++eev)
      if (hvm[hev2v[e * 2 + eev]]) code = do_collapse(code, eev);
    hcodes[e] = code;
  }
  Read<I8> edge_codes(hcodes.write());
  dump("c_edge_codes", edge_codes);
  auto cands2edges = collect_marked(each_neq_to(edge_codes, I8(DONT_COLLAPSE)));
  auto cand_codes = read(unmap(cands2edges, edge_codes, 1));
  cand_codes = check_collapse_class(mesh, cands2edges, cand_codes);
  dump("c_class_codes", cand_codes);
  if (get_max(cand_codes) <= DONT_COLLAPSE) return;
  edge_codes = map_onto(cand_codes, cands2edges, nedges, I8(DONT_COLLAPSE), 1);
  cands2edges = collect_marked(each_neq_to(edge_codes, I8(DONT_COLLAPSE)));
  cand_codes = read(unmap(cands2edges, edge_codes, 1));
  dump("c_cands2edges0", cands2edges);
  cand_codes = check_collapse_exposure(mesh, cands2edges, cand_codes);
  dump("c_expo_codes", cand_codes);
  auto filt = [&](Reals* quals) {
    auto keep = each_neq_to(cand_codes, I8(DONT_COLLAPSE));
    auto new2old = collect_marked(keep);
    cands2edges = unmap(new2old, cands2edges, 1);
    cand_codes = unmap(new2old, cand_codes, 1);
    if (quals) *quals = unmap(new2old, *quals, 2);
  };
  filt(nullptr);
  dump("c_cands2edges1", cands2edges);
  cand_codes = prevent_coarsen_overshoot(
      mesh, opts.max_length_desired, cands2edges, cand_codes);
  dump("c_over_codes", cand_codes);
  filt(nullptr);
  dump("c_cands2edges2", cands2edges);
  if (cands2edges.size() == 0) return;
  auto quals = coarsen_qualities(mesh, cands2edges, cand_codes);
  dump("c_quals", quals);
  cand_codes = filter_coarsen_min_qual(cand_codes, quals, opts.min_quality_allowed);
  dump("c_minq_codes", cand_codes);
  filt(&quals);
  dump("c_cands2edges3", cands2edges);
  dump("c_cand_codes3", cand_codes);
  if (cands2edges.size() == 0) return;
  Read<I8> verts_are_cands;
  Reals vert_quals;
  Read<GO> vert_rails;
  choose_rails(mesh, cands2edges, cand_codes, quals, &verts_are_cands,
      &vert_quals, &vert_rails);
  dump("c_verts_are_cands", verts_are_cands);
  dump("c_vert_quals", vert_quals);
  dump("c_vert_rails", vert_rails);
  auto keys = find_indset(mesh, VERT, vert_quals, verts_are_cands);
  dump("c_keys", keys);
  auto keys2verts = collect_marked(keys);
  LOs rails2edges;
  Read<I8> rail_col_dirs;
  find_rails(mesh, keys2verts, vert_rails, &rails2edges, &rail_col_dirs);
  dump("c_rails2edges", rails2edges);
  dump("c_rail_col_dirs", rail_col_dirs);
  auto dead = mark_dead_ents(mesh, rails2edges, rail_col_dirs);
  for (int d = 1; d <= mesh->dim(); ++d)
    dump("c_dead_" + std::to_string(d), dead[d]);
}

// swap stage intermediates, following swap_part1 and swap3d_ghosted
// (src/Omega_h_swap.cpp:14-43, src/Omega_h_swap3d.cpp:14-37)
static void dump_swap_stage(Mesh* mesh, AdaptOpts const& opts) {
  auto elems_are_cands =
      mark_sliver_layers(mesh, opts.min_quality_desired, opts.nsliver_layers);
  dump("s_elem_cands", elems_are_cands);
  auto edges_are_cands = mark_down(mesh, mesh->dim(), EDGE, elems_are_cands);
  auto inter = mark_by_class_dim(mesh, EDGE, mesh->dim());
  edges_are_cands = land_each(edges_are_cands, inter);
  dump("s_edge_cands", edges_are_cands);
  if (get_max(edges_are_cands) <= 0) return;
  auto cands2edges = collect_marked(edges_are_cands);
  Reals cand_quals;
  if (mesh->dim() == 3) {
    Read<I8> cand_configs;
    swap3d_qualities(mesh, opts, cands2edges, &cand_quals, &cand_configs);
    dump("s_cand_configs", cand_configs);
  } else {
    cand_quals = swap2d_qualities(mesh, opts, cands2edges);
  }
  dump("s_cands2edges", cands2edges);
  dump("s_cand_quals", cand_quals);
  auto keep = filter_swap_improve(mesh, cands2edges, cand_quals);
  dump("s_keep", keep);
  filter_swap(keep, &cands2edges, &cand_quals);
  if (cands2edges.size() == 0) return;
  auto is_cand = mark_image(cands2edges, mesh->nedges());
  auto edge_quals = map_onto(cand_quals, cands2edges, mesh->nedges(), -1.0, 1);
  auto keys = find_indset(mesh, EDGE, edge_quals, is_cand);
  dump("s_keys", keys);
}

static void dump_swap_tables() {
  std::vector<I32> t;
  for (int n = 3; n <= 7; ++n) {
    int nmesh = swap3d::swap_mesh_counts[n];
    int ntri = swap3d::swap_mesh_sizes[n];
    int nuniq = 0;
    for (int i = 0; i < nmesh * ntri; ++i)
      nuniq = std::max(nuniq, swap3d::swap_meshes[n][i] + 1);
    t.push_back(n);
    t.push_back(nmesh);
    t.push_back(ntri);
    t.push_back(nuniq);
    for (int u = 0; u < nuniq; ++u)
      for (int k = 0; k < 3; ++k) t.push_back(swap3d::swap_triangles[n][u][k]);
    for (int i = 0; i < nmesh * ntri; ++i) t.push_back(swap3d::swap_meshes[n][i]);
    int ne = swap3d::nedges[n];
    t.push_back(ne);
    int nuedge = 0;
    if (ne) {
      for (int m = 0; m < nmesh; ++m)
        for (int e = 0; e < ne; ++e)
          nuedge = std::max(nuedge, swap3d::edges2unique[n][m][e] + 1);
    }
    t.push_back(nuedge);
    for (int u = 0; u < nuedge; ++u)
      for (int k = 0; k < 2; ++k) t.push_back(swap3d::unique_edges[n][u][k]);
    for (int m = 0; m < nmesh; ++m)
      for (int e = 0; e < ne; ++e) t.push_back(swap3d::edges2unique[n][m][e]);
  }
  HostWrite<I32> h(LO(t.size()));
  for (size_t i = 0; i < t.size(); ++i) h[LO(i)] = t[i];
  dump("swap3d_tables", Read<I32>(h.write()));
}

// A smooth scalar field's Hessian at each vertex, packed like a metric:
// f = sin(4x) cos(3y) (+ z^2 in 3D).  The same numbers feed the GPU side
// through the dump.
static Reals analytic_hessians(Mesh* mesh) {
  int dim = mesh->dim();
  int nc = dim == 3 ? 6 : 3;
  HostRead<Real> c(mesh->coords());
  HostWrite<Real> h(mesh->nverts() * nc);
  for (LO v = 0; v < mesh->nverts(); ++v) {
    double x = c[v * dim], y = c[v * dim + 1];
    double sx = std::sin(4 * x), cx = std::cos(4 * x), sy = std::sin(3 * y), cy = std::cos(3 * y);
    double fxx = -16 * sx * cy, fyy = -9 * sx * cy, fxy = -12 * cx * sy;
    if (dim == 3) {
      double r[6] = {fxx, fyy, 2.0, fxy, 0.0, 0.0};
      for (int k = 0; k < 6; ++k) h[v * 6 + k] = r[k];
    } else {
      double r[3] = {fxx, fyy, fxy};
      for (int k = 0; k < 3; ++k) h[v * 3 + k] = r[k];
    }
  }
  return Reals(h.write());
}

// "metric": the metric tools on the box after the workload
static void dump_metric_tools(Mesh* mesh) {
  auto n = mesh->nverts();
  auto given = mesh->get_array<Real>(VERT, "metric");
  dump("mt_given", given);
  auto implied = get_implied_metrics(mesh);
  dump("mt_implied", implied);
  dump("mt_intersect", intersect_metrics(n, given, implied));
  dump("mt_clamp", clamp_metrics(n, given, 0.02, 0.2));
  auto hess = analytic_hessians(mesh);
  dump("mt_hessians", hess);
  dump("mt_hessian_metrics", get_hessian_metrics(mesh->dim(), hess, 0.01));
  dump("mt_gradation", limit_metric_gradation(mesh, given, 1.0, 1e-3, false));
  dump("mt_expected_nelems", Reals({get_expected_nelems(mesh, given)}));
  MetricInput in;
  in.verbose = false;
  in.add_source(MetricSource(OMEGA_H_GIVEN, 1.0, "metric", OMEGA_H_ANISOTROPIC, OMEGA_H_SCALES));
  in.add_source(MetricSource(OMEGA_H_IMPLIED, 2.0, "", OMEGA_H_ISO_SIZE, OMEGA_H_ABSOLUTE));
  in.add_source(MetricSource(OMEGA_H_CONSTANT, 0.3, "", OMEGA_H_ANISOTROPIC, OMEGA_H_ABSOLUTE));
  in.should_limit_lengths = true;
  in.min_length = 0.05;
  in.max_length = 0.5;
  in.should_limit_gradation = true;
  in.max_gradation_rate = 1.0;
  in.nsmoothing_steps = 1;
  in.should_limit_element_count = true;
  in.max_element_count = 4.0 * mesh->nelems();
  in.min_element_count = 1.0 * mesh->nelems();
  dump("mt_generated", generate_metrics(mesh, in));
}

// "intersect": intersect_metrics on seeded pairs of partially degenerate
// metrics (rank 1 and 2 in 3D, rank 1 in 2D), in random orientations and in
// shared eigenbases, plus the reference's unit-test cases; inputs and the
// reference's outputs packed (xx, yy, zz, yx, zy, zx) / (xx, yy, yx)
template <Int dim>
static Tensor<dim> random_rotation(std::mt19937_64& g) {
  std::normal_distribution<double> nd(0.0, 1.0);
  Tensor<dim> q;
  // Gram-Schmidt on Gaussian columns
  for (Int j = 0; j < dim; ++j) {
    Vector<dim> v;
    for (Int i = 0; i < dim; ++i) v[i] = nd(g);
    for (Int k = 0; k < j; ++k) v = v - (v * q[k]) * q[k];
    q[j] = normalize(v);
  }
  return q;
}
template <Int dim>
static void dump_degenerate_intersections(std::mt19937_64& g) {
  std::uniform_real_distribution<double> ud(0.25, 4.0);
  std::vector<Tensor<dim>> as, bs;
  const int npairs = 96;
  for (int p = 0; p < npairs; ++p) {
    Tensor<dim> qa = random_rotation<dim>(g);
    // a third of the pairs share the eigenbasis (up to a permutation of it)
    Tensor<dim> qb = (p % 3 == 0) ? qa : random_rotation<dim>(g);
    if (p % 3 == 0 && dim == 3 && (p / 3) % 2) {
      auto t = qb[0];
      qb[0] = qb[2];
      qb[2] = t;
    }
    int ra = (dim == 2) ? 1 : 1 + int(g() % 2);
    int rb = (dim == 2) ? 1 : 1 + int(g() % 2);
    Vector<dim> la, lb;
    for (Int i = 0; i < dim; ++i) {
      la[i] = i < ra ? ud(g) : 0.0;
      lb[i] = i < rb ? ud(g) : 0.0;
    }
    as.push_back(compose_ortho(qa, la));
    bs.push_back(compose_ortho(qb, lb));
  }
  if (dim == 3) {
    // src/unit_math.cpp:221-252
    double cases[6][2][3] = {{{1, 0, 0}, {0, 0, 1}}, {{1, 0, 0}, {2, 0, 0}},
        {{1, 0, 0}, {2, 1, 0}}, {{1, 0, 0}, {0, 1, 2}}, {{1, 0, 2}, {2, 0, 1}},
        {{1, 0, 2}, {2, 1, 0}}};
    for (auto& c : cases) {
      Vector<dim> a, b;
      for (Int i = 0; i < dim; ++i) {
        a[i] = c[0][i];
        b[i] = c[1][i];
      }
      as.push_back(diagonal(a));
      bs.push_back(diagonal(b));
    }
  }
  LO n = LO(as.size());
  int nc = symm_ncomps(dim);
  HostWrite<Real> ha(n * nc), hb(n * nc), ho(n * nc);
  for (LO i = 0; i < n; ++i) {
    auto o = intersect_metrics(as[i], bs[i]);
    auto va = symm2vector(as[i]), vb = symm2vector(bs[i]), vo = symm2vector(o);
    for (int k = 0; k < nc; ++k) {
      ha[i * nc + k] = va[k];
      hb[i * nc + k] = vb[k];
      ho[i * nc + k] = vo[k];
    }
  }
  std::string pre = "di" + std::to_string(dim) + "_";
  dump(pre + "a", Reals(ha.write()));
  dump(pre + "b", Reals(hb.write()));
  dump(pre + "out", Reals(ho.write()));
}

int main(int argc, char** argv) {
  if (argc == 3 && std::string(argv[1]) == "intersect") {
    g_out = argv[2];
    g_manifest = std::fopen((g_out + "/manifest.txt").c_str(), "w");
    std::mt19937_64 g(20261204);
    dump_degenerate_intersections<2>(g);
    dump_degenerate_intersections<3>(g);
    std::fclose(g_manifest);
    return 0;
  }
  if (argc < 7) {
    std::fprintf(stderr,
        "usage: %s DIM N METRIC SEED MIN_QUAL_ALLOWED OUTDIR [nopass]\n",
        argv[0]);
    return 2;
  }
  int dim = std::atoi(argv[1]);
  int n = std::atoi(argv[2]);
  int metric_kind = std::atoi(argv[3]);
  unsigned long long seed = std::strtoull(argv[4], nullptr, 10);
  double mqa = std::atof(argv[5]);
  g_out = argv[6];
  std::string mode = argc < 8 ? "" : argv[7];
  bool stages = mode.empty();
  g_manifest = std::fopen((g_out + "/manifest.txt").c_str(), "w");
  auto lib = Library(&argc, &argv);
  auto t0 = std::chrono::steady_clock::now();
  auto mesh = build_box(lib.world(), OMEGA_H_SIMPLEX, 1., 1., dim == 3 ? 1. : 0.,
      n, n, dim == 3 ? n : 0);
  double t_build = seconds_since(t0);
  // seeded jitter of interior vertices, then the analytic metric
  auto coords = mesh.coords();
  auto vcd = mesh.get_array<I8>(VERT, "class_dim");
  HostWrite<Real> hc(deep_copy(coords));
  HostRead<I8> hcd(vcd);
  for (LO v = 0; v < mesh.nverts(); ++v) {
    if (hcd[v] != dim) continue;
    for (int j = 0; j < dim; ++j)
      hc[v * dim + j] += ohg::workload::jitter(seed, v, j, dim, n);
  }
  mesh.set_coords(Reals(hc.write()));
  ohg::workload::MetricParams mp =
      ohg::workload::make_params(ohg::workload::base_kind(metric_kind), seed);
  int ncomp = dim == 3 ? 6 : 3;
  HostWrite<Real> hm(mesh.nverts() * ncomp);
  HostRead<Real> hc2(mesh.coords());
  for (LO v = 0; v < mesh.nverts(); ++v)
    ohg::workload::metric_at(mp, dim, &hc2[v * dim], &hm[v * ncomp]);
  if (ohg::workload::scalar_kind(metric_kind)) {
    // an isotropic metric tag of one component per vertex
    HostWrite<Real> hs(mesh.nverts());
    for (LO v = 0; v < mesh.nverts(); ++v) hs[v] = hm[v * ncomp];
    mesh.add_tag(VERT, "metric", 1, Reals(hs.write()));
  } else {
    mesh.add_tag(VERT, "metric", ncomp, Reals(hm.write()));
  }

  AdaptOpts opts(&mesh);
  opts.min_quality_allowed = mqa;
  opts.verbosity = SILENT;
  dump_scalar("opts",
      0.0);  // placeholder so the manifest always has an entry
  dump("opts_values", Reals({opts.min_length_desired, opts.max_length_desired,
                          opts.max_length_allowed, opts.min_quality_allowed,
                          opts.min_quality_desired, Real(opts.nsliver_layers)}));
  if (stages) {
    dump_mesh(&mesh, "in_");
    dump_adjacency(&mesh, "in_");
    dump("in_length_fresh", measure_edges_metric(&mesh));
    dump("in_quality_fresh", measure_qualities(&mesh));
    dump("in_hilbert_perm", hilbert::sort_coords(mesh.coords(), dim));
    if (dim == 3) dump_swap_tables();
  }
  // "osh": the mesh before and after one pass in the reference's own binary
  // format (binary::write, src/Omega_h_file.cpp:355-396), for the .osh
  // reader/writer parity tests
  if (mode == "metric") {
    dump_metric_tools(&mesh);
    std::fclose(g_manifest);
    std::printf("metric tools on %d verts\n", int(mesh.nverts()));
    return 0;
  }
  bool osh = mode == "osh";
  if (osh) binary::write(filesystem::path(g_out + "/in.osh"), &mesh);
  if (mode == "adapt") {
    // the full Omega_h::adapt() instead of one pass; the counts of operator
    // calls are not observable from outside adapt(), so only the outcome and
    // the mesh are dumped
    auto ta = std::chrono::steady_clock::now();
    bool did = adapt(&mesh, opts);
    double t_ad = seconds_since(ta);
    dump("adapt_did", LOs({int(did)}));
    dump_mesh(&mesh, "out_");
    if (argc > 8 && std::string(argv[8]) == "osh")
      binary::write(filesystem::path(g_out + "/out.osh"), &mesh);
    std::fclose(g_manifest);
    std::printf("build %.4f adapt %.4f elems_out %d\n", t_build, t_ad, int(mesh.nelems()));
    return 0;
  }
  // one adapt pass
  double t_ref = 0, t_coa = 0, t_swp = 0;
  mesh.set_parting(OMEGA_H_GHOSTED);
  if (stages) dump_refine_stage(&mesh, opts);
  auto t1 = std::chrono::steady_clock::now();
  bool did_refine = refine_by_size(&mesh, opts);
  t_ref = seconds_since(t1);
  if (stages) dump_mesh(&mesh, "r_out_");
  mesh.set_parting(OMEGA_H_GHOSTED);
  if (stages) dump_coarsen_stage(&mesh, opts);
  t1 = std::chrono::steady_clock::now();
  bool did_coarsen = coarsen_by_size(&mesh, opts);
  t_coa = seconds_since(t1);
  if (stages) dump_mesh(&mesh, "c_out_");
  mesh.set_parting(OMEGA_H_GHOSTED);
  double minq = get_min(mesh.ask_qualities());
  bool did_swap = false;
  if (minq < opts.min_quality_desired) {
    if (stages) dump_swap_stage(&mesh, opts);
    t1 = std::chrono::steady_clock::now();
    did_swap = swap_edges(&mesh, opts);
    t_swp = seconds_since(t1);
  }
  dump("pass_flags", LOs({did_refine, did_coarsen, did_swap}));
  dump_mesh(&mesh, "out_");
  if (osh) binary::write(filesystem::path(g_out + "/out.osh"), &mesh);
  std::fclose(g_manifest);
  std::printf(
      "build %.4f refine %.4f coarsen %.4f swap %.4f pass %.4f "
      "flags %d %d %d minq %.6f elems_in %d elems_out %d\n",
      t_build, t_ref, t_coa, t_swp, t_ref + t_coa + t_swp, int(did_refine),
      int(did_coarsen), int(did_swap), minq,
      int(std::pow(double(n), dim) * (dim == 3 ? 6 : 2)), int(mesh.nelems()));
  return 0;
}
