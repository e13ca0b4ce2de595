// ORACLE — test infrastructure only.  Runs the oracle restatement on a seeded
// box workload and writes the same per-stage arrays, under the same names, as
// oracle/ref_driver.cpp writes for the reference, so tests can compare the two
// (and the GPU product) array by array.
//
//   oracle_driver DIM N METRIC SEED MIN_QUAL_ALLOWED OUTDIR [nostages|time|adapt]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <string>

#include "../omega_h_gb300/csrc/ohg_workload.hpp"
#include "oracle_core.hpp"

using namespace orc;

static std::string g_out;
static FILE* g_manifest = nullptr;

template <class T>
static const char* dtn();
template <>
const char* dtn<I8>() { return "i1"; }
template <>
const char* dtn<LO>() { return "i4"; }
template <>
const char* dtn<GO>() { return "i8"; }
template <>
const char* dtn<double>() { return "f8"; }

template <class T>
static void dump(const std::string& name, const V<T>& a) {
  if (!g_manifest) return;
  FILE* f = std::fopen((g_out + "/" + name + ".bin").c_str(), "wb");
  if (!a.empty()) std::fwrite(a.data(), sizeof(T), a.size(), f);
  std::fclose(f);
  std::fprintf(g_manifest, "%s %s %d\n", name.c_str(), dtn<T>(), int(a.size()));
}

static void dump_mesh(Mesh& m, const std::string& p) {
  dump(p + "nents", V<double>{double(m.nverts())});
  for (int d = 1; d <= m.dim; ++d) {
    if (d > 1) dump(p + "ev2v_" + std::to_string(d), m.ask_verts_of(d));
    const Adj& dn = m.ask_down(d, d - 1);
    dump(p + "down_" + std::to_string(d), dn.ab2b);
    if (d > 1) dump(p + "downcodes_" + std::to_string(d), dn.codes);
  }
  for (int d = 0; d <= m.dim; ++d) {
    dump(p + "class_dim_" + std::to_string(d), m.class_dim[d]);
    dump(p + "class_id_" + std::to_string(d), m.class_id[d]);
  }
  dump(p + "coords", m.coords);
  dump(p + "metric", m.metric);
  if (m.has_length) dump(p + "length", m.length);
  if (m.has_quality) dump(p + "quality", m.quality);
}

static void dump_adjacency(Mesh& m, const std::string& p) {
  for (int lo = 0; lo < m.dim; ++lo)
    for (int hi = lo + 1; hi <= m.dim; ++hi) {
      std::string s = std::to_string(lo) + std::to_string(hi);
      const Adj& up = m.ask_up(lo, hi);
      dump(p + "up_a2ab_" + s, up.a2ab);
      dump(p + "up_ab2b_" + s, up.ab2b);
      dump(p + "up_codes_" + s, up.codes);
    }
  if (m.dim == 3) {
    const Adj& t2e = m.ask_down(3, 1);
    dump(p + "down31", t2e.ab2b);
    dump(p + "downcodes31", t2e.codes);
  }
  for (int d = 0; d <= 1; ++d) {
    const Adj& s = m.ask_adj(d, d);
    dump(p + "star_a2ab_" + std::to_string(d), s.a2ab);
    dump(p + "star_ab2b_" + std::to_string(d), s.ab2b);
  }
  const Adj& dual = m.ask_adj(m.dim, m.dim);
  dump(p + "dual_a2ab", dual.a2ab);
  dump(p + "dual_ab2b", dual.ab2b);
}

template <class T>
static V<T> gather(const V<LO>& idx, const V<T>& a) {
  V<T> o(idx.size());
  for (size_t i = 0; i < idx.size(); ++i) o[i] = a[idx[i]];
  return o;
}

static void dump_refine_stage(Mesh& m, const AdaptOpts& o) {
  const V<double>& len = m.ask_lengths();
  V<I8> cands(len.size());
  bool any = false;
  for (size_t i = 0; i < len.size(); ++i) any |= bool((cands[i] = len[i] > o.max_length_desired));
  dump("r_cands", cands);
  if (!any) return;
  V<LO> c2e = collect_marked(cands);
  dump("r_cands2edges", c2e);
  dump("r_midmetrics", get_mident_metrics(m, c2e));
  V<double> cq = refine_qualities(m, c2e);
  dump("r_cand_quals", cq);
  LO ne = m.nedges();
  V<I8> init((size_t)(ne), 0);
  V<double> eq((size_t)(ne), 0.0);
  bool good = false;
  for (size_t i = 0; i < c2e.size(); ++i) {
    init[c2e[i]] = cq[i] >= o.min_quality_allowed;
    good |= bool(init[c2e[i]]);
    eq[c2e[i]] = cq[i];
  }
  if (!good) return;
  V<I8> keys = find_indset(m, EDGE, eq, init);
  dump("r_keys", keys);
  dump("r_rep2md", get_rep2md_order_adapt(m, EDGE, VERT, keys));
}

static void dump_coarsen_stage(Mesh& m, const AdaptOpts& o) {
  const V<double>& len = m.ask_lengths();
  V<I8> ec(len.size());
  bool any = false;
  for (size_t i = 0; i < len.size(); ++i) any |= bool((ec[i] = len[i] < o.min_length_desired));
  dump("c_edge_is_cand", ec);
  if (!any) return;
  // mark_down(EDGE -> VERT)
  const Adj& v2e = m.ask_up(0, 1);
  V<I8> vm((size_t)(m.nverts()), 0);
  for (LO v = 0; v < m.nverts(); ++v)
    for (LO j = v2e.a2ab[v]; j < v2e.a2ab[v + 1]; ++j)
      if (ec[v2e.ab2b[j]]) vm[v] = 1;
  dump("c_vert_marks", vm);
  const V<LO>& ev2v = m.ask_verts_of(1);
  V<I8> codes_e(len.size());
  for (size_t e = 0; e < len.size(); ++e)
    codes_e[e] = I8((vm[ev2v[e * 2]] ? 1 : 0) | (vm[ev2v[e * 2 + 1]] ? 2 : 0));
  dump("c_edge_codes", codes_e);
  V<LO> c2e = collect_marked(codes_e);
  V<I8> codes = check_collapse_class(m, c2e, gather(c2e, codes_e));
  dump("c_class_codes", codes);
  I8 mx = 0;
  for (I8 c : codes) mx = std::max(mx, c);
  if (mx <= 0) return;
  std::fill(codes_e.begin(), codes_e.end(), I8(0));
  for (size_t i = 0; i < c2e.size(); ++i) codes_e[c2e[i]] = codes[i];
  c2e = collect_marked(codes_e);
  codes = gather(c2e, codes_e);
  dump("c_cands2edges0", c2e);
  codes = check_collapse_exposure(m, c2e, codes);
  dump("c_expo_codes", codes);
  V<double> quals;
  auto filt = [&](bool q) {
    V<LO> keep;
    for (size_t i = 0; i < codes.size(); ++i)
      if (codes[i]) keep.push_back(LO(i));
    c2e = gather(keep, c2e);
    codes = gather(keep, codes);
    if (q) {
      V<double> nq(keep.size() * 2);
      for (size_t i = 0; i < keep.size(); ++i) {
        nq[i * 2] = quals[(size_t)(keep[i]) * 2];
        nq[i * 2 + 1] = quals[(size_t)(keep[i]) * 2 + 1];
      }
      quals = nq;
    }
  };
  filt(false);
  dump("c_cands2edges1", c2e);
  codes = prevent_coarsen_overshoot(m, o.max_length_desired, c2e, codes);
  dump("c_over_codes", codes);
  filt(false);
  dump("c_cands2edges2", c2e);
  if (c2e.empty()) return;
  quals = coarsen_qualities(m, c2e, codes);
  dump("c_quals", quals);
  for (size_t c = 0; c < codes.size(); ++c)
    for (int d = 0; d < 2; ++d)
      if (!(quals[c * 2 + d] >= o.min_quality_allowed)) codes[c] = I8(codes[c] & ~(1 << d));
  dump("c_minq_codes", codes);
  filt(true);
  dump("c_cands2edges3", c2e);
  dump("c_cand_codes3", codes);
  if (c2e.empty()) return;
  V<I8> vc;
  V<double> vq;
  V<GO> vr;
  choose_rails(m, c2e, codes, quals, &vc, &vq, &vr);
  dump("c_verts_are_cands", vc);
  dump("c_vert_quals", vq);
  dump("c_vert_rails", vr);
  V<I8> keys = find_indset(m, VERT, vq, vc);
  dump("c_keys", keys);
  V<LO> r2e;
  V<I8> rdir;
  find_rails(m, collect_marked(keys), vr, &r2e, &rdir);
  dump("c_rails2edges", r2e);
  dump("c_rail_col_dirs", rdir);
  V<I8> dead[4];
  mark_dead_ents(m, r2e, rdir, dead);
  for (int d = 1; d <= m.dim; ++d) dump("c_dead_" + std::to_string(d), dead[d]);
}

static void dump_swap_stage(Mesh& m, const AdaptOpts& o) {
  V<I8> ec = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  dump("s_elem_cands", ec);
  const Adj& e2t = m.ask_up(1, m.dim);
  V<I8> edc((size_t)(m.nedges()), 0);
  bool any = false;
  for (LO e = 0; e < m.nedges(); ++e) {
    for (LO j = e2t.a2ab[e]; j < e2t.a2ab[e + 1]; ++j)
      if (ec[e2t.ab2b[j]]) edc[e] = 1;
    edc[e] = edc[e] && m.class_dim[1][e] == m.dim;
    any |= bool(edc[e]);
  }
  dump("s_edge_cands", edc);
  if (!any) return;
  V<LO> c2e = collect_marked(edc);
  V<double> cq;
  if (m.dim == 3) {
    V<I8> cc;
    swap3d_qualities(m, o, c2e, &cq, &cc);
    dump("s_cand_configs", cc);
  } else {
    cq = swap2d_qualities(m, o, c2e);
  }
  dump("s_cands2edges", c2e);
  dump("s_cand_quals", cq);
  V<I8> keep = filter_swap_improve(m, c2e, cq);
  dump("s_keep", keep);
  V<LO> kept;
  for (size_t i = 0; i < keep.size(); ++i)
    if (keep[i]) kept.push_back(LO(i));
  if (kept.empty()) return;
  V<I8> is_cand((size_t)(m.nedges()), 0);
  V<double> eq((size_t)(m.nedges()), -1.0);
  for (LO i : kept) {
    is_cand[c2e[i]] = 1;
    eq[c2e[i]] = cq[i];
  }
  dump("s_keys", find_indset(m, EDGE, eq, is_cand));
}

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: %s DIM N METRIC SEED MQA OUTDIR [nostages|time|adapt]\n", argv[0]);
    return 2;
  }
  int dim = std::atoi(argv[1]), n = std::atoi(argv[2]), kind = std::atoi(argv[3]);
  unsigned long long seed = std::strtoull(argv[4], nullptr, 10);
  double mqa = std::atof(argv[5]);
  g_out = argv[6];
  std::string mode = argc > 7 ? argv[7] : "";
  bool stages = mode.empty();
  if (mode != "time") g_manifest = std::fopen((g_out + "/manifest.txt").c_str(), "w");
  try {
    auto t0 = std::chrono::steady_clock::now();
    Mesh m = build_box(dim, n);
    for (LO v = 0; v < m.nverts(); ++v) {
      if (m.class_dim[0][v] != dim) continue;
      for (int j = 0; j < dim; ++j)
        m.coords[(size_t)(v) * dim + j] += ohg::workload::jitter(seed, v, j, dim, n);
    }
    ohg::workload::MetricParams mp = ohg::workload::make_params(kind, seed);
    int mc = m.mcomp();
    m.metric.resize((size_t)(m.nverts()) * mc);
    for (LO v = 0; v < m.nverts(); ++v)
      ohg::workload::metric_at(mp, dim, &m.coords[(size_t)(v) * dim], &m.metric[(size_t)(v) * mc]);
    double t_build = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    AdaptOpts o(dim);
    o.min_quality_allowed = mqa;
    if (stages) {
      dump_mesh(m, "in_");
      dump_adjacency(m, "in_");
      V<LO> all_e((size_t)(m.nedges())), all_t((size_t)(m.nelems()));
      std::iota(all_e.begin(), all_e.end(), 0);
      std::iota(all_t.begin(), all_t.end(), 0);
      dump("in_length_fresh", measure_edges_metric(m, all_e));
      dump("in_quality_fresh", measure_qualities(m, all_t));
      dump("in_hilbert_perm", hilbert_sort(m.coords, dim));
    }
    if (mode == "adapt") {
      // the full adapt() loop instead of one pass
      auto ta = std::chrono::steady_clock::now();
      AdaptResult ar = adapt(m, o);
      double t_ad = std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
      dump("adapt_result", V<LO>{ar.did, ar.quality_satisfied, ar.refines, ar.coarsens, ar.swaps,
                                 ar.sliver_coarsens, ar.length_rounds});
      dump_mesh(m, "out_");
      if (g_manifest) std::fclose(g_manifest);
      std::printf("build %.4f adapt %.4f elems_out %d\n", t_build, t_ad, int(m.nelems()));
      return 0;
    }
    auto t1 = std::chrono::steady_clock::now();
    if (stages) dump_refine_stage(m, o);
    PassResult r;
    auto since = [](std::chrono::steady_clock::time_point t) {
      return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
    };
    r.did_refine = refine_by_size(m, o);
    double t_ref = since(t1);
    if (stages) dump_mesh(m, "r_out_");
    if (stages) dump_coarsen_stage(m, o);
    auto t2 = std::chrono::steady_clock::now();
    r.did_coarsen = coarsen_by_size(m, o);
    double t_coa = since(t2);
    if (stages) dump_mesh(m, "c_out_");
    auto t3 = std::chrono::steady_clock::now();
    const V<double>& q = m.ask_qualities();
    double minq = q[0];
    for (double x : q) minq = std::min(minq, x);
    if (minq < o.min_quality_desired) {
      if (stages) dump_swap_stage(m, o);
      r.did_swap = swap_edges(m, o);
    }
    double t_swp = since(t3);
    double t_pass = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    if (mode == "time") std::printf("refine %.4f coarsen %.4f swap %.4f ", t_ref, t_coa, t_swp);
    dump("pass_flags", V<LO>{r.did_refine, r.did_coarsen, r.did_swap});
    dump_mesh(m, "out_");
    if (g_manifest) std::fclose(g_manifest);
    std::printf("build %.4f pass %.4f flags %d %d %d minq %.6f elems_out %d\n", t_build, t_pass,
                int(r.did_refine), int(r.did_coarsen), int(r.did_swap), minq, int(m.nelems()));
  } catch (std::exception& e) {
    std::fprintf(stderr, "oracle error: %s\n", e.what());
    return 1;
  }
  return 0;
}
