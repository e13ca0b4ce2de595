// ORACLE — test infrastructure only (see oracle_core.hpp).
// Independent sets, refine/coarsen/swap operators, the rebuild (modify) and
// field transfer of one adapt pass.
#include <algorithm>
#include <numeric>

#include "oracle_core.hpp"

namespace orc {

#define OHG_SWAP3D_TABLE_QUAL static
#include "../omega_h_gb300/csrc/ohg_swap3d_tables.inc"

static inline double min2(double a, double b) { return (b < a) ? b : a; }

template <class T>
static V<T> unmap(const V<LO>& a2b, const V<T>& b, int w) {
  V<T> a(a2b.size() * (size_t)(w));
  for (size_t i = 0; i < a2b.size(); ++i)
    for (int j = 0; j < w; ++j) a[i * w + j] = b[(size_t)(a2b[i]) * w + j];
  return a;
}
template <class T>
static void map_into(const V<T>& a, const V<LO>& a2b, V<T>& b, int w) {
  for (size_t i = 0; i < a2b.size(); ++i)
    for (int j = 0; j < w; ++j) b[(size_t)(a2b[i]) * w + j] = a[i * w + j];
}
static V<LO> iota_lo(LO n) {
  V<LO> a((size_t)(n));
  std::iota(a.begin(), a.end(), 0);
  return a;
}

// ------------------------------------------------------------ swap3d tables
namespace swap3d {
struct Tab {
  int off_tri[8], off_mesh[8], off_uedge[8], off_e2u[8];
  int nmesh[8], ntri[8], nedge[8];
  Tab() {
    for (int i = 0; i < 8; ++i) nmesh[i] = ntri[i] = nedge[i] = 0;
    int p = 0;
    while (p < OHG_SWAP3D_TABLE_LEN) {
      int n = OHG_SWAP3D_TABLE[p], nm = OHG_SWAP3D_TABLE[p + 1],
          nt = OHG_SWAP3D_TABLE[p + 2], nu = OHG_SWAP3D_TABLE[p + 3];
      p += 4;
      nmesh[n] = nm;
      ntri[n] = nt;
      off_tri[n] = p;
      p += nu * 3;
      off_mesh[n] = p;
      p += nm * nt;
      int ne = OHG_SWAP3D_TABLE[p], nue = OHG_SWAP3D_TABLE[p + 1];
      p += 2;
      nedge[n] = ne;
      off_uedge[n] = p;
      p += nue * 2;
      off_e2u[n] = p;
      p += nm * ne;
    }
  }
};
static const Tab& tab() {
  static Tab t;
  return t;
}
int mesh_count(int n) { return tab().nmesh[n]; }
int mesh_size(int n) { return tab().ntri[n]; }
const int* triangle(int n, int u) { return &OHG_SWAP3D_TABLE[tab().off_tri[n] + u * 3]; }
int mesh_tri(int n, int m, int t) {
  return OHG_SWAP3D_TABLE[tab().off_mesh[n] + m * tab().ntri[n] + t];
}
int nedges(int n) { return tab().nedge[n]; }
const int* unique_edge(int n, int u) { return &OHG_SWAP3D_TABLE[tab().off_uedge[n] + u * 2]; }
int edge2unique(int n, int m, int e) {
  return OHG_SWAP3D_TABLE[tab().off_e2u[n] + m * tab().nedge[n] + e];
}
}  // namespace swap3d

// ------------------------------------------------------------ indset
// (src/Omega_h_indset.cpp:5-34, src/Omega_h_indset_inline.hpp:14-72)
enum { NOT_IN = 0, IN = 1, UNKNOWN = 2 };
V<I8> find_indset(const Adj& g, const V<double>& q, const V<I8>& cands, int* nrounds) {
  LO n = LO(g.a2ab.size() - 1);
  V<I8> state((size_t)(n));
  for (LO i = 0; i < n; ++i) state[i] = cands[i] ? UNKNOWN : NOT_IN;
  int rounds = 0;
  auto compare = [&](LO u, LO v) {
    if (q[u] != q[v]) return q[u] < q[v];
    return u < v;  // global numbers equal local numbers on one rank
  };
  while (std::find(state.begin(), state.end(), I8(UNKNOWN)) != state.end()) {
    V<I8> ns = state;
    ORC_PARALLEL_FOR
    for (LO v = 0; v < n; ++v) {
      if (state[v] != UNKNOWN) continue;
      bool rejected = false;
      for (LO j = g.a2ab[v]; j < g.a2ab[v + 1]; ++j)
        if (state[g.ab2b[j]] == IN) {
          rejected = true;
          break;
        }
      if (rejected) {
        ns[v] = NOT_IN;
        continue;
      }
      bool local_max = true;
      for (LO j = g.a2ab[v]; j < g.a2ab[v + 1]; ++j) {
        LO u = g.ab2b[j];
        if (state[u] == NOT_IN) continue;
        if (!compare(u, v)) {
          local_max = false;
          break;
        }
      }
      if (local_max) ns[v] = IN;
    }
    state.swap(ns);
    ++rounds;
  }
  if (nrounds) *nrounds = rounds;
  return state;
}
V<I8> find_indset(Mesh& m, int d, const V<double>& q, const V<I8>& cands) {
  if (d == m.dim) return cands;
  return find_indset(m.ask_adj(d, d), q, cands, nullptr);
}

// ------------------------------------------------------------ marks
static V<I8> mark_image(const V<LO>& a2b, LO nb) {
  V<I8> out((size_t)(nb), 0);
  for (LO b : a2b) out[b] = 1;
  return out;
}
static V<I8> mark_up(Mesh& m, int ld, int hd, const V<I8>& lm) {
  const V<LO>& hl2l = m.ask_down(hd, ld).ab2b;
  int deg = simplex_degree(hd, ld);
  LO nh = m.nents[hd];
  V<I8> out((size_t)(nh), 0);
  for (LO h = 0; h < nh; ++h)
    for (int k = 0; k < deg; ++k)
      if (lm[hl2l[(size_t)(h) * deg + k]]) out[h] = 1;
  return out;
}
static V<I8> mark_down(Mesh& m, int hd, int ld, const V<I8>& hm) {
  if (hd == ld) return hm;
  const Adj& l2h = m.ask_up(ld, hd);
  LO nl = m.nents[ld];
  V<I8> out((size_t)(nl), 0);
  for (LO l = 0; l < nl; ++l)
    for (LO lh = l2h.a2ab[l]; lh < l2h.a2ab[l + 1]; ++lh)
      if (hm[l2h.ab2b[lh]]) out[l] = 1;
  return out;
}

// ------------------------------------------------------------ modify
// get_rep2md_order (src/Omega_h_modify.cpp:269-338) for one kind of
// modified entity (mod_dim) with nprods products each
static V<LO> rep2md_order(Mesh& m, int rep_dim, int mod_dim, const V<LO>& mods2mds,
                          const V<LO>& mods2nprods) {
  V<LO> order((size_t)(m.nents[mod_dim]), -1);
  V<LO> mds2mods((size_t)(m.nents[mod_dim]), -1);
  for (size_t i = 0; i < mods2mds.size(); ++i) mds2mods[mods2mds[i]] = LO(i);
  const Adj& r2m = m.ask_up(rep_dim, mod_dim);
  for (LO rep = 0; rep < m.nents[rep_dim]; ++rep) {
    LO offset = 0;
    for (LO rm = r2m.a2ab[rep]; rm < r2m.a2ab[rep + 1]; ++rm) {
      LO md = r2m.ab2b[rm];
      LO mod = mds2mods[md];
      if (mod >= 0 && code_which_down(r2m.codes[rm]) == 0) {
        order[md] = offset;
        offset += mods2nprods[mod];
      }
    }
  }
  return order;
}
V<LO> get_rep2md_order_adapt(Mesh& m, int key_dim, int rep_dim, const V<I8>& keys) {
  V<LO> mods = collect_marked(keys);
  return rep2md_order(m, rep_dim, key_dim, mods, V<LO>(mods.size(), 1));
}

struct ModifyOut {
  V<LO> prods2new, same2old, same2new, old2new;
};

// modify_ents_adapt + modify_ents + modify_conn (src/Omega_h_modify.cpp:20-70,
// 141-517) on one rank, where global numbers coincide with local ones
static ModifyOut modify_ents_adapt(Mesh& om, Mesh& nm, int ent_dim, int key_dim,
                                   const V<LO>& keys2kds, const V<LO>& keys2prods,
                                   const V<LO>& prod_verts2verts,
                                   const V<LO>& old_lows2new_lows) {
  int dim = om.dim;
  V<I8> mds_are_mods[4];
  mds_are_mods[key_dim] = mark_image(keys2kds, om.nents[key_dim]);
  for (int md = key_dim + 1; md <= dim; ++md)
    mds_are_mods[md] = mark_up(om, key_dim, md, mds_are_mods[key_dim]);
  ModifyOut out;
  LO nold = om.nents[ent_dim];
  if (ent_dim >= key_dim) {
    for (LO e = 0; e < nold; ++e)
      if (!mds_are_mods[ent_dim][e]) out.same2old.push_back(e);
  } else {
    out.same2old = iota_lo(nold);
  }
  LO nkeys = LO(keys2kds.size());
  V<LO> nprods((size_t)(nkeys));
  for (LO k = 0; k < nkeys; ++k) nprods[k] = keys2prods[k + 1] - keys2prods[k];
  // representatives (get_mods2reps)
  V<LO> reps((size_t)(nkeys));
  if (key_dim == ent_dim) {
    reps = keys2kds;
  } else if (ent_dim > key_dim) {
    const Adj& up = om.ask_up(key_dim, ent_dim);
    for (LO k = 0; k < nkeys; ++k) reps[k] = up.ab2b[up.a2ab[keys2kds[k]]];
  } else {
    const V<LO>& dn = om.ask_down(key_dim, ent_dim).ab2b;
    int deg = simplex_degree(key_dim, ent_dim);
    for (LO k = 0; k < nkeys; ++k) reps[k] = dn[(size_t)(keys2kds[k]) * deg];
  }
  V<LO> counts((size_t)(nold), 0);
  for (LO e : out.same2old) counts[e] = 1;
  for (LO k = 0; k < nkeys; ++k) counts[reps[k]] += nprods[k];
  V<LO> offs = offset_scan(counts);
  LO nnew = offs[nold];
  bool has_order = key_dim > ent_dim;
  V<LO> order;
  if (has_order) order = rep2md_order(om, ent_dim, key_dim, keys2kds, nprods);
  out.same2new = unmap(out.same2old, offs, 1);
  out.prods2new.resize((size_t)(keys2prods[nkeys]));
  int self = has_order ? 1 : 0;
  for (LO k = 0; k < nkeys; ++k) {
    LO offset = offs[reps[k]] + self;
    if (has_order) offset += order[keys2kds[k]];
    for (LO p = keys2prods[k]; p < keys2prods[k + 1]; ++p) out.prods2new[p] = offset++;
  }
  out.old2new.assign((size_t)(nold), -1);
  map_into(out.same2new, out.same2old, out.old2new, 1);
  if (ent_dim == VERT) {
    nm.nents[0] = nnew;
    return out;
  }
  int ld = ent_dim - 1;
  int deg = simplex_degree(ent_dim, ld);
  const Adj& od = om.ask_down(ent_dim, ld);
  Adj nd;
  nd.ab2b.resize((size_t)(nnew) * deg);
  Adj pd;
  if (ld > VERT) {
    pd = reflect_down(prod_verts2verts, nm.ask_verts_of(ld), nm.ask_up(VERT, ld), ent_dim, ld);
  } else {
    pd.ab2b = prod_verts2verts;
  }
  map_into(pd.ab2b, out.prods2new, nd.ab2b, deg);
  V<LO> same_lows = unmap(out.same2old, od.ab2b, deg);
  for (LO& l : same_lows) l = old_lows2new_lows[l];
  map_into(same_lows, out.same2new, nd.ab2b, deg);
  if (ld > VERT) {
    nd.codes.resize((size_t)(nnew) * deg);
    map_into(unmap(out.same2old, od.codes, deg), out.same2new, nd.codes, deg);
    map_into(pd.codes, out.prods2new, nd.codes, deg);
  }
  nm.set_ents(ent_dim, std::move(nd));
  return out;
}

// transfer_common (src/Omega_h_transfer.cpp:160-180)
template <class T>
static V<T> xfer(const V<T>& old_data, const ModifyOut& mo, LO nnew, const V<T>& prod_data, int w) {
  V<T> nd((size_t)(nnew) * w);
  map_into(prod_data, mo.prods2new, nd, w);
  map_into(unmap(mo.same2old, old_data, w), mo.same2new, nd, w);
  return nd;
}

static void xfer_lengths_qualities(Mesh& om, Mesh& nm, int d, const ModifyOut& mo) {
  if (d == EDGE && om.has_length) {
    nm.length = xfer(om.length, mo, nm.nents[1], measure_edges_metric(nm, mo.prods2new), 1);
    nm.has_length = true;
  }
  if (d == om.dim && om.has_quality) {
    nm.quality = xfer(om.quality, mo, nm.nents[d], measure_qualities(nm, mo.prods2new), 1);
    nm.has_quality = true;
  }
}

// ------------------------------------------------------------ refine
// refine_qualities_tmpl (src/Omega_h_refine_qualities.cpp:34-86)
V<double> refine_qualities(Mesh& m, const V<LO>& c2e) {
  int dim = m.dim;
  const V<LO>& ev2v = m.ask_verts_of(1);
  const V<LO>& cv2v = m.ask_verts_of(dim);
  const Adj& e2c = m.ask_up(1, dim);
  V<double> mid = get_mident_metrics(m, c2e);
  V<double> out(c2e.size());
  ORC_PARALLEL_FOR
  for (size_t cand = 0; cand < c2e.size(); ++cand) {
    LO e = c2e[cand];
    LO ev[2] = {ev2v[(size_t)(e) * 2], ev2v[(size_t)(e) * 2 + 1]};
    double midp[3];
    for (int j = 0; j < dim; ++j)
      midp[j] = (m.coords[(size_t)(ev[0]) * dim + j] + m.coords[(size_t)(ev[1]) * dim + j]) / 2.;
    double minqual = 1.0;
    for (LO ec = e2c.a2ab[e]; ec < e2c.a2ab[e + 1]; ++ec) {
      LO c = e2c.ab2b[ec];
      I8 code = e2c.codes[ec];
      int cce = code_which_down(code), rot = code_rotation(code);
      const LO* ccv2v = &cv2v[(size_t)(c) * (dim + 1)];
      for (int eev = 0; eev < 2; ++eev) {
        int cev = eev ^ rot;
        int ccv = down_template(dim, 1, cce, cev);
        int ccs = opposite_template(dim, 0, ccv);
        LO csv2v[3];
        for (int csv = 0; csv < dim; ++csv) csv2v[csv] = ccv2v[down_template(dim, dim - 1, ccs, csv)];
        if (dim == 3) std::swap(csv2v[1], csv2v[2]);
        double q;
        if (dim == 3) {
          Vec3 p[4];
          Mat3 ms[4];
          for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) p[i][j] = m.coords[(size_t)(csv2v[i]) * 3 + j];
            ms[i] = symm3(&m.metric[(size_t)(csv2v[i]) * 6]);
          }
          for (int j = 0; j < 3; ++j) p[3][j] = midp[j];
          ms[3] = symm3(&mid[cand * 6]);
          q = tet_quality(p, maxdet3(ms, 4));
        } else {
          Vec2 p[3];
          Mat2 ms[3];
          for (int i = 0; i < 2; ++i) {
            for (int j = 0; j < 2; ++j) p[i][j] = m.coords[(size_t)(csv2v[i]) * 2 + j];
            ms[i] = symm2(&m.metric[(size_t)(csv2v[i]) * 3]);
          }
          for (int j = 0; j < 2; ++j) p[2][j] = midp[j];
          ms[2] = symm2(&mid[cand * 3]);
          q = tri_quality(p, maxdet2(ms, 3));
        }
        minqual = min2(minqual, q);
      }
    }
    out[cand] = minqual;
  }
  return out;
}

// refine_products (src/Omega_h_refine_topology.cpp:13-205)
static void refine_products(Mesh& m, int ed, const V<LO>& k2e, const V<LO>& k2mid,
                            const V<LO>& ov2nv, V<LO>& k2p, V<LO>& pv2v) {
  int dim = m.dim;
  LO nkeys = LO(k2e.size());
  const V<LO>& ev2v = m.ask_verts_of(1);
  V<LO> k2pairs((size_t)(nkeys) + 1, 0), pair_v;
  if (ed == EDGE) {
    for (LO k = 0; k < nkeys; ++k) {
      LO e = k2e[k];
      pair_v.push_back(ov2nv[ev2v[(size_t)(e) * 2]]);
      pair_v.push_back(k2mid[k]);
      pair_v.push_back(k2mid[k]);
      pair_v.push_back(ov2nv[ev2v[(size_t)(e) * 2 + 1]]);
      k2pairs[k + 1] = 2 * (k + 1);
    }
  } else {
    const V<LO>& dv2v = m.ask_verts_of(ed);
    const Adj& e2d = m.ask_up(1, ed);
    for (LO k = 0; k < nkeys; ++k) {
      LO e = k2e[k];
      for (LO ed_ = e2d.a2ab[e]; ed_ < e2d.a2ab[e + 1]; ++ed_) {
        LO dom = e2d.ab2b[ed_];
        I8 code = e2d.codes[ed_];
        int dde = code_which_down(code), rot = code_rotation(code);
        for (int eev = 0; eev < 2; ++eev) {
          int dev = eev ^ rot;
          int ddv = down_template(ed, 1, dde, dev);
          int dds = opposite_template(ed, 0, ddv);
          LO pv[4];
          for (int dsv = 0; dsv < ed; ++dsv)
            pv[dsv] = ov2nv[dv2v[(size_t)(dom) * (ed + 1) + down_template(ed, ed - 1, dds, dsv)]];
          pv[ed] = k2mid[k];
          if (ed == 3) std::swap(pv[1], pv[2]);
          for (int i = 0; i <= ed; ++i) pair_v.push_back(pv[i]);
        }
      }
      k2pairs[k + 1] = k2pairs[k] + 2 * (e2d.a2ab[e + 1] - e2d.a2ab[e]);
    }
  }
  if (ed == dim) {
    k2p = k2pairs;
    pv2v = pair_v;
    return;
  }
  int cd = ed + 1;  // cut domains
  const V<LO>& dv2v = m.ask_verts_of(cd);
  const Adj& e2d = m.ask_up(1, cd);
  V<LO> k2cuts((size_t)(nkeys) + 1, 0), cut_v;
  for (LO k = 0; k < nkeys; ++k) {
    LO e = k2e[k];
    for (LO ed_ = e2d.a2ab[e]; ed_ < e2d.a2ab[e + 1]; ++ed_) {
      LO dom = e2d.ab2b[ed_];
      int dde = code_which_down(e2d.codes[ed_]);
      int ddt = opposite_template(cd, 1, dde);
      for (int dtv = 0; dtv < cd - 1; ++dtv)
        cut_v.push_back(ov2nv[dv2v[(size_t)(dom) * (cd + 1) + down_template(cd, cd - 2, ddt, dtv)]]);
      cut_v.push_back(k2mid[k]);
    }
    k2cuts[k + 1] = k2cuts[k] + (e2d.a2ab[e + 1] - e2d.a2ab[e]);
  }
  int nppv = ed + 1;
  k2p.assign((size_t)(nkeys) + 1, 0);
  for (LO k = 0; k < nkeys; ++k)
    k2p[k + 1] = k2p[k] + (k2cuts[k + 1] - k2cuts[k]) + (k2pairs[k + 1] - k2pairs[k]);
  pv2v.resize((size_t)(k2p[nkeys]) * nppv);
  for (LO k = 0; k < nkeys; ++k) {
    LO prod = k2p[k];
    for (LO p = k2pairs[k]; p < k2pairs[k + 1]; ++p, ++prod)
      for (int i = 0; i < nppv; ++i) pv2v[(size_t)(prod) * nppv + i] = pair_v[(size_t)(p) * nppv + i];
    for (LO c = k2cuts[k]; c < k2cuts[k + 1]; ++c, ++prod)
      for (int i = 0; i < nppv; ++i) pv2v[(size_t)(prod) * nppv + i] = cut_v[(size_t)(c) * nppv + i];
  }
}

// refine_ghosted + refine_element_based (src/Omega_h_refine.cpp:17-82)
static bool refine(Mesh& m, const AdaptOpts& o, const V<I8>& cands) {
  int dim = m.dim, mc = m.mcomp();
  V<LO> c2e = collect_marked(cands);
  V<double> cq = refine_qualities(m, c2e);
  bool any = false;
  for (double q : cq) any |= (q >= o.min_quality_allowed);
  if (!any) return false;
  LO ne = m.nedges();
  V<I8> initial((size_t)(ne), 0);
  V<double> eq((size_t)(ne), 0.0);
  for (size_t i = 0; i < c2e.size(); ++i) {
    initial[c2e[i]] = cq[i] >= o.min_quality_allowed;
    eq[c2e[i]] = cq[i];
  }
  V<I8> keys = find_indset(m, EDGE, eq, initial);
  V<LO> k2e = collect_marked(keys);
  LO nkeys = LO(k2e.size());
  Mesh nm;
  nm.dim = dim;
  V<LO> k2mid, ov2nv, old_lows2new;
  for (int d = 0; d <= dim; ++d) {
    V<LO> k2p, pv2v;
    if (d == VERT) {
      k2p = iota_lo(nkeys + 1);
    } else {
      refine_products(m, d, k2e, k2mid, ov2nv, k2p, pv2v);
    }
    ModifyOut mo = modify_ents_adapt(m, nm, d, EDGE, k2e, k2p, pv2v, old_lows2new);
    LO nnew = nm.nents[d];
    if (d == VERT) {
      k2mid = mo.prods2new;
      ov2nv = mo.old2new;
    }
    // transfer_refine (src/Omega_h_transfer.cpp:391-436)
    V<I8> pcd((size_t)(k2p[nkeys]));
    V<LO> pci((size_t)(k2p[nkeys]));
    if (d > VERT) {
      const Adj& e2d = m.ask_up(1, d);
      for (LO k = 0; k < nkeys; ++k) {
        LO prod = k2p[k];
        if (d == EDGE) {
          for (int pr = 0; pr < 2; ++pr, ++prod) {
            pcd[prod] = m.class_dim[1][k2e[k]];
            pci[prod] = m.class_id[1][k2e[k]];
          }
        } else {
          for (LO x = e2d.a2ab[k2e[k]]; x < e2d.a2ab[k2e[k] + 1]; ++x)
            for (int pr = 0; pr < 2; ++pr, ++prod) {
              pcd[prod] = m.class_dim[d][e2d.ab2b[x]];
              pci[prod] = m.class_id[d][e2d.ab2b[x]];
            }
        }
      }
    }
    if (d < dim) {
      // cut products inherit from the (d+1)-dimensional domain they split;
      // for vertices that domain is the key edge itself (identity graph)
      for (LO k = 0; k < nkeys; ++k) {
        LO e = k2e[k];
        if (d + 1 == EDGE) {
          pcd[k2p[k + 1] - 1] = m.class_dim[1][e];
          pci[k2p[k + 1] - 1] = m.class_id[1][e];
          continue;
        }
        const Adj& e2d = m.ask_up(1, d + 1);
        LO prod = k2p[k + 1] - (e2d.a2ab[e + 1] - e2d.a2ab[e]);
        for (LO x = e2d.a2ab[e]; x < e2d.a2ab[e + 1]; ++x, ++prod) {
          pcd[prod] = m.class_dim[d + 1][e2d.ab2b[x]];
          pci[prod] = m.class_id[d + 1][e2d.ab2b[x]];
        }
      }
    }
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, pcd, 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, pci, 1);
    if (d == VERT) {
      const V<LO>& ev2v = m.ask_verts_of(1);
      V<double> pc((size_t)(nkeys) * dim);
      for (LO k = 0; k < nkeys; ++k)
        for (int j = 0; j < dim; ++j) {
          double comp = 0;
          comp += m.coords[(size_t)(ev2v[(size_t)(k2e[k]) * 2]) * dim + j];
          comp += m.coords[(size_t)(ev2v[(size_t)(k2e[k]) * 2 + 1]) * dim + j];
          comp /= 2;
          pc[(size_t)(k) * dim + j] = comp;
        }
      nm.coords = xfer(m.coords, mo, nnew, pc, dim);
      nm.metric = xfer(m.metric, mo, nnew, get_mident_metrics(m, k2e), mc);
    }
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

bool refine_by_size(Mesh& m, const AdaptOpts& o) {
  const V<double>& len = m.ask_lengths();
  V<I8> cands(len.size());
  bool any = false;
  for (size_t i = 0; i < len.size(); ++i) {
    cands[i] = len[i] > o.max_length_desired;
    any |= bool(cands[i]);
  }
  if (!any) return false;
  return refine(m, o, cands);
}

// ------------------------------------------------------------ coarsen
static inline bool collapses(I8 code, int v) { return (code & (1 << v)) != 0; }
static inline I8 dont_collapse(I8 code, int v) { return I8(code & ~(1 << v)); }

V<I8> check_collapse_class(Mesh& m, const V<LO>& c2e, const V<I8>& codes) {
  const V<LO>& ev2v = m.ask_verts_of(1);
  V<I8> out(codes.size());
  for (size_t c = 0; c < c2e.size(); ++c) {
    I8 code = codes[c];
    LO e = c2e[c];
    int vcd[2] = {m.class_dim[0][ev2v[(size_t)(e) * 2]], m.class_dim[0][ev2v[(size_t)(e) * 2 + 1]]};
    int ecd = m.class_dim[1][e];
    if (vcd[0] == vcd[1]) {
      if (vcd[0] != ecd) code = 0;
    } else {
      for (int v = 0; v < 2; ++v)
        if (collapses(codes[c], v) && vcd[v] != ecd) code = dont_collapse(code, v);
    }
    out[c] = code;
  }
  return out;
}

V<I8> check_collapse_exposure(Mesh& m, const V<LO>& c2e, const V<I8>& codes_in) {
  V<I8> codes = codes_in;
  for (int cd = 2; cd <= m.dim; ++cd) {
    const Adj& e2c = m.ask_up(1, cd);
    const V<LO>& cs2s = m.ask_down(cd, cd - 1).ab2b;
    int nccs = simplex_degree(cd, cd - 1);
    V<I8> out(codes.size());
    for (size_t cand = 0; cand < c2e.size(); ++cand) {
      I8 code = codes[cand];
      LO e = c2e[cand];
      for (LO ec = e2c.a2ab[e]; ec < e2c.a2ab[e + 1]; ++ec) {
        LO c = e2c.ab2b[ec];
        I8 ecc = e2c.codes[ec];
        int cce = code_which_down(ecc), rot = code_rotation(ecc);
        int c_dim = m.class_dim[cd][c];
        for (int col = 0; col < 2; ++col) {
          if (!collapses(code, col)) continue;
          int onto = 1 - col;
          int cev_onto = rot ^ onto;
          int ccv_onto = down_template(cd, 1, cce, cev_onto);
          int ccs_opp = opposite_template(cd, 0, ccv_onto);
          LO s_opp = cs2s[(size_t)(c) * nccs + ccs_opp];
          if (m.class_dim[cd - 1][s_opp] != c_dim) code = dont_collapse(code, col);
        }
      }
      out[cand] = code;
    }
    codes = out;
  }
  return codes;
}

V<I8> prevent_coarsen_overshoot(Mesh& m, double max_length, const V<LO>& c2e,
                                const V<I8>& codes) {
  const V<LO>& ev2v = m.ask_verts_of(1);
  const Adj& v2e = m.ask_up(0, 1);
  int dim = m.dim, mc = m.mcomp();
  V<I8> out(codes.size());
  ORC_PARALLEL_FOR
  for (size_t cand = 0; cand < c2e.size(); ++cand) {
    LO e = c2e[cand];
    I8 code = codes[cand];
    for (int col = 0; col < 2; ++col) {
      if (!collapses(code, col)) continue;
      LO v_col = ev2v[(size_t)(e) * 2 + col];
      LO v_onto = ev2v[(size_t)(e) * 2 + (1 - col)];
      for (LO ve = v2e.a2ab[v_col]; ve < v2e.a2ab[v_col + 1]; ++ve) {
        LO e2 = v2e.ab2b[ve];
        if (e2 == e) continue;
        int ein = code_which_down(v2e.codes[ve]), eout = 1 - ein;
        LO nv[2];
        nv[ein] = v_onto;
        nv[eout] = ev2v[(size_t)(e2) * 2 + eout];
        const double* p0 = &m.coords[(size_t)(nv[0]) * dim];
        const double* p1 = &m.coords[(size_t)(nv[1]) * dim];
        const double* m0 = &m.metric[(size_t)(nv[0]) * mc];
        const double* m1 = &m.metric[(size_t)(nv[1]) * mc];
        double len = dim == 3 ? edge_length3(p0, p1, m0, m1) : edge_length2(p0, p1, m0, m1);
        if (len >= max_length) {
          code = dont_collapse(code, col);
          break;
        }
      }
    }
    out[cand] = code;
  }
  return out;
}

V<double> coarsen_qualities(Mesh& m, const V<LO>& c2e, const V<I8>& codes) {
  int dim = m.dim;
  const V<LO>& ev2v = m.ask_verts_of(1);
  const V<LO>& cv2v = m.ask_verts_of(dim);
  const Adj& v2c = m.ask_up(0, dim);
  V<double> q(c2e.size() * 2, -1.0);
  ORC_PARALLEL_FOR
  for (size_t cand = 0; cand < c2e.size(); ++cand) {
    LO e = c2e[cand];
    I8 code = codes[cand];
    for (int col = 0; col < 2; ++col) {
      if (!collapses(code, col)) continue;
      LO v_col = ev2v[(size_t)(e) * 2 + col];
      LO v_onto = ev2v[(size_t)(e) * 2 + (1 - col)];
      double minqual = 1.0;
      for (LO vc = v2c.a2ab[v_col]; vc < v2c.a2ab[v_col + 1]; ++vc) {
        LO c = v2c.ab2b[vc];
        int ccv_col = code_which_down(v2c.codes[vc]);
        LO cv[4];
        for (int k = 0; k <= dim; ++k) cv[k] = cv2v[(size_t)(c) * (dim + 1) + k];
        bool will_die = false;
        for (int k = 0; k <= dim; ++k)
          if (k != ccv_col && cv[k] == v_onto) {
            will_die = true;
            break;
          }
        if (will_die) continue;
        cv[ccv_col] = v_onto;
        minqual = min2(minqual, elem_quality(m, cv));
      }
      q[cand * 2 + col] = minqual;
    }
  }
  return q;
}

void choose_rails(Mesh& m, const V<LO>& c2e, const V<I8>& codes, const V<double>& quals,
                  V<I8>* vc, V<double>* vq, V<GO>* vr) {
  V<LO> e2c((size_t)(m.nedges()), -1);
  for (size_t i = 0; i < c2e.size(); ++i) e2c[c2e[i]] = LO(i);
  const Adj& v2e = m.ask_up(0, 1);
  const V<double>& lengths = m.ask_lengths();
  LO nv = m.nverts();
  vc->assign((size_t)(nv), 0);
  vq->assign((size_t)(nv), 0.0);
  vr->assign((size_t)(nv), 0);
  ORC_PARALLEL_FOR
  for (LO v = 0; v < nv; ++v) {
    bool is_cand = false;
    GO best_global = -1;
    double best_length = -1, best_qual = -1;
    for (LO ve = v2e.a2ab[v]; ve < v2e.a2ab[v + 1]; ++ve) {
      LO e = v2e.ab2b[ve];
      LO cand = e2c[e];
      if (cand == -1) continue;
      int eev = code_which_down(v2e.codes[ve]);
      if (!collapses(codes[cand], eev)) continue;
      double length = lengths[e];
      double qual = quals[(size_t)(cand) * 2 + eev];
      if ((best_global == -1) || (length < best_length) ||
          ((length == best_length) && (qual > best_qual))) {
        is_cand = true;
        best_global = e;
        best_length = length;
        best_qual = qual;
      }
    }
    (*vc)[v] = is_cand;
    (*vq)[v] = best_qual;
    (*vr)[v] = best_global;
  }
}

// find_rails (src/Omega_h_collapse_rail.cpp:79-108)
void find_rails(Mesh& m, const V<LO>& k2v, const V<GO>& vr, V<LO>* r2e, V<I8>* rdir) {
  const Adj& v2e = m.ask_up(0, 1);
  LO nkeys = LO(k2v.size());
  r2e->assign((size_t)(nkeys), -1);
  rdir->assign((size_t)(nkeys), -1);
  for (LO k = 0; k < nkeys; ++k) {
    LO v = k2v[k];
    for (LO ve = v2e.a2ab[v]; ve < v2e.a2ab[v + 1]; ++ve)
      if (GO(v2e.ab2b[ve]) == vr[v]) {
        (*r2e)[k] = v2e.ab2b[ve];
        (*rdir)[k] = I8(code_which_down(v2e.codes[ve]));
        break;
      }
    OCHECK((*r2e)[k] >= 0);
  }
}

// mark_dead_ents (src/Omega_h_coarsen_topology.cpp:28-70)
void mark_dead_ents(Mesh& m, const V<LO>& r2e, const V<I8>& rdir, V<I8>* dead) {
  int dim = m.dim;
  dead[1] = mark_image(r2e, m.nedges());
  for (int d = 2; d <= dim; ++d) dead[d].assign((size_t)(m.nents[d]), 0);
  for (int cd = dim; cd > EDGE; --cd) {
    const Adj& e2c = m.ask_up(1, cd);
    const V<LO>& cs2s = m.ask_down(cd, cd - 1).ab2b;
    int nccs = simplex_degree(cd, cd - 1);
    for (size_t r = 0; r < r2e.size(); ++r) {
      LO e = r2e[r];
      int onto = 1 - rdir[r];
      for (LO ec = e2c.a2ab[e]; ec < e2c.a2ab[e + 1]; ++ec) {
        LO c = e2c.ab2b[ec];
        I8 ecc = e2c.codes[ec];
        int cce = code_which_down(ecc), rot = code_rotation(ecc);
        int ccv_onto = down_template(cd, 1, cce, rot ^ onto);
        int ccs_opp = opposite_template(cd, 0, ccv_onto);
        dead[cd][c] = 1;
        dead[cd - 1][cs2s[(size_t)(c) * nccs + ccs_opp]] = 1;
      }
    }
  }
}

// coarsen_by_size .. coarsen_element_based2 (src/Omega_h_coarsen.cpp:29-208)
// coarsen_verts + coarsen (src/Omega_h_coarsen.cpp:29-176, 178-196):
// collapse the marked vertices; allowed selects max_length_allowed as the
// overshoot limit, improve the filter_coarsen_improve step
// (src/Omega_h_coarsen_qualities.cpp:111-122)
static bool coarsen_verts(Mesh& m, const AdaptOpts& o, const V<I8>& vmarks, bool allowed,
                          bool improve) {
  int dim = m.dim;
  const V<LO>& ev2v = m.ask_verts_of(1);
  LO ne = m.nedges();
  V<I8> ecodes((size_t)(ne));
  for (LO e = 0; e < ne; ++e) {
    I8 code = 0;
    for (int k = 0; k < 2; ++k)
      if (vmarks[ev2v[(size_t)(e) * 2 + k]]) code = I8(code | (1 << k));
    ecodes[e] = code;
  }
  // coarsen_element_based1
  V<LO> c2e = collect_marked(ecodes);
  V<I8> codes = check_collapse_class(m, c2e, unmap(c2e, ecodes, 1));
  I8 mx = 0;
  for (I8 c : codes) mx = std::max(mx, c);
  if (mx <= 0) return false;
  std::fill(ecodes.begin(), ecodes.end(), I8(0));
  map_into(codes, c2e, ecodes, 1);
  // coarsen_ghosted
  c2e = collect_marked(ecodes);
  codes = check_collapse_exposure(m, c2e, unmap(c2e, ecodes, 1));
  auto filt = [&](V<double>* q) {
    V<LO> keep;
    for (size_t i = 0; i < codes.size(); ++i)
      if (codes[i] != 0) keep.push_back(LO(i));
    c2e = unmap(keep, c2e, 1);
    codes = unmap(keep, codes, 1);
    if (q) *q = unmap(keep, *q, 2);
  };
  filt(nullptr);
  codes = prevent_coarsen_overshoot(m, allowed ? o.max_length_allowed : o.max_length_desired,
                                    c2e, codes);
  filt(nullptr);
  if (c2e.empty()) return false;
  V<double> quals = coarsen_qualities(m, c2e, codes);
  for (size_t c = 0; c < codes.size(); ++c)
    for (int d = 0; d < 2; ++d)
      if (!(quals[c * 2 + d] >= o.min_quality_allowed)) codes[c] = dont_collapse(codes[c], d);
  if (improve) {
    // the worst element quality at each vertex (graph_reduce MIN over v2e)
    const V<double>& eq = m.ask_qualities();
    const Adj& v2c = m.ask_up(0, dim);
    V<double> vold((size_t)(m.nverts()));
    for (LO v = 0; v < m.nverts(); ++v) {
      double mq = 1.79769313486231570815e+308;
      for (LO x = v2c.a2ab[v]; x < v2c.a2ab[v + 1]; ++x) mq = min2(mq, eq[v2c.ab2b[x]]);
      vold[v] = mq;
    }
    for (size_t c = 0; c < codes.size(); ++c)
      for (int d = 0; d < 2; ++d)
        if (!(quals[c * 2 + d] > vold[ev2v[(size_t)(c2e[c]) * 2 + d]]))
          codes[c] = dont_collapse(codes[c], d);
  }
  filt(&quals);
  if (c2e.empty()) return false;
  V<I8> vc;
  V<double> vq;
  V<GO> vr;
  choose_rails(m, c2e, codes, quals, &vc, &vq, &vr);
  V<I8> vkeys = find_indset(m, VERT, vq, vc);
  // coarsen_element_based2
  V<LO> k2v = collect_marked(vkeys);
  LO nkeys = LO(k2v.size());
  V<LO> r2e;
  V<I8> rdir;
  find_rails(m, k2v, vr, &r2e, &rdir);
  V<I8> dead[4];
  mark_dead_ents(m, r2e, rdir, dead);
  V<LO> k2onto((size_t)(nkeys));
  for (LO k = 0; k < nkeys; ++k) k2onto[k] = ev2v[(size_t)(r2e[k]) * 2 + (1 - rdir[k])];
  Mesh nm;
  nm.dim = dim;
  V<LO> ov2nv, old_lows2new;
  for (int d = 0; d <= dim; ++d) {
    V<LO> k2p, pv2v, kd2d;  // keys2doms (a2ab = k2p)
    V<I8> kd_codes;
    if (d == VERT) {
      k2p.assign((size_t)(nkeys) + 1, 0);
    } else {
      // find_coarsen_domains: live entities adjacent to each key vertex
      const Adj& v2d = m.ask_up(0, d);
      k2p.assign((size_t)(nkeys) + 1, 0);
      for (LO k = 0; k < nkeys; ++k) {
        LO v = k2v[k];
        for (LO vd = v2d.a2ab[v]; vd < v2d.a2ab[v + 1]; ++vd)
          if (!dead[d][v2d.ab2b[vd]]) {
            kd2d.push_back(v2d.ab2b[vd]);
            kd_codes.push_back(v2d.codes[vd]);
          }
        k2p[k + 1] = LO(kd2d.size());
      }
      // coarsen_topology
      const V<LO>& cv2v = m.ask_verts_of(d);
      int nccv = d + 1;
      pv2v.resize(kd2d.size() * (size_t)(nccv));
      for (LO k = 0; k < nkeys; ++k)
        for (LO kc = k2p[k]; kc < k2p[k + 1]; ++kc) {
          int ccv_col = code_which_down(kd_codes[kc]);
          for (int ccv = 0; ccv < nccv; ++ccv) {
            LO ov = ccv == ccv_col ? k2onto[k] : cv2v[(size_t)(kd2d[kc]) * nccv + ccv];
            pv2v[(size_t)(kc) * nccv + ccv] = ov2nv[ov];
          }
        }
    }
    ModifyOut mo = modify_ents_adapt(m, nm, d, VERT, k2v, k2p, pv2v, old_lows2new);
    LO nnew = nm.nents[d];
    if (d == VERT) ov2nv = mo.old2new;
    // transfer_coarsen (src/Omega_h_transfer.cpp:585-620)
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, unmap(kd2d, m.class_dim[d], 1), 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, unmap(kd2d, m.class_id[d], 1), 1);
    if (d == VERT) {
      nm.coords = xfer(m.coords, mo, nnew, V<double>(), dim);
      nm.metric = xfer(m.metric, mo, nnew, V<double>(), m.mcomp());
    }
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

// coarsen_by_size (src/Omega_h_coarsen.cpp:198-208)
bool coarsen_by_size(Mesh& m, const AdaptOpts& o) {
  const V<double>& len = m.ask_lengths();
  V<I8> ecand(len.size());
  bool any = false;
  for (size_t i = 0; i < len.size(); ++i) {
    ecand[i] = len[i] < o.min_length_desired;
    any |= bool(ecand[i]);
  }
  if (!any) return false;
  return coarsen_verts(m, o, mark_down(m, EDGE, VERT, ecand), false, false);
}

// coarsen_slivers (src/Omega_h_coarsen.cpp:210-220)
bool coarsen_slivers(Mesh& m, const AdaptOpts& o) {
  V<I8> ec = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  bool any = false;
  for (I8 x : ec) any |= bool(x);
  if (!any) return false;
  return coarsen_verts(m, o, mark_down(m, m.dim, VERT, ec), true, true);
}

// ------------------------------------------------------------ swap (3D)
V<I8> mark_sliver_layers(Mesh& m, double ceil, int nlayers) {
  const V<double>& q = m.ask_qualities();
  V<I8> marks(q.size());
  ORC_PARALLEL_FOR
  for (size_t i = 0; i < q.size(); ++i) marks[i] = q[i] < ceil;
  const Adj& dual = m.ask_adj(m.dim, m.dim);
  for (int l = 0; l < nlayers; ++l) {
    V<I8> nmk(marks.size());
    ORC_PARALLEL_FOR
    for (size_t e = 0; e < marks.size(); ++e) {
      I8 r = -128;  // fan_reduce MAX starts from the lowest I8
      for (LO j = dual.a2ab[e]; j < dual.a2ab[e + 1]; ++j) r = std::max(r, marks[dual.ab2b[j]]);
      nmk[e] = r;
    }
    marks.swap(nmk);
  }
  return marks;
}

struct Loop {
  int size;
  LO eev2v[2];
  LO lv[7];
};
// swap3d::find_loop (src/Omega_h_swap3d_loop.hpp:24-78)
static Loop find_loop(Mesh& m, LO edge) {
  const Adj& e2t = m.ask_up(1, 3);
  const V<LO>& ev2v = m.ask_verts_of(1);
  const V<LO>& tv2v = m.ask_verts_of(3);
  Loop loop;
  LO b = e2t.a2ab[edge], e = e2t.a2ab[edge + 1];
  loop.size = e - b;
  if (loop.size > 7) return loop;
  OCHECK(loop.size >= 3);
  loop.eev2v[0] = ev2v[(size_t)(edge) * 2];
  loop.eev2v[1] = ev2v[(size_t)(edge) * 2 + 1];
  LO tmp[7][2];
  for (int le = 0; le < loop.size; ++le) {
    LO et = b + le;
    LO tet = e2t.ab2b[et];
    I8 code = e2t.codes[et];
    int rre = code_which_down(code), rot = code_rotation(code);
    int opp = opposite_template(3, 1, rre);
    for (int eev = 0; eev < 2; ++eev)
      tmp[le][eev] = tv2v[(size_t)(tet) * 4 + down_template(3, 1, opp, rot ^ eev)];
  }
  for (int i = 0; i < loop.size - 1; ++i) {
    int j;
    for (j = i + 1; j < loop.size; ++j)
      if (tmp[j][0] == tmp[i][1]) break;
    OCHECK(j < loop.size);
    std::swap(tmp[i + 1][0], tmp[j][0]);
    std::swap(tmp[i + 1][1], tmp[j][1]);
  }
  for (int i = 0; i < loop.size; ++i) loop.lv[i] = tmp[i][0];
  return loop;
}

void swap3d_qualities(Mesh& m, const AdaptOpts& o, const V<LO>& c2e, V<double>* quals,
                      V<I8>* configs) {
  quals->assign(c2e.size(), -1.0);
  configs->assign(c2e.size(), -1);
  m.ask_up(1, 3);  // caches used inside the parallel loop
  m.ask_verts_of(1);
  m.ask_verts_of(3);
  ORC_PARALLEL_FOR
  for (size_t cand = 0; cand < c2e.size(); ++cand) {
    Loop loop = find_loop(m, c2e[cand]);
    if (loop.size > 7) continue;
    int n = loop.size;
    int nmeshes = swap3d::mesh_count(n), ntris = swap3d::mesh_size(n);
    bool tcached[35] = {false};
    double tq[35] = {0};
    bool ecached[26] = {false};
    double el[26] = {0};
    int best = -1;
    double bestq = 0.0;
    for (int mesh = 0; mesh < nmeshes; ++mesh) {
      double mq = 1.0;
      for (int t = 0; t < ntris; ++t) {
        int u = swap3d::mesh_tri(n, mesh, t);
        if (!tcached[u]) {
          const int* tv = swap3d::triangle(n, u);
          LO tet[4];
          for (int k = 0; k < 3; ++k) tet[k] = loop.lv[tv[k]];
          double tmq = 1.0;
          for (int tt = 0; tt < 2; ++tt) {
            tet[3] = loop.eev2v[1 - tt];
            tmq = min2(tmq, elem_quality(m, tet));
            std::swap(tet[1], tet[2]);
          }
          tcached[u] = true;
          tq[u] = tmq;
        }
        mq = min2(mq, tq[u]);
        if (mq < 0.0) break;
      }
      if (mq > bestq) {
        bool over = false;
        for (int me = 0; me < swap3d::nedges(n); ++me) {
          int ue = swap3d::edge2unique(n, mesh, me);
          if (!ecached[ue]) {
            const int* ev = swap3d::unique_edge(n, ue);
            LO a = loop.lv[ev[0]], b = loop.lv[ev[1]];
            el[ue] = edge_length3(&m.coords[(size_t)(a) * 3], &m.coords[(size_t)(b) * 3],
                                  &m.metric[(size_t)(a) * 6], &m.metric[(size_t)(b) * 6]);
            ecached[ue] = true;
          }
          if (el[ue] > o.max_length_allowed) {
            over = true;
            break;
          }
        }
        if (!over) {
          best = mesh;
          bestq = mq;
        }
      }
    }
    (*configs)[cand] = I8(best);
    (*quals)[cand] = bestq;
  }
}

// swap2d_qualities_tmpl (src/Omega_h_swap2d_qualities.cpp:15-67): the two
// triangles of an interior edge, replaced by the two across the other
// diagonal (ov[0], ov[1]); -1 where that diagonal is longer than
// max_length_allowed, else the min of 1 and the two new qualities.
static void swap2d_cavity(Mesh& m, LO edge, LO ov[2]) {
  const Adj& e2t = m.ask_up(1, 2);
  const V<LO>& tv2v = m.ask_verts_of(2);
  OCHECK(e2t.a2ab[edge + 1] == 2 + e2t.a2ab[edge]);
  for (int i = 0; i < 2; ++i) {
    LO et = e2t.a2ab[edge] + i;
    I8 code = e2t.codes[et];
    int tte = code_which_down(code), rot = code_rotation(code);
    LO t = e2t.ab2b[et];
    ov[rot] = tv2v[(size_t)(t) * 3 + opposite_template(2, 1, tte)];
  }
}
V<double> swap2d_qualities(Mesh& m, const AdaptOpts& o, const V<LO>& c2e) {
  const V<LO>& ev2v = m.ask_verts_of(1);
  V<double> out(c2e.size());
  m.ask_up(1, 2);  // caches used inside the parallel loop
  m.ask_verts_of(2);
  ORC_PARALLEL_FOR
  for (size_t cand = 0; cand < c2e.size(); ++cand) {
    LO edge = c2e[cand];
    LO ov[2];
    swap2d_cavity(m, edge, ov);
    const double* p0 = &m.coords[(size_t)(ov[0]) * 2];
    const double* p1 = &m.coords[(size_t)(ov[1]) * 2];
    double l = edge_length2(p0, p1, &m.metric[(size_t)(ov[0]) * 3], &m.metric[(size_t)(ov[1]) * 3]);
    if (l > o.max_length_allowed) {
      out[cand] = -1.0;
      continue;
    }
    LO ev[2] = {ev2v[(size_t)(edge) * 2], ev2v[(size_t)(edge) * 2 + 1]};
    double minq = 1.0;
    for (int i = 0; i < 2; ++i) {
      LO ntv[3] = {ev[1 - i], ov[i], ov[1 - i]};
      minq = min2(minq, elem_quality(m, ntv));
    }
    out[cand] = minq;
  }
  return out;
}

// filter_swap_improve (src/Omega_h_swap.cpp:35-43)
V<I8> filter_swap_improve(Mesh& m, const V<LO>& c2e, const V<double>& cq) {
  const V<double>& eq = m.ask_qualities();
  const Adj& e2t = m.ask_up(1, m.dim);
  V<I8> keep(c2e.size());
  for (size_t i = 0; i < c2e.size(); ++i) {
    LO e = c2e[i];
    double old = 1.79769313486231570815e+308;
    for (LO j = e2t.a2ab[e]; j < e2t.a2ab[e + 1]; ++j) old = min2(old, eq[e2t.ab2b[j]]);
    keep[i] = cq[i] > old;
  }
  return keep;
}

// products inherit the key edge's classification; lengths and qualities
// are re-measured for products (transfer_swap, src/Omega_h_transfer.cpp)
static void swap_rebuild(Mesh& m, const V<LO>& k2e, V<LO>* k2p, V<LO>* pv2v) {
  int dim = m.dim;
  LO nkeys = LO(k2e.size());
  Mesh nm;
  nm.dim = dim;
  nm.nents[0] = m.nverts();
  nm.coords = m.coords;
  nm.metric = m.metric;
  nm.class_dim[0] = m.class_dim[0];
  nm.class_id[0] = m.class_id[0];
  V<LO> old_lows2new = iota_lo(m.nverts());
  for (int d = 1; d <= dim; ++d) {
    ModifyOut mo = modify_ents_adapt(m, nm, d, EDGE, k2e, k2p[d], pv2v[d], old_lows2new);
    LO nnew = nm.nents[d];
    V<I8> pcd((size_t)(k2p[d][nkeys]));
    V<LO> pci((size_t)(k2p[d][nkeys]));
    for (LO k = 0; k < nkeys; ++k)
      for (LO p = k2p[d][k]; p < k2p[d][k + 1]; ++p) {
        pcd[p] = m.class_dim[1][k2e[k]];
        pci[p] = m.class_id[1][k2e[k]];
      }
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, pcd, 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, pci, 1);
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
}

// swap_edges_2d (src/Omega_h_swap2d.cpp:14-80) with swap2d_topology
// (src/Omega_h_swap2d_topology.cpp:37-95): one new edge (ov[0], ov[1]) and
// two new triangles (ev[1-i], ov[i], ov[1-i]) per key
static bool swap_edges_2d(Mesh& m, const AdaptOpts& o, const V<LO>& c2e_in) {
  V<LO> c2e = c2e_in;
  V<double> cq = swap2d_qualities(m, o, c2e);
  V<I8> keepm = filter_swap_improve(m, c2e, cq);
  V<LO> keep = collect_marked(keepm);
  c2e = unmap(keep, c2e, 1);
  cq = unmap(keep, cq, 1);
  if (c2e.empty()) return false;
  LO ne = m.nedges();
  V<I8> is_cand = mark_image(c2e, ne);
  V<double> edge_q((size_t)(ne), -1.0);
  map_into(cq, c2e, edge_q, 1);
  V<I8> keys = find_indset(m, EDGE, edge_q, is_cand);
  V<LO> k2e = collect_marked(keys);
  LO nkeys = LO(k2e.size());
  const V<LO>& ev2v = m.ask_verts_of(1);
  V<LO> k2p[4], pv2v[4];
  k2p[1].resize((size_t)(nkeys) + 1);
  k2p[2].resize((size_t)(nkeys) + 1);
  for (LO k = 0; k <= nkeys; ++k) {
    k2p[1][k] = k;
    k2p[2][k] = 2 * k;
  }
  pv2v[1].resize((size_t)(nkeys) * 2);
  pv2v[2].resize((size_t)(nkeys) * 6);
  for (LO k = 0; k < nkeys; ++k) {
    LO e = k2e[k];
    LO ov[2];
    swap2d_cavity(m, e, ov);
    pv2v[1][(size_t)(k) * 2] = ov[0];
    pv2v[1][(size_t)(k) * 2 + 1] = ov[1];
    LO ev[2] = {ev2v[(size_t)(e) * 2], ev2v[(size_t)(e) * 2 + 1]};
    for (int i = 0; i < 2; ++i) {
      size_t t = (size_t)(k) * 2 + i;
      pv2v[2][t * 3] = ev[1 - i];
      pv2v[2][t * 3 + 1] = ov[i];
      pv2v[2][t * 3 + 2] = ov[1 - i];
    }
  }
  swap_rebuild(m, k2e, k2p, pv2v);
  return true;
}

// swap_edges (src/Omega_h_swap.cpp:45-53): swap_part1 (src/Omega_h_swap.cpp:
// 14-27), then swap_edges_3d (src/Omega_h_swap3d.cpp:14-84) or swap_edges_2d
bool swap_edges(Mesh& m, const AdaptOpts& o) {
  int dim = m.dim;
  V<I8> ecands = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  V<I8> edc = mark_down(m, dim, 1, ecands);
  bool any = false;
  for (size_t e = 0; e < edc.size(); ++e) {
    edc[e] = edc[e] && (m.class_dim[1][e] == dim);
    any |= bool(edc[e]);
  }
  if (!any) return false;
  V<LO> c2e = collect_marked(edc);
  if (dim == 2) return swap_edges_2d(m, o, c2e);
  V<double> cq;
  V<I8> cc;
  swap3d_qualities(m, o, c2e, &cq, &cc);
  LO ne = m.nedges();
  V<I8> econfigs((size_t)(ne), -1);
  map_into(cc, c2e, econfigs, 1);
  V<I8> keepm = filter_swap_improve(m, c2e, cq);
  V<LO> keep = collect_marked(keepm);
  c2e = unmap(keep, c2e, 1);
  cq = unmap(keep, cq, 1);
  if (c2e.empty()) return false;
  V<I8> is_cand = mark_image(c2e, ne);
  V<double> edge_q((size_t)(ne), -1.0);
  map_into(cq, c2e, edge_q, 1);
  V<I8> keys = find_indset(m, EDGE, edge_q, is_cand);
  V<LO> k2e = collect_marked(keys);
  LO nkeys = LO(k2e.size());
  // swap3d_keys_to_prods + swap3d_topology (src/Omega_h_swap3d_topology.cpp)
  V<LO> k2p[4], pv2v[4];
  for (int d = 1; d <= 3; ++d) k2p[d].assign((size_t)(nkeys) + 1, 0);
  V<Loop> loops((size_t)(nkeys));
  // the adjacencies find_loop reads, derived before the parallel loop
  m.ask_up(1, 3);
  m.ask_verts_of(1);
  m.ask_verts_of(3);
  ORC_PARALLEL_FOR
  for (LO k = 0; k < nkeys; ++k) loops[k] = find_loop(m, k2e[k]);
  for (LO k = 0; k < nkeys; ++k) {
    int n = loops[k].size;
    int npt = swap3d::mesh_size(n), npe = swap3d::nedges(n);
    k2p[1][k + 1] = k2p[1][k] + npe;
    k2p[2][k + 1] = k2p[2][k] + npt + 2 * npe;
    k2p[3][k + 1] = k2p[3][k] + 2 * npt;
  }
  for (int d = 1; d <= 3; ++d) pv2v[d].resize((size_t)(k2p[d][nkeys]) * (d + 1));
  ORC_PARALLEL_FOR
  for (LO k = 0; k < nkeys; ++k) {
    const Loop& loop = loops[k];
    int n = loop.size;
    int config = econfigs[k2e[k]];
    int npt = swap3d::mesh_size(n), npe = swap3d::nedges(n);
    for (int pe = 0; pe < npe; ++pe) {
      const int* ev = swap3d::unique_edge(n, swap3d::edge2unique(n, config, pe));
      LO pev[2] = {loop.lv[ev[0]], loop.lv[ev[1]]};
      LO pedge = k2p[1][k] + pe;
      pv2v[1][(size_t)(pedge) * 2] = pev[0];
      pv2v[1][(size_t)(pedge) * 2 + 1] = pev[1];
      for (int eev = 0; eev < 2; ++eev) {
        LO ptri = k2p[2][k] + 2 * pe + eev;
        pv2v[2][(size_t)(ptri) * 3] = pev[0];
        pv2v[2][(size_t)(ptri) * 3 + 1] = pev[1];
        pv2v[2][(size_t)(ptri) * 3 + 2] = loop.eev2v[eev];
      }
    }
    for (int pt = 0; pt < npt; ++pt) {
      const int* tv = swap3d::triangle(n, swap3d::mesh_tri(n, config, pt));
      LO ptv[3] = {loop.lv[tv[0]], loop.lv[tv[1]], loop.lv[tv[2]]};
      LO ptri = k2p[2][k] + 2 * npe + pt;
      for (int i = 0; i < 3; ++i) pv2v[2][(size_t)(ptri) * 3 + i] = ptv[i];
      for (int eev = 0; eev < 2; ++eev) {
        LO ptet = k2p[3][k] + 2 * pt + eev;
        LO tv4[4] = {ptv[0], ptv[1], ptv[2], loop.eev2v[eev]};
        if (eev == 0) std::swap(tv4[1], tv4[2]);
        for (int i = 0; i < 4; ++i) pv2v[3][(size_t)(ptet) * 4 + i] = tv4[i];
      }
    }
  }
  swap_rebuild(m, k2e, k2p, pv2v);
  return true;
}

// ------------------------------------------------------------ adapt()
// Omega_h::adapt (src/Omega_h_adapt.cpp:153-212, 272-288) without
// conservation tags or geometry
AdaptResult adapt(Mesh& m, const AdaptOpts& o) {
  AdaptResult r;
  auto minv = [](const V<double>& a) {
    double x = 1.79769313486231570815e+308;
    for (double y : a) x = min2(x, y);
    return x;
  };
  auto maxv = [](const V<double>& a) {
    double x = -1.79769313486231570815e+308;
    for (double y : a) x = std::max(x, y);
    return x;
  };
  {
    const V<double>& len = m.ask_lengths();
    if (minv(m.ask_qualities()) >= o.min_quality_desired && minv(len) >= o.min_length_desired &&
        maxv(len) <= o.max_length_desired)
      return r;
  }
  r.did = true;
  bool any;
  do {
    any = false;
    if (refine_by_size(m, o)) {
      ++r.refines;
      any = true;
    }
    if (coarsen_by_size(m, o)) {
      ++r.coarsens;
      any = true;
    }
    ++r.length_rounds;
    OCHECK(r.length_rounds <= 1000);
  } while (any);
  if (minv(m.ask_qualities()) >= o.min_quality_desired) {
    r.quality_satisfied = true;
    return r;
  }
  int rounds = 0;
  do {
    OCHECK(++rounds <= 1000);
    if (swap_edges(m, o)) {
      ++r.swaps;
      continue;
    }
    if (coarsen_slivers(m, o)) {
      ++r.sliver_coarsens;
      continue;
    }
    return r;
  } while (minv(m.ask_qualities()) < o.min_quality_desired);
  r.quality_satisfied = true;
  return r;
}

// ------------------------------------------------------------ the pass
PassResult adapt_pass(Mesh& m, const AdaptOpts& o) {
  PassResult r;
  r.did_refine = refine_by_size(m, o);
  r.did_coarsen = coarsen_by_size(m, o);
  const V<double>& q = m.ask_qualities();
  double minq = 1.79769313486231570815e+308;
  for (double x : q) minq = min2(minq, x);
  if (minq < o.min_quality_desired) r.did_swap = swap_edges(m, o);
  return r;
}

}  // namespace orc
