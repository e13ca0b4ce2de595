// Refine, coarsen and 3D edge-swap operators of one adapt pass, the
// topology rebuild (modify) and field transfer, all on device arrays.
#include <cfloat>

#include "ohg_adapt.cuh"
#include "ohg_math.cuh"

namespace ohg {

#define OHG_SWAP3D_TABLE_QUAL static
#include "ohg_swap3d_tables.inc"

AdaptOpts::AdaptOpts(int dim) {
  min_length_desired = 1.0 / std::sqrt(2.0);
  max_length_desired = std::sqrt(2.0);
  max_length_allowed = max_length_desired * 2.0;
  min_quality_allowed = dim == 3 ? 0.20 : 0.30;
  min_quality_desired = dim == 3 ? 0.30 : 0.40;
  nsliver_layers = 4;
}

__device__ __forceinline__ double elem_quality_v(int dim, const double* c, const double* mt,
                                                 const LO* v) {
  if (dim == 3) {
    V3 p[4];
    M3 ms[4];
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j < 3; ++j) p[i].x[j] = c[LO(v[i]) * 3 + j];
      ms[i] = symm3(mt + LO(v[i]) * 6);
    }
    return tet_quality(p, ms[maxdet_index3(ms, 4)]);
  }
  double p[3][2];
  int best = 0;
  double bd = det2p(mt + LO(v[0]) * 3);
  for (int i = 0; i < 3; ++i) {
    p[i][0] = c[LO(v[i]) * 2];
    p[i][1] = c[LO(v[i]) * 2 + 1];
    if (i) {
      double d = det2p(mt + LO(v[i]) * 3);
      if (d > bd) {
        best = i;
        bd = d;
      }
    }
  }
  return tri_quality(p, mt + LO(v[best]) * 3);
}

// ------------------------------------------------------------ indset
enum { NOT_IN = 0, IN = 1, UNKNOWN = 2 };
constexpr int kMaxIndsetRounds = 4096;

Arr<I8> find_indset(const Adj& g, LO n, const Arr<double>& quality, const Arr<I8>& cands,
                    int* rounds_out) {
  Ctx& c = ctx();
  Arr<I8> a(n), b(n);
  const I8* cd = cands.data();
  I8* s0 = a.data();
  pfor(n, [=] __device__(LO i) { s0[i] = cd[i] ? UNKNOWN : NOT_IN; });
  Arr<int> flag(1);
  int* fl = flag.data();
  const LO* xa = g.a2ab.data();
  const LO* xb = g.ab2b.data();
  const double* q = quality.data();
  int rounds = 0;
  int any = count_marked(cands) > 0;
  while (any) {
    if (rounds >= kMaxIndsetRounds) throw Error(5, "independent set did not converge");
    OHG_CUDA(cudaMemsetAsync(fl, 0, sizeof(int), c.stream));
    const I8* old = a.data();
    I8* nw = b.data();
    pfor(n, [=] __device__(LO v) {
      I8 sv = old[v];
      if (sv != UNKNOWN) {
        nw[v] = sv;
        return;
      }
      LO beg = xa[v], end = xa[v + 1];
      for (LO j = beg; j < end; ++j)
        if (old[xb[j]] == IN) {
          nw[v] = NOT_IN;
          return;
        }
      double qv = q[v];
      for (LO j = beg; j < end; ++j) {
        LO u = xb[j];
        if (old[u] == NOT_IN) continue;
        double qu = q[u];
        bool less = (qu != qv) ? (qu < qv) : (u < v);
        if (!less) {
          nw[v] = UNKNOWN;
          *fl = 1;
          return;
        }
      }
      nw[v] = IN;
    });
    std::swap(a, b);
    ++rounds;
    OHG_CUDA(cudaMemcpyAsync(c.h_pinned, fl, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    any = c.h_pinned[0];
  }
  if (rounds_out) *rounds_out += rounds;
  return a;
}
Arr<I8> find_indset(Mesh& m, int d, const Arr<double>& q, const Arr<I8>& cands, int* rounds) {
  if (d == m.dim) return cands;
  return find_indset(m.ask_adj(d, d), m.nents[d], q, cands, rounds);
}

// ------------------------------------------------------------ marks
static Arr<I8> mark_up(Mesh& m, int ld, int hd, const Arr<I8>& lm) {
  const LO* hl = m.ask_down(hd, ld).ab2b.data();
  int deg = simplex_degree(hd, ld);
  Arr<I8> out(m.nents[hd]);
  const I8* l = lm.data();
  I8* o = out.data();
  pfor(m.nents[hd], [=] __device__(LO h) {
    I8 r = 0;
    for (int k = 0; k < deg; ++k)
      if (l[hl[h * deg + k]]) r = 1;
    o[h] = r;
  });
  return out;
}
static Arr<I8> mark_down(Mesh& m, int hd, int ld, const Arr<I8>& hm) {
  const Adj& l2h = m.ask_up(ld, hd);
  const LO* a = l2h.a2ab.data();
  const LO* b = l2h.ab2b.data();
  const I8* h = hm.data();
  Arr<I8> out(m.nents[ld]);
  I8* o = out.data();
  pfor(m.nents[ld], [=] __device__(LO l) {
    I8 r = 0;
    for (LO x = a[l]; x < a[l + 1]; ++x)
      if (h[b[x]]) r = 1;
    o[l] = r;
  });
  return out;
}

// ------------------------------------------------------------ modify
struct ModifyOut {
  Arr<LO> prods2new, same2old, same2new, old2new;
};

// modify_ents_adapt / modify_ents / modify_conn (src/Omega_h_modify.cpp:20-70,
// 141-517) for one entity dimension; global numbers equal local numbers on
// one device, so the local numbering is the global numbering
static ModifyOut modify_ents_adapt(Mesh& om, Mesh& nm, int ent_dim, int key_dim,
                                   const Arr<LO>& keys2kds, const Arr<LO>& keys2prods,
                                   const Arr<LO>& prod_verts2verts,
                                   const Arr<LO>& old_lows2new_lows) {
  int dim = om.dim;
  LO nkeys = keys2kds.size();
  ModifyOut out;
  LO nold = om.nents[ent_dim];
  Arr<I8> mods_ent;
  if (ent_dim >= key_dim) {
    Arr<I8> km = mark_image(keys2kds, om.nents[key_dim]);
    mods_ent = ent_dim == key_dim ? km : mark_up(om, key_dim, ent_dim, km);
    Arr<I8> same(nold);
    const I8* me = mods_ent.data();
    I8* sm = same.data();
    pfor(nold, [=] __device__(LO e) { sm[e] = !me[e]; });
    out.same2old = collect_marked(same);
  } else {
    out.same2old = iota(nold);
  }
  // representatives (get_mods2reps)
  Arr<LO> reps(nkeys);
  {
    const LO* kd = keys2kds.data();
    LO* r = reps.data();
    if (key_dim == ent_dim) {
      r = nullptr;
      reps = keys2kds;
    } else if (ent_dim > key_dim) {
      const Adj& up = om.ask_up(key_dim, ent_dim);
      const LO* ua = up.a2ab.data();
      const LO* ub = up.ab2b.data();
      int* stw = ctx().d_status;
      pfor(nkeys, [=] __device__(LO k) {
        LO b = ua[kd[k]];
        if (b == ua[kd[k] + 1]) {
          raise_status(stw, ST_TOPOLOGY);
          r[k] = 0;
        } else {
          r[k] = ub[b];
        }
      });
    } else {
      const LO* dn = om.ask_down(key_dim, ent_dim).ab2b.data();
      int deg = simplex_degree(key_dim, ent_dim);
      pfor(nkeys, [=] __device__(LO k) { r[k] = dn[LO(kd[k]) * deg]; });
    }
  }
  Arr<LO> counts = fill<LO>(nold, 0);
  {
    LO* ct = counts.data();
    const LO* s2o = out.same2old.data();
    pfor(out.same2old.size(), [=] __device__(LO i) { ct[s2o[i]] = 1; });
    const LO* r = reps.data();
    const LO* kp = keys2prods.data();
    pfor(nkeys, [=] __device__(LO k) { atomicAdd(&ct[r[k]], kp[k + 1] - kp[k]); });
  }
  Arr<LO> offs = offset_scan(counts);
  LO nnew = last(offs);
  bool has_order = key_dim > ent_dim;
  Arr<LO> order;
  if (has_order) {
    // get_rep2md_order (src/Omega_h_modify.cpp:283-338)
    order = fill<LO>(om.nents[key_dim], -1);
    Arr<LO> md2mod = fill<LO>(om.nents[key_dim], -1);
    LO* m2m = md2mod.data();
    const LO* kd = keys2kds.data();
    pfor(nkeys, [=] __device__(LO k) { m2m[kd[k]] = k; });
    const Adj& r2m = om.ask_up(ent_dim, key_dim);
    const LO* ra = r2m.a2ab.data();
    const LO* rb = r2m.ab2b.data();
    const I8* rc = r2m.codes.data();
    const LO* kp = keys2prods.data();
    LO* ord = order.data();
    pfor(nold, [=] __device__(LO rep) {
      LO offset = 0;
      for (LO x = ra[rep]; x < ra[rep + 1]; ++x) {
        LO md = rb[x];
        LO mod = m2m[md];
        if (mod >= 0 && code_which_down(rc[x]) == 0) {
          ord[md] = offset;
          offset += kp[mod + 1] - kp[mod];
        }
      }
    });
  }
  out.same2new = unmap(out.same2old, offs, 1);
  out.prods2new = Arr<LO>(last(keys2prods));
  {
    const LO* of = offs.data();
    const LO* r = reps.data();
    const LO* kp = keys2prods.data();
    const LO* kd = keys2kds.data();
    const LO* ord = has_order ? order.data() : nullptr;
    LO* p2n = out.prods2new.data();
    int self = has_order ? 1 : 0;
    pfor(nkeys, [=] __device__(LO k) {
      LO offset = of[r[k]] + self;
      if (ord) offset += ord[kd[k]];
      for (LO p = kp[k]; p < kp[k + 1]; ++p) p2n[p] = offset++;
    });
  }
  out.old2new = map_onto(out.same2new, out.same2old, nold, LO(-1), 1);
  if (ent_dim == VERT) {
    nm.nents[0] = nnew;
    return out;
  }
  int ld = ent_dim - 1;
  int deg = simplex_degree(ent_dim, ld);
  const Adj& od = om.ask_down(ent_dim, ld);
  Adj nd;
  // zero-filled so that every slot holds a valid index even if a caller's
  // keys were not independent (the writes below then overlap)
  nd.ab2b = fill<LO>(nnew * deg, 0);
  LO nprods = out.prods2new.size();
  Adj pd;
  if (ld > VERT) {
    pd = reflect_down(prod_verts2verts, nprods, nm.ask_verts_of(ld), nm.ask_up(VERT, ld), ent_dim,
                      ld);
  } else {
    pd.ab2b = prod_verts2verts;
  }
  map_into(pd.ab2b, out.prods2new, nd.ab2b, deg);
  {
    const LO* s2o = out.same2old.data();
    const LO* s2n = out.same2new.data();
    const LO* ob = od.ab2b.data();
    const LO* l2n = old_lows2new_lows.data();
    LO* nb = nd.ab2b.data();
    pfor(out.same2old.size(), [=] __device__(LO i) {
      for (int k = 0; k < deg; ++k) nb[LO(s2n[i]) * deg + k] = l2n[ob[LO(s2o[i]) * deg + k]];
    });
  }
  if (ld > VERT) {
    nd.codes = fill<I8>(nnew * deg, 0);
    nd.has_codes = true;
    map_into(unmap(out.same2old, od.codes, deg), out.same2new, nd.codes, deg);
    map_into(pd.codes, out.prods2new, nd.codes, deg);
  }
  nm.set_ents(ent_dim, std::move(nd));
  return out;
}

// transfer_common (src/Omega_h_transfer.cpp:160-180)
template <class T>
static Arr<T> xfer(const Arr<T>& old, const ModifyOut& mo, LO nnew, const Arr<T>& prod, int w) {
  Arr<T> nd(nnew * w);
  if (prod.size()) map_into(prod, mo.prods2new, nd, w);
  const LO* s2o = mo.same2old.data();
  const LO* s2n = mo.same2new.data();
  const T* o = old.data();
  T* d = nd.data();
  pfor(mo.same2old.size(), [=] __device__(LO i) {
    for (int j = 0; j < w; ++j) d[LO(s2n[i]) * w + j] = o[LO(s2o[i]) * w + j];
  });
  return nd;
}

static void xfer_lengths_qualities(Mesh& om, Mesh& nm, int d, const ModifyOut& mo) {
  LO np = mo.prods2new.size();
  if (d == EDGE && om.has_length) {
    Arr<double> pl(np);
    measure_edges_metric(nm, mo.prods2new.data(), np, pl.data());
    nm.length = xfer(om.length, mo, nm.nents[1], pl, 1);
    nm.has_length = true;
  }
  if (d == om.dim && om.has_quality) {
    Arr<double> pq(np);
    measure_qualities(nm, mo.prods2new.data(), np, pq.data());
    nm.quality = xfer(om.quality, mo, nm.nents[d], pq, 1);
    nm.has_quality = true;
  }
}

// ------------------------------------------------------------ refine
// refine_qualities_tmpl (src/Omega_h_refine_qualities.cpp:34-86): one thread
// per candidate edge, two child simplices per adjacent element
void refine_qualities(Mesh& m, const LO* c2e, LO n, const double* mid, double* out) {
  int dim = m.dim;
  const LO* ev = m.ask_verts_of(1).data();
  const LO* cv = m.ask_verts_of(dim).data();
  const Adj& e2c = m.ask_up(1, dim);
  const LO* ea = e2c.a2ab.data();
  const LO* eb = e2c.ab2b.data();
  const I8* ec = e2c.codes.data();
  const double* c = m.coords.data();
  const double* mt = m.metric.data();
  pfor(n, [=] __device__(LO cand) {
    LO e = c2e[cand];
    LO v0 = ev[e * 2], v1 = ev[e * 2 + 1];
    double midp[3];
    for (int j = 0; j < dim; ++j) midp[j] = (c[v0 * dim + j] + c[v1 * dim + j]) / 2.;
    double minq = 1.0;
    for (LO x = ea[e]; x < ea[e + 1]; ++x) {
      LO el = eb[x];
      I8 code = ec[x];
      int cce = code_which_down(code), rot = code_rotation(code);
      const LO* ccv2v = cv + el * (dim + 1);
      for (int eev = 0; eev < 2; ++eev) {
        int ccv = down_template(dim, 1, cce, eev ^ rot);
        int ccs = opposite_template(dim, 0, ccv);
        LO sv[3];
        for (int k = 0; k < dim; ++k) sv[k] = ccv2v[down_template(dim, dim - 1, ccs, k)];
        double q;
        if (dim == 3) {
          LO t = sv[1];
          sv[1] = sv[2];
          sv[2] = t;
          V3 p[4];
          M3 ms[4];
          for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) p[i].x[j] = c[LO(sv[i]) * 3 + j];
            ms[i] = symm3(mt + LO(sv[i]) * 6);
          }
          for (int j = 0; j < 3; ++j) p[3].x[j] = midp[j];
          ms[3] = symm3(mid + LO(cand) * 6);
          q = tet_quality(p, ms[maxdet_index3(ms, 4)]);
        } else {
          double p[3][2];
          const double* mm[3];
          for (int i = 0; i < 2; ++i) {
            p[i][0] = c[LO(sv[i]) * 2];
            p[i][1] = c[LO(sv[i]) * 2 + 1];
            mm[i] = mt + LO(sv[i]) * 3;
          }
          p[2][0] = midp[0];
          p[2][1] = midp[1];
          mm[2] = mid + LO(cand) * 3;
          int best = 0;
          double bd = det2p(mm[0]);
          for (int i = 1; i < 3; ++i) {
            double d = det2p(mm[i]);
            if (d > bd) {
              best = i;
              bd = d;
            }
          }
          q = tri_quality(p, mm[best]);
        }
        minq = min2d(minq, q);
      }
    }
    out[cand] = minq;
  });
}

// refine_products (src/Omega_h_refine_topology.cpp:13-205): per key, the two
// halves of every adjacent d-entity ("pairs"), then the (d+1)-entities'
// mid-cuts ("cuts")
static void refine_products(Mesh& m, int ed, const Arr<LO>& k2e, const Arr<LO>& k2mid,
                            const Arr<LO>& ov2nv, Arr<LO>& k2p, Arr<LO>& pv2v) {
  int dim = m.dim;
  LO nkeys = k2e.size();
  const LO* ke = k2e.data();
  const LO* km = k2mid.data();
  const LO* o2n = ov2nv.data();
  const LO* ev = m.ask_verts_of(1).data();
  const LO *pa = nullptr, *pb = nullptr, *ca = nullptr, *cb = nullptr;
  const I8 *pc = nullptr, *cc = nullptr;
  const LO *pdv = nullptr, *cdv = nullptr;
  if (ed > EDGE) {
    const Adj& e2d = m.ask_up(1, ed);
    pa = e2d.a2ab.data();
    pb = e2d.ab2b.data();
    pc = e2d.codes.data();
    pdv = m.ask_verts_of(ed).data();
  }
  int cd = ed + 1;
  if (ed < dim) {
    const Adj& e2c = m.ask_up(1, cd);
    ca = e2c.a2ab.data();
    cb = e2c.ab2b.data();
    cc = e2c.codes.data();
    cdv = m.ask_verts_of(cd).data();
  }
  Arr<LO> cnt(nkeys);
  LO* ct = cnt.data();
  pfor(nkeys, [=] __device__(LO k) {
    LO e = ke[k];
    LO np = ed == EDGE ? 2 : 2 * (pa[e + 1] - pa[e]);
    if (ed < dim) np += ca[e + 1] - ca[e];
    ct[k] = np;
  });
  k2p = offset_scan(cnt);
  int nppv = ed + 1;
  pv2v = Arr<LO>(last(k2p) * nppv);
  const LO* kp = k2p.data();
  LO* pv = pv2v.data();
  pfor(nkeys, [=] __device__(LO k) {
    LO e = ke[k];
    LO prod = kp[k];
    LO mid = km[k];
    if (ed == EDGE) {
      LO* o = pv + prod * 2;
      o[0] = o2n[ev[e * 2]];
      o[1] = mid;
      o[2] = mid;
      o[3] = o2n[ev[e * 2 + 1]];
      prod += 2;
    } else {
      for (LO x = pa[e]; x < pa[e + 1]; ++x) {
        LO dom = pb[x];
        int dde = code_which_down(pc[x]), rot = code_rotation(pc[x]);
        for (int eev = 0; eev < 2; ++eev) {
          int ddv = down_template(ed, 1, dde, eev ^ rot);
          int dds = opposite_template(ed, 0, ddv);
          LO* o = pv + prod * nppv;
          for (int k2 = 0; k2 < ed; ++k2) o[k2] = o2n[pdv[dom * (ed + 1) + down_template(ed, ed - 1, dds, k2)]];
          o[ed] = mid;
          if (ed == 3) {
            LO t = o[1];
            o[1] = o[2];
            o[2] = t;
          }
          ++prod;
        }
      }
    }
    if (ed < dim) {
      for (LO x = ca[e]; x < ca[e + 1]; ++x) {
        LO dom = cb[x];
        int ddt = opposite_template(cd, 1, code_which_down(cc[x]));
        LO* o = pv + prod * nppv;
        for (int k2 = 0; k2 < cd - 1; ++k2)
          o[k2] = o2n[cdv[dom * (cd + 1) + down_template(cd, cd - 2, ddt, k2)]];
        o[cd - 1] = mid;
        ++prod;
      }
    }
  });
}

template <class T>
static void inherit_refine(Mesh& m, int d, const Arr<LO>& k2e, const Arr<LO>& k2p,
                           const Arr<T>* data, Arr<T>& prod) {
  // class tags: pairs inherit their split d-entity, cuts their (d+1)-entity
  // (transfer_inherit_refine, src/Omega_h_transfer.cpp:213-263)
  int dim = m.dim;
  LO nkeys = k2e.size();
  const LO* ke = k2e.data();
  const LO* kp = k2p.data();
  const LO *pa = nullptr, *pb = nullptr, *ca = nullptr, *cb = nullptr;
  if (d > EDGE) {
    const Adj& a = m.ask_up(1, d);
    pa = a.a2ab.data();
    pb = a.ab2b.data();
  }
  if (d + 1 > EDGE && d < dim) {
    const Adj& a = m.ask_up(1, d + 1);
    ca = a.a2ab.data();
    cb = a.ab2b.data();
  }
  const T* pdat = d > VERT ? data[d].data() : nullptr;
  const T* cdat = d < dim ? data[d + 1].data() : nullptr;
  const T* edat = data[1].data();
  T* o = prod.data();
  pfor(nkeys, [=] __device__(LO k) {
    LO e = ke[k];
    LO p = kp[k];
    if (d == EDGE) {
      o[p++] = edat[e];
      o[p++] = edat[e];
    } else if (d > EDGE) {
      for (LO x = pa[e]; x < pa[e + 1]; ++x) {
        o[p++] = pdat[pb[x]];
        o[p++] = pdat[pb[x]];
      }
    }
    if (d < dim) {
      if (d + 1 == EDGE) {
        o[p++] = cdat[e];
      } else {
        for (LO x = ca[e]; x < ca[e + 1]; ++x) o[p++] = cdat[cb[x]];
      }
    }
  });
}

static bool refine(Mesh& m, const AdaptOpts& o, const Arr<I8>& cands, PassStats* st) {
  int dim = m.dim, mc = m.mcomp();
  Arr<LO> c2e = collect_marked(cands);
  LO nc = c2e.size();
  Arr<double> mid(nc * mc);
  mident_metrics(m, c2e.data(), nc, mid.data());
  Arr<double> cq(nc);
  refine_qualities(m, c2e.data(), nc, mid.data(), cq.data());
  LO ne = m.nedges();
  Arr<I8> initial = fill<I8>(ne, 0);
  Arr<double> eq = fill<double>(ne, 0.0);
  Arr<int> anyg = fill<int>(1, 0);
  {
    const LO* ce = c2e.data();
    const double* q = cq.data();
    I8* in = initial.data();
    double* e = eq.data();
    int* ag = anyg.data();
    double mqa = o.min_quality_allowed;
    pfor(nc, [=] __device__(LO i) {
      bool g = q[i] >= mqa;
      in[ce[i]] = g;
      e[ce[i]] = q[i];
      if (g) *ag = 1;
    });
  }
  if (!get_elem(anyg, 0)) return false;
  Arr<I8> keys = find_indset(m, EDGE, eq, initial, &st->indset_rounds);
  Arr<LO> k2e = collect_marked(keys);
  LO nkeys = k2e.size();
  st->refine_keys = nkeys;
  Mesh nm;
  nm.dim = dim;
  Arr<LO> k2mid, ov2nv, old_lows2new;
  for (int d = 0; d <= dim; ++d) {
    Arr<LO> k2p, pv2v;
    if (d == VERT) {
      k2p = iota(nkeys + 1);
    } else {
      refine_products(m, d, k2e, k2mid, ov2nv, k2p, pv2v);
    }
    ModifyOut mo = modify_ents_adapt(m, nm, d, EDGE, k2e, k2p, pv2v, old_lows2new);
    LO nnew = nm.nents[d];
    if (d == VERT) {
      k2mid = mo.prods2new;
      ov2nv = mo.old2new;
    }
    LO np = mo.prods2new.size();
    Arr<I8> pcd(np);
    Arr<LO> pci(np);
    inherit_refine(m, d, k2e, k2p, m.class_dim, pcd);
    inherit_refine(m, d, k2e, k2p, m.class_id, pci);
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, pcd, 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, pci, 1);
    if (d == VERT) {
      Arr<double> pc(nkeys * dim);
      const LO* ev = m.ask_verts_of(1).data();
      const LO* ke = k2e.data();
      const double* c = m.coords.data();
      double* p = pc.data();
      pfor(nkeys, [=] __device__(LO k) {
        LO e = ke[k];
        for (int j = 0; j < dim; ++j) {
          double comp = 0;
          comp += c[LO(ev[e * 2]) * dim + j];
          comp += c[LO(ev[e * 2 + 1]) * dim + j];
          comp /= 2;
          p[k * dim + j] = comp;
        }
      });
      nm.coords = xfer(m.coords, mo, nnew, pc, dim);
      Arr<double> pm(nkeys * mc);
      mident_metrics(m, k2e.data(), nkeys, pm.data());
      nm.metric = xfer(m.metric, mo, nnew, pm, mc);
    }
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

bool refine_by_size(Mesh& m, const AdaptOpts& o, PassStats* st) {
  const Arr<double>& len = m.ask_lengths();
  Arr<I8> cands(len.size());
  const double* l = len.data();
  I8* c = cands.data();
  double mx = o.max_length_desired;
  pfor(len.size(), [=] __device__(LO i) { c[i] = l[i] > mx; });
  if (count_marked(cands) == 0) return false;
  return refine(m, o, cands, st);
}

// ------------------------------------------------------------ coarsen
__device__ __forceinline__ bool collapses(I8 code, int v) { return (code & (1 << v)) != 0; }
__device__ __forceinline__ I8 dont_collapse(I8 code, int v) { return I8(code & ~(1 << v)); }

// check_collapse_class (src/Omega_h_check_collapse.cpp:10-45)
void check_collapse_class(Mesh& m, const LO* c2e, LO n, const I8* ci, I8* co) {
  const LO* ev = m.ask_verts_of(1).data();
  const I8* vcd = m.class_dim[0].data();
  const I8* ecd = m.class_dim[1].data();
  pfor(n, [=] __device__(LO c) {
    I8 code = ci[c];
    LO e = c2e[c];
    int v0 = vcd[ev[e * 2]], v1 = vcd[ev[e * 2 + 1]], ed = ecd[e];
    if (v0 == v1) {
      if (v0 != ed) code = 0;
    } else {
      if (collapses(ci[c], 0) && v0 != ed) code = dont_collapse(code, 0);
      if (collapses(ci[c], 1) && v1 != ed) code = dont_collapse(code, 1);
    }
    co[c] = code;
  });
}

// check_collapse_exposure (src/Omega_h_check_collapse.cpp:69-119)
void check_collapse_exposure(Mesh& m, const LO* c2e, LO n, const I8* ci, I8* co) {
  Arr<I8> tmp(n);
  const I8* in = ci;
  for (int cd = 2; cd <= m.dim; ++cd) {
    I8* out = cd == m.dim ? co : tmp.data();
    const Adj& e2c = m.ask_up(1, cd);
    const LO* ea = e2c.a2ab.data();
    const LO* eb = e2c.ab2b.data();
    const I8* ecc = e2c.codes.data();
    const LO* cs = m.ask_down(cd, cd - 1).ab2b.data();
    const I8* cdim = m.class_dim[cd].data();
    const I8* sdim = m.class_dim[cd - 1].data();
    int nccs = simplex_degree(cd, cd - 1);
    pfor(n, [=] __device__(LO c) {
      I8 code = in[c];
      LO e = c2e[c];
      for (LO x = ea[e]; x < ea[e + 1]; ++x) {
        LO el = eb[x];
        int cce = code_which_down(ecc[x]), rot = code_rotation(ecc[x]);
        int cdv = cdim[el];
        for (int col = 0; col < 2; ++col) {
          if (!collapses(code, col)) continue;
          int ccv = down_template(cd, 1, cce, rot ^ (1 - col));
          LO s = cs[el * nccs + opposite_template(cd, 0, ccv)];
          if (sdim[s] != cdv) code = dont_collapse(code, col);
        }
      }
      out[c] = code;
    });
    in = out;
  }
}

// prevent_coarsen_overshoot (src/Omega_h_coarsen_overshoot.cpp:11-49)
void prevent_coarsen_overshoot(Mesh& m, double max_length, const LO* c2e, LO n, const I8* ci,
                               I8* co) {
  const LO* ev = m.ask_verts_of(1).data();
  const Adj& v2e = m.ask_up(0, 1);
  const LO* va = v2e.a2ab.data();
  const LO* vb = v2e.ab2b.data();
  const I8* vc = v2e.codes.data();
  const double* c = m.coords.data();
  const double* mt = m.metric.data();
  int dim = m.dim, mc = m.mcomp();
  pfor(n, [=] __device__(LO cand) {
    LO e = c2e[cand];
    I8 code = ci[cand];
    for (int col = 0; col < 2; ++col) {
      if (!collapses(code, col)) continue;
      LO v_col = ev[e * 2 + col], v_onto = ev[e * 2 + (1 - col)];
      for (LO x = va[v_col]; x < va[v_col + 1]; ++x) {
        LO e2 = vb[x];
        if (e2 == e) continue;
        int ein = code_which_down(vc[x]), eout = 1 - ein;
        LO nv[2];
        nv[ein] = v_onto;
        nv[eout] = ev[e2 * 2 + eout];
        double len = dim == 3 ? edge_length3(c + nv[0] * 3, c + nv[1] * 3, mt + nv[0] * mc, mt + nv[1] * mc)
                              : edge_length2(c + nv[0] * 2, c + nv[1] * 2, mt + nv[0] * mc, mt + nv[1] * mc);
        if (len >= max_length) {
          code = dont_collapse(code, col);
          break;
        }
      }
    }
    co[cand] = code;
  });
}

// coarsen_qualities_tmpl (src/Omega_h_coarsen_qualities.cpp:15-63)
void coarsen_qualities(Mesh& m, const LO* c2e, LO n, const I8* codes, double* q2) {
  int dim = m.dim;
  const LO* ev = m.ask_verts_of(1).data();
  const LO* cv = m.ask_verts_of(dim).data();
  const Adj& v2c = m.ask_up(0, dim);
  const LO* va = v2c.a2ab.data();
  const LO* vb = v2c.ab2b.data();
  const I8* vc = v2c.codes.data();
  const double* c = m.coords.data();
  const double* mt = m.metric.data();
  pfor(n, [=] __device__(LO cand) {
    LO e = c2e[cand];
    I8 code = codes[cand];
    for (int col = 0; col < 2; ++col) {
      q2[cand * 2 + col] = -1.0;
      if (!collapses(code, col)) continue;
      LO v_col = ev[e * 2 + col], v_onto = ev[e * 2 + (1 - col)];
      double minq = 1.0;
      for (LO x = va[v_col]; x < va[v_col + 1]; ++x) {
        LO el = vb[x];
        int ccv_col = code_which_down(vc[x]);
        LO vv[4];
        for (int k = 0; k <= dim; ++k) vv[k] = cv[el * (dim + 1) + k];
        bool dies = false;
        for (int k = 0; k <= dim; ++k)
          if (k != ccv_col && vv[k] == v_onto) dies = true;
        if (dies) continue;
        vv[ccv_col] = v_onto;
        minq = min2d(minq, elem_quality_v(dim, c, mt, vv));
      }
      q2[cand * 2 + col] = minq;
    }
  });
}

// choose_rails (src/Omega_h_collapse_rail.cpp:15-67)
void choose_rails(Mesh& m, const LO* c2e, LO n, const I8* codes, const double* quals2,
                  I8* vcand, double* vqual, GO* vrail) {
  Arr<LO> e2c = fill<LO>(m.nedges(), -1);
  LO* ec = e2c.data();
  pfor(n, [=] __device__(LO i) { ec[c2e[i]] = i; });
  const Adj& v2e = m.ask_up(0, 1);
  const LO* va = v2e.a2ab.data();
  const LO* vb = v2e.ab2b.data();
  const I8* vc = v2e.codes.data();
  const double* len = m.ask_lengths().data();
  pfor(m.nverts(), [=] __device__(LO v) {
    bool is_cand = false;
    GO best_g = -1;
    double best_l = -1, best_q = -1;
    for (LO x = va[v]; x < va[v + 1]; ++x) {
      LO e = vb[x];
      LO cand = ec[e];
      if (cand == -1) continue;
      int eev = code_which_down(vc[x]);
      if (!collapses(codes[cand], eev)) continue;
      double l = len[e], q = quals2[cand * 2 + eev];
      if ((best_g == -1) || (l < best_l) || ((l == best_l) && (q > best_q))) {
        is_cand = true;
        best_g = e;
        best_l = l;
        best_q = q;
      }
    }
    vcand[v] = is_cand;
    vqual[v] = best_q;
    vrail[v] = best_g;
  });
}

static void filter_cands(Arr<LO>& c2e, Arr<I8>& codes, Arr<double>* q2) {
  Arr<LO> keep = collect_marked(codes);
  c2e = unmap(keep, c2e, 1);
  codes = unmap(keep, codes, 1);
  if (q2) *q2 = unmap(keep, *q2, 2);
}

bool coarsen_by_size(Mesh& m, const AdaptOpts& o, PassStats* st) {
  int dim = m.dim;
  const Arr<double>& len = m.ask_lengths();
  LO ne = m.nedges();
  Arr<I8> ecand(ne);
  {
    const double* l = len.data();
    I8* c = ecand.data();
    double mn = o.min_length_desired;
    pfor(ne, [=] __device__(LO i) { c[i] = l[i] < mn; });
  }
  if (count_marked(ecand) == 0) return false;
  Arr<I8> vm = mark_down(m, EDGE, VERT, ecand);
  Arr<I8> ecodes(ne);
  {
    const LO* ev = m.ask_verts_of(1).data();
    const I8* v = vm.data();
    I8* ec = ecodes.data();
    pfor(ne, [=] __device__(LO e) { ec[e] = I8((v[ev[e * 2]] ? 1 : 0) | (v[ev[e * 2 + 1]] ? 2 : 0)); });
  }
  Arr<LO> c2e = collect_marked(ecodes);
  Arr<I8> codes0 = unmap(c2e, ecodes, 1);
  Arr<I8> codes(c2e.size());
  check_collapse_class(m, c2e.data(), c2e.size(), codes0.data(), codes.data());
  if (max_i8(codes) <= 0) return false;
  filter_cands(c2e, codes, nullptr);
  Arr<I8> codes2(c2e.size());
  check_collapse_exposure(m, c2e.data(), c2e.size(), codes.data(), codes2.data());
  codes = codes2;
  filter_cands(c2e, codes, nullptr);
  codes2 = Arr<I8>(c2e.size());
  prevent_coarsen_overshoot(m, o.max_length_desired, c2e.data(), c2e.size(), codes.data(),
                            codes2.data());
  codes = codes2;
  filter_cands(c2e, codes, nullptr);
  if (c2e.size() == 0) return false;
  LO nc = c2e.size();
  Arr<double> q2(nc * 2);
  coarsen_qualities(m, c2e.data(), nc, codes.data(), q2.data());
  {
    I8* cd = codes.data();
    const double* q = q2.data();
    double mqa = o.min_quality_allowed;
    pfor(nc, [=] __device__(LO i) {
      I8 code = cd[i];
      for (int d = 0; d < 2; ++d)
        if (!(q[i * 2 + d] >= mqa)) code = dont_collapse(code, d);
      cd[i] = code;
    });
  }
  filter_cands(c2e, codes, &q2);
  if (c2e.size() == 0) return false;
  LO nv = m.nverts();
  Arr<I8> vc(nv);
  Arr<double> vq(nv);
  Arr<GO> vr(nv);
  choose_rails(m, c2e.data(), c2e.size(), codes.data(), q2.data(), vc.data(), vq.data(), vr.data());
  Arr<I8> vkeys = find_indset(m, VERT, vq, vc, &st->indset_rounds);
  Arr<LO> k2v = collect_marked(vkeys);
  LO nkeys = k2v.size();
  st->coarsen_keys = nkeys;
  // find_rails (src/Omega_h_collapse_rail.cpp:79-108) and the vertices onto
  Arr<LO> r2e(nkeys);
  Arr<I8> rdir(nkeys);
  Arr<LO> k2onto(nkeys);
  {
    const Adj& v2e = m.ask_up(0, 1);
    const LO* va = v2e.a2ab.data();
    const LO* vb = v2e.ab2b.data();
    const I8* vcd = v2e.codes.data();
    const LO* kv = k2v.data();
    const GO* rail = vr.data();
    const LO* ev = m.ask_verts_of(1).data();
    LO* re = r2e.data();
    I8* rd = rdir.data();
    LO* ko = k2onto.data();
    int* stw = ctx().d_status;
    pfor(nkeys, [=] __device__(LO k) {
      LO v = kv[k];
      re[k] = -1;
      for (LO x = va[v]; x < va[v + 1]; ++x)
        if (GO(vb[x]) == rail[v]) {
          re[k] = vb[x];
          rd[k] = I8(code_which_down(vcd[x]));
          break;
        }
      if (re[k] < 0) {
        raise_status(stw, ST_TOPOLOGY);
        re[k] = 0;
        rd[k] = 0;
      }
      ko[k] = ev[LO(re[k]) * 2 + (1 - rd[k])];
    });
  }
  // mark_dead_ents (src/Omega_h_coarsen_topology.cpp:28-70)
  Arr<I8> dead[4];
  dead[1] = mark_image(r2e, ne);
  for (int d = 2; d <= dim; ++d) dead[d] = fill<I8>(m.nents[d], 0);
  for (int cd = dim; cd > EDGE; --cd) {
    const Adj& e2c = m.ask_up(1, cd);
    const LO* ea = e2c.a2ab.data();
    const LO* eb = e2c.ab2b.data();
    const I8* ecc = e2c.codes.data();
    const LO* cs = m.ask_down(cd, cd - 1).ab2b.data();
    int nccs = simplex_degree(cd, cd - 1);
    const LO* re = r2e.data();
    const I8* rd = rdir.data();
    I8* dc = dead[cd].data();
    I8* ds = dead[cd - 1].data();
    pfor(nkeys, [=] __device__(LO r) {
      LO e = re[r];
      int onto = 1 - rd[r];
      for (LO x = ea[e]; x < ea[e + 1]; ++x) {
        LO el = eb[x];
        int cce = code_which_down(ecc[x]), rot = code_rotation(ecc[x]);
        int ccv = down_template(cd, 1, cce, rot ^ onto);
        dc[el] = 1;
        ds[cs[el * nccs + opposite_template(cd, 0, ccv)]] = 1;
      }
    });
  }
  // coarsen_element_based2 (src/Omega_h_coarsen.cpp:106-156)
  Mesh nm;
  nm.dim = dim;
  Arr<LO> ov2nv, old_lows2new;
  for (int d = 0; d <= dim; ++d) {
    Arr<LO> k2p, pv2v, kd2d;
    if (d == VERT) {
      k2p = fill<LO>(nkeys + 1, 0);
    } else {
      // find_coarsen_domains: live d-entities around each key vertex
      const Adj& v2d = m.ask_up(0, d);
      const LO* va = v2d.a2ab.data();
      const LO* vb = v2d.ab2b.data();
      const I8* vcd = v2d.codes.data();
      const I8* dd = dead[d].data();
      const LO* kv = k2v.data();
      Arr<LO> cnt(nkeys);
      LO* ct = cnt.data();
      pfor(nkeys, [=] __device__(LO k) {
        LO v = kv[k], n2 = 0;
        for (LO x = va[v]; x < va[v + 1]; ++x) n2 += !dd[vb[x]];
        ct[k] = n2;
      });
      k2p = offset_scan(cnt);
      LO nprod = last(k2p);
      kd2d = Arr<LO>(nprod);
      int nccv = d + 1;
      pv2v = Arr<LO>(nprod * nccv);
      const LO* kp = k2p.data();
      const LO* cv = m.ask_verts_of(d).data();
      const LO* ko = k2onto.data();
      const LO* o2n = ov2nv.data();
      LO* kd = kd2d.data();
      LO* pv = pv2v.data();
      pfor(nkeys, [=] __device__(LO k) {
        LO v = kv[k], p = kp[k];
        for (LO x = va[v]; x < va[v + 1]; ++x) {
          LO el = vb[x];
          if (dd[el]) continue;
          int ccv_col = code_which_down(vcd[x]);
          kd[p] = el;
          for (int ccv = 0; ccv < nccv; ++ccv) {
            LO ov = ccv == ccv_col ? ko[k] : cv[el * nccv + ccv];
            pv[p * nccv + ccv] = o2n[ov];
          }
          ++p;
        }
      });
    }
    ModifyOut mo = modify_ents_adapt(m, nm, d, VERT, k2v, k2p, pv2v, old_lows2new);
    LO nnew = nm.nents[d];
    if (d == VERT) ov2nv = mo.old2new;
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, unmap(kd2d, m.class_dim[d], 1), 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, unmap(kd2d, m.class_id[d], 1), 1);
    if (d == VERT) {
      nm.coords = xfer(m.coords, mo, nnew, Arr<double>(), dim);
      nm.metric = xfer(m.metric, mo, nnew, Arr<double>(), m.mcomp());
    }
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

// ------------------------------------------------------------ swap (3D)
struct SwapTables {
  int off_tri[8], off_mesh[8], off_uedge[8], off_e2u[8];
  int nmesh[8], ntri[8], nedge[8];
  int data[OHG_SWAP3D_TABLE_LEN];
};
__constant__ SwapTables c_swap;
static void upload_swap_tables() {
  static bool done = false;
  if (done) return;
  SwapTables t;
  for (int i = 0; i < 8; ++i) t.nmesh[i] = t.ntri[i] = t.nedge[i] = 0;
  int p = 0;
  while (p < OHG_SWAP3D_TABLE_LEN) {
    int n = OHG_SWAP3D_TABLE[p], nm = OHG_SWAP3D_TABLE[p + 1], nt = OHG_SWAP3D_TABLE[p + 2],
        nu = OHG_SWAP3D_TABLE[p + 3];
    p += 4;
    t.nmesh[n] = nm;
    t.ntri[n] = nt;
    t.off_tri[n] = p;
    p += nu * 3;
    t.off_mesh[n] = p;
    p += nm * nt;
    int nedge = OHG_SWAP3D_TABLE[p], nue = OHG_SWAP3D_TABLE[p + 1];
    p += 2;
    t.nedge[n] = nedge;
    t.off_uedge[n] = p;
    p += nue * 2;
    t.off_e2u[n] = p;
    p += nm * nedge;
  }
  for (int i = 0; i < OHG_SWAP3D_TABLE_LEN; ++i) t.data[i] = OHG_SWAP3D_TABLE[i];
  OHG_CUDA(cudaMemcpyToSymbolAsync(c_swap, &t, sizeof(t), 0, cudaMemcpyHostToDevice, ctx().stream));
  done = true;
}

struct Loop {
  int size;
  LO eev2v[2];
  LO lv[7];
};
// swap3d::find_loop (src/Omega_h_swap3d_loop.hpp:24-78)
__device__ __forceinline__ Loop find_loop(const LO* ea, const LO* eb, const I8* ec, const LO* ev,
                                          const LO* tv, LO edge, int* st) {
  Loop loop;
  LO b = ea[edge], e = ea[edge + 1];
  loop.size = e - b;
  if (loop.size > 7) return loop;
  loop.eev2v[0] = ev[edge * 2];
  loop.eev2v[1] = ev[edge * 2 + 1];
  LO t0[7], t1[7];
  for (int le = 0; le < loop.size; ++le) {
    LO tet = eb[b + le];
    I8 code = ec[b + le];
    int opp = opposite_template(3, 1, code_which_down(code));
    int rot = code_rotation(code);
    t0[le] = tv[tet * 4 + down_template(3, 1, opp, rot ^ 0)];
    t1[le] = tv[tet * 4 + down_template(3, 1, opp, rot ^ 1)];
  }
  for (int i = 0; i < loop.size - 1; ++i) {
    int j;
    for (j = i + 1; j < loop.size; ++j)
      if (t0[j] == t1[i]) break;
    if (j >= loop.size) {
      raise_status(st, ST_TOPOLOGY);
      loop.size = 8;
      return loop;
    }
    LO a0 = t0[i + 1], a1 = t1[i + 1];
    t0[i + 1] = t0[j];
    t1[i + 1] = t1[j];
    t0[j] = a0;
    t1[j] = a1;
  }
  for (int i = 0; i < loop.size; ++i) loop.lv[i] = t0[i];
  return loop;
}

// swap3d_qualities + swap3d::choose (src/Omega_h_swap3d_qualities.cpp:10-58,
// src/Omega_h_swap3d_choice.hpp:15-100)
void swap3d_qualities(Mesh& m, double max_len, const LO* c2e, LO n, double* quals, I8* configs) {
  upload_swap_tables();
  const Adj& e2t = m.ask_up(1, 3);
  const LO* ea = e2t.a2ab.data();
  const LO* eb = e2t.ab2b.data();
  const I8* ec = e2t.codes.data();
  const LO* ev = m.ask_verts_of(1).data();
  const LO* tv = m.ask_verts_of(3).data();
  const double* c = m.coords.data();
  const double* mt = m.metric.data();
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO cand) {
    Loop loop = find_loop(ea, eb, ec, ev, tv, c2e[cand], st);
    quals[cand] = -1.0;
    configs[cand] = -1;
    if (loop.size > 7) return;
    int ls = loop.size;
    int nmeshes = c_swap.nmesh[ls], ntris = c_swap.ntri[ls], nedges = c_swap.nedge[ls];
    const int* tri = c_swap.data + c_swap.off_tri[ls];
    const int* msh = c_swap.data + c_swap.off_mesh[ls];
    const int* ued = c_swap.data + c_swap.off_uedge[ls];
    const int* e2u = c_swap.data + c_swap.off_e2u[ls];
    unsigned long long tcached = 0;
    unsigned ecached = 0;
    double tq[35];
    double el[26];
    int best = -1;
    double bestq = 0.0;
    for (int mesh = 0; mesh < nmeshes; ++mesh) {
      double mq = 1.0;
      for (int t = 0; t < ntris; ++t) {
        int u = msh[mesh * ntris + t];
        if (!((tcached >> u) & 1ull)) {
          LO tet[4];
          for (int k = 0; k < 3; ++k) tet[k] = loop.lv[tri[u * 3 + k]];
          double tmq = 1.0;
          for (int tt = 0; tt < 2; ++tt) {
            tet[3] = loop.eev2v[1 - tt];
            tmq = min2d(tmq, elem_quality_v(3, c, mt, tet));
            LO s = tet[1];
            tet[1] = tet[2];
            tet[2] = s;
          }
          tcached |= (1ull << u);
          tq[u] = tmq;
        }
        mq = min2d(mq, tq[u]);
        if (mq < 0.0) break;
      }
      if (mq > bestq) {
        bool over = false;
        for (int me = 0; me < nedges; ++me) {
          int ue = e2u[mesh * nedges + me];
          if (!((ecached >> ue) & 1u)) {
            LO a = loop.lv[ued[ue * 2]], b = loop.lv[ued[ue * 2 + 1]];
            el[ue] = edge_length3(c + a * 3, c + b * 3, mt + a * 6, mt + b * 6);
            ecached |= (1u << ue);
          }
          if (el[ue] > max_len) {
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
    configs[cand] = I8(best);
    quals[cand] = bestq;
  });
}

// mark_sliver_layers (src/Omega_h_mark.cpp:190-212): elements below the
// quality ceiling, then nlayers rounds of max over dual-graph neighbours
Arr<I8> mark_sliver_layers(Mesh& m, double ceil, int nlayers) {
  const Arr<double>& q = m.ask_qualities();
  LO ne = m.nelems();
  Arr<I8> a(ne), b(ne);
  const double* qq = q.data();
  I8* s = a.data();
  pfor(ne, [=] __device__(LO i) { s[i] = qq[i] < ceil; });
  const Adj& dual = m.ask_adj(m.dim, m.dim);
  const LO* da = dual.a2ab.data();
  const LO* db = dual.ab2b.data();
  for (int l = 0; l < nlayers; ++l) {
    const I8* o = a.data();
    I8* nw = b.data();
    pfor(ne, [=] __device__(LO e) {
      I8 r = -128;
      for (LO x = da[e]; x < da[e + 1]; ++x) r = max(r, o[db[x]]);
      nw[e] = r;
    });
    std::swap(a, b);
  }
  return a;
}

bool swap_edges(Mesh& m, const AdaptOpts& o, PassStats* st) {
  if (m.dim != 3) return false;
  Arr<I8> ec = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  Arr<I8> edc = mark_down(m, 3, 1, ec);
  {
    I8* e = edc.data();
    const I8* cd = m.class_dim[1].data();
    pfor(m.nedges(), [=] __device__(LO i) { e[i] = e[i] && cd[i] == 3; });
  }
  if (count_marked(edc) == 0) return false;
  Arr<LO> c2e = collect_marked(edc);
  LO nc = c2e.size();
  Arr<double> cq(nc);
  Arr<I8> cc(nc);
  swap3d_qualities(m, o.max_length_allowed, c2e.data(), nc, cq.data(), cc.data());
  LO ne = m.nedges();
  Arr<I8> econfig = map_onto(cc, c2e, ne, I8(-1), 1);
  // filter_swap_improve (src/Omega_h_swap.cpp:35-43)
  Arr<I8> keep(nc);
  {
    const double* eq = m.ask_qualities().data();
    const Adj& e2t = m.ask_up(1, 3);
    const LO* ea = e2t.a2ab.data();
    const LO* eb = e2t.ab2b.data();
    const LO* ce = c2e.data();
    const double* q = cq.data();
    I8* kp = keep.data();
    pfor(nc, [=] __device__(LO i) {
      LO e = ce[i];
      double old = DBL_MAX;
      for (LO x = ea[e]; x < ea[e + 1]; ++x) old = min2d(old, eq[eb[x]]);
      kp[i] = q[i] > old;
    });
  }
  Arr<LO> kept = collect_marked(keep);
  if (kept.size() == 0) return false;
  c2e = unmap(kept, c2e, 1);
  cq = unmap(kept, cq, 1);
  Arr<I8> is_cand = mark_image(c2e, ne);
  Arr<double> edge_q = map_onto(cq, c2e, ne, -1.0, 1);
  Arr<I8> keys = find_indset(m, EDGE, edge_q, is_cand, &st->indset_rounds);
  Arr<LO> k2e = collect_marked(keys);
  LO nkeys = k2e.size();
  st->swap_keys = nkeys;
  // swap3d_keys_to_prods + swap3d_topology (src/Omega_h_swap3d_topology.cpp)
  const Adj& e2t = m.ask_up(1, 3);
  const LO* ea = e2t.a2ab.data();
  Arr<LO> cnt[4], k2p[4], pv2v[4];
  for (int d = 1; d <= 3; ++d) cnt[d] = Arr<LO>(nkeys);
  {
    const LO* ke = k2e.data();
    LO* c1 = cnt[1].data();
    LO* c2 = cnt[2].data();
    LO* c3 = cnt[3].data();
    pfor(nkeys, [=] __device__(LO k) {
      int ls = ea[ke[k] + 1] - ea[ke[k]];
      if (ls > 7) ls = 0;
      int npt = c_swap.ntri[ls], npe = c_swap.nedge[ls];
      c1[k] = npe;
      c2[k] = npt + 2 * npe;
      c3[k] = 2 * npt;
    });
  }
  for (int d = 1; d <= 3; ++d) {
    k2p[d] = offset_scan(cnt[d]);
    pv2v[d] = Arr<LO>(last(k2p[d]) * (d + 1));
  }
  {
    const LO* eb = e2t.ab2b.data();
    const I8* ecd = e2t.codes.data();
    const LO* ev = m.ask_verts_of(1).data();
    const LO* tv = m.ask_verts_of(3).data();
    const LO* ke = k2e.data();
    const I8* cfg = econfig.data();
    const LO* p1 = k2p[1].data();
    const LO* p2 = k2p[2].data();
    const LO* p3 = k2p[3].data();
    LO* v1 = pv2v[1].data();
    LO* v2 = pv2v[2].data();
    LO* v3 = pv2v[3].data();
    int* stw = ctx().d_status;
    pfor(nkeys, [=] __device__(LO k) {
      Loop loop = find_loop(ea, eb, ecd, ev, tv, ke[k], stw);
      int config = cfg[ke[k]];
      if (loop.size > 7 || loop.size < 3 || config < 0 || config >= c_swap.nmesh[loop.size]) {
        // no valid configuration: products get the key edge's own vertices
        // (valid indices) and the status word reports the failure
        raise_status(stw, ST_TOPOLOGY);
        LO a = ev[ke[k] * 2];
        for (LO p = p1[k] * 2; p < p1[k + 1] * 2; ++p) v1[p] = a;
        for (LO p = p2[k] * 3; p < p2[k + 1] * 3; ++p) v2[p] = a;
        for (LO p = p3[k] * 4; p < p3[k + 1] * 4; ++p) v3[p] = a;
        return;
      }
      int ls = loop.size;
      int npt = c_swap.ntri[ls], npe = c_swap.nedge[ls];
      const int* tri = c_swap.data + c_swap.off_tri[ls];
      const int* msh = c_swap.data + c_swap.off_mesh[ls];
      const int* ued = c_swap.data + c_swap.off_uedge[ls];
      const int* e2u = c_swap.data + c_swap.off_e2u[ls];
      for (int pe = 0; pe < npe; ++pe) {
        int ue = e2u[config * npe + pe];
        LO a = loop.lv[ued[ue * 2]], b = loop.lv[ued[ue * 2 + 1]];
        LO pedge = p1[k] + pe;
        v1[pedge * 2] = a;
        v1[pedge * 2 + 1] = b;
        for (int eev = 0; eev < 2; ++eev) {
          LO ptri = p2[k] + 2 * pe + eev;
          v2[ptri * 3] = a;
          v2[ptri * 3 + 1] = b;
          v2[ptri * 3 + 2] = loop.eev2v[eev];
        }
      }
      for (int pt = 0; pt < npt; ++pt) {
        int ut = msh[config * npt + pt];
        LO t0 = loop.lv[tri[ut * 3]], t1 = loop.lv[tri[ut * 3 + 1]], t2 = loop.lv[tri[ut * 3 + 2]];
        LO ptri = p2[k] + 2 * npe + pt;
        v2[ptri * 3] = t0;
        v2[ptri * 3 + 1] = t1;
        v2[ptri * 3 + 2] = t2;
        for (int eev = 0; eev < 2; ++eev) {
          LO ptet = p3[k] + 2 * pt + eev;
          v3[ptet * 4] = t0;
          v3[ptet * 4 + 1] = eev == 0 ? t2 : t1;
          v3[ptet * 4 + 2] = eev == 0 ? t1 : t2;
          v3[ptet * 4 + 3] = loop.eev2v[eev];
        }
      }
    });
  }
  if (ctx().take_status() & ST_TOPOLOGY) throw Error(10, "edge swap found an invalid edge ring");
  Mesh nm;
  nm.dim = 3;
  nm.nents[0] = m.nverts();
  nm.coords = m.coords;
  nm.metric = m.metric;
  nm.class_dim[0] = m.class_dim[0];
  nm.class_id[0] = m.class_id[0];
  Arr<LO> old_lows2new = iota(m.nverts());
  for (int d = 1; d <= 3; ++d) {
    ModifyOut mo = modify_ents_adapt(m, nm, d, EDGE, k2e, k2p[d], pv2v[d], old_lows2new);
    LO nnew = nm.nents[d];
    // transfer_inherit_swap: every product inherits the key edge's class
    LO np = mo.prods2new.size();
    Arr<I8> pcd(np);
    Arr<LO> pci(np);
    {
      const LO* ke = k2e.data();
      const LO* kp = k2p[d].data();
      const I8* ecd = m.class_dim[1].data();
      const LO* eci = m.class_id[1].data();
      I8* a = pcd.data();
      LO* b = pci.data();
      pfor(nkeys, [=] __device__(LO k) {
        for (LO p = kp[k]; p < kp[k + 1]; ++p) {
          a[p] = ecd[ke[k]];
          b[p] = eci[ke[k]];
        }
      });
    }
    nm.class_dim[d] = xfer(m.class_dim[d], mo, nnew, pcd, 1);
    nm.class_id[d] = xfer(m.class_id[d], mo, nnew, pci, 1);
    xfer_lengths_qualities(m, nm, d, mo);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

// ------------------------------------------------------------ the pass
PassStats adapt_pass(Mesh& m, const AdaptOpts& o) {
  Ctx& c = ctx();
  PassStats st;
  st.nelems_in = m.nelems();
  cudaEvent_t e0, e1, e2, e3;
  OHG_CUDA(cudaEventCreate(&e0));
  OHG_CUDA(cudaEventCreate(&e1));
  OHG_CUDA(cudaEventCreate(&e2));
  OHG_CUDA(cudaEventCreate(&e3));
  OHG_CUDA(cudaEventRecord(e0, c.stream));
  st.did_refine = refine_by_size(m, o, &st);
  OHG_CUDA(cudaEventRecord(e1, c.stream));
  st.did_coarsen = coarsen_by_size(m, o, &st);
  OHG_CUDA(cudaEventRecord(e2, c.stream));
  st.min_quality = min_f64(m.ask_qualities());
  if (st.min_quality < o.min_quality_desired && m.dim == 3) st.did_swap = swap_edges(m, o, &st);
  OHG_CUDA(cudaEventRecord(e3, c.stream));
  c.sync();
  OHG_CUDA(cudaEventElapsedTime(&st.ms_refine, e0, e1));
  OHG_CUDA(cudaEventElapsedTime(&st.ms_coarsen, e1, e2));
  OHG_CUDA(cudaEventElapsedTime(&st.ms_swap, e2, e3));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaEventDestroy(e3);
  st.nelems_out = m.nelems();
  return st;
}

}  // namespace ohg
