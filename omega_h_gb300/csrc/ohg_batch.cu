// Many meshes as one: the disjoint union of K meshes of one dimension, on
// which one adapt pass does the work of K passes in the same number of
// launches, and its split back into K meshes.
//
// Why the union pass equals the K separate passes, bit for bit: every
// decision on the pass reads one cavity, one star or one upward row, all of
// which stay inside one mesh; the only orderings used (independent-set and
// rail tie-breaks by entity number, the renumbering scans of a rebuild)
// compare entities of the same mesh, whose relative order a constant offset
// keeps; a rebuild numbers new entities in the order of their old
// representatives, so each mesh stays one contiguous block per dimension.
// The mesh index rides in the class ids (class_id + k * kPartStride), which
// the pass only ever copies, never compares.
#include <algorithm>

#include "ohg_batch.cuh"

namespace ohg {

// dst[i] = src_k[i - start_k] (+ add_k) for i in mesh k's range
// (with range > 0, a source value outside [0, range) raises ST_BOUNDS)
template <class T>
__global__ void k_concat(int K, const LO* starts, const T* const* srcs, const LO* adds, T* dst,
                         LO total, LO range, int* st) {
  LO i = LO(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int lo = 0, hi = K;  // largest k with starts[k] <= i
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (starts[mid] <= i) lo = mid; else hi = mid;
  }
  T v = srcs[lo][i - starts[lo]];
  if (range > 0 && (LO(v) < 0 || LO(v) >= range)) raise_status(st, ST_BOUNDS);
  if (adds) v = T(v + adds[lo]);
  dst[i] = v;
}

template <class T>
static Arr<T> concat_arrays(const std::vector<const Arr<T>*>& parts, int width,
                            const std::vector<LO>* adds, LO range = 0) {
  int K = int(parts.size());
  std::vector<LO> starts(K + 1, 0);
  std::vector<const T*> srcs(K);
  for (int k = 0; k < K; ++k) {
    starts[k + 1] = starts[k] + parts[k]->size();
    srcs[k] = parts[k]->data();
  }
  LO total = starts[K];
  (void)width;
  Arr<T> out(total);
  if (total == 0) return out;
  Arr<LO> d_starts = to_device(starts);
  Arr<const T*> d_srcs = to_device(srcs);
  Arr<LO> d_adds;
  if (adds) d_adds = to_device(*adds);
  Ctx& c = ctx();
  k_concat<T><<<(total + kBlock - 1) / kBlock, kBlock, 0, c.stream>>>(
      K, d_starts.data(), d_srcs.data(), adds ? d_adds.data() : nullptr, out.data(), total, range,
      c.d_status);
  ++c.launches;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
  return out;
}

Mesh concat_meshes(const std::vector<Mesh*>& ms) {
  int K = int(ms.size());
  if (K == 0) throw Error(8, "concat of no meshes");
  if (K > kMaxParts) throw Error(8, "concat of more than " + std::to_string(kMaxParts) + " meshes");
  int dim = ms[0]->dim;
  for (Mesh* m : ms) {
    if (m->dim != dim) throw Error(8, "concat of meshes of different dimensions");
    if (m->mcomp() != ms[0]->mcomp())
      throw Error(8, "concat of meshes with isotropic and anisotropic metrics");
  }
  Mesh u;
  u.dim = dim;
  u.metric_comps = ms[0]->metric_comps;
  std::vector<std::vector<LO>> off(dim + 1, std::vector<LO>(K, 0));
  for (int d = 0; d <= dim; ++d) {
    LO run = 0;
    for (int k = 0; k < K; ++k) {
      off[d][k] = run;
      run += ms[k]->nents[d];
    }
    u.nents[d] = run;
  }
  std::vector<const Arr<double>*> cs, mts;
  for (Mesh* m : ms) {
    cs.push_back(&m->coords);
    mts.push_back(&m->metric);
  }
  u.coords = concat_arrays(cs, dim, nullptr);
  u.metric = concat_arrays(mts, u.mcomp(), nullptr);
  std::vector<LO> part_add(K);
  for (int k = 0; k < K; ++k) part_add[k] = k * kPartStride;
  for (int d = 0; d <= dim; ++d) {
    std::vector<const Arr<I8>*> cd;
    std::vector<const Arr<LO>*> ci;
    for (Mesh* m : ms) {
      cd.push_back(&m->class_dim[d]);
      ci.push_back(&m->class_id[d]);
    }
    u.class_dim[d] = concat_arrays(cd, 1, nullptr);
    u.class_id[d] = concat_arrays(ci, 1, &part_add, kPartStride);
  }
  if (ctx().take_status() & ST_BOUNDS)
    throw Error(8, "concat: a class id outside [0, 2^20)");
  for (int d = 1; d <= dim; ++d) {
    std::vector<const Arr<LO>*> dn;
    std::vector<const Arr<I8>*> dc;
    bool codes = d > 1;
    for (Mesh* m : ms) {
      const Adj& a = m->ask_down(d, d - 1);
      dn.push_back(&a.ab2b);
      dc.push_back(&a.codes);
    }
    Adj a;
    a.ab2b = concat_arrays(dn, 1, &off[d - 1]);
    if (codes) {
      a.codes = concat_arrays(dc, 1, nullptr);
      a.has_codes = true;
    }
    u.set_ents(d, std::move(a));
  }
  bool all_len = true, all_q = true;
  for (Mesh* m : ms) {
    all_len = all_len && m->has_length;
    all_q = all_q && m->has_quality;
  }
  if (all_len) {
    std::vector<const Arr<double>*> ls;
    for (Mesh* m : ms) ls.push_back(&m->length);
    u.length = concat_arrays(ls, 1, nullptr);
    u.has_length = true;
  }
  if (all_q) {
    std::vector<const Arr<double>*> qs;
    for (Mesh* m : ms) qs.push_back(&m->quality);
    u.quality = concat_arrays(qs, 1, nullptr);
    u.has_quality = true;
  }
  u.parting = ms[0]->parting;
  u.rebuilt = ms[0]->rebuilt;
  u.class_sets = ms[0]->class_sets;
  return u;
}

template <class T>
static Arr<T> slice(const Arr<T>& a, LO begin, LO count) {
  Arr<T> s;
  s.buf = a.buf;
  s.ptr = a.ptr + begin;
  s.n = count;
  return s;
}

std::vector<Mesh> split_mesh(Mesh& u, int K) {
  int dim = u.dim;
  int mc = u.mcomp();
  Ctx& c = ctx();
  // entities per part and dimension; parts must be contiguous and ordered
  Arr<LO> cnt = fill<LO>((dim + 1) * K, 0);
  int* st = c.d_status;
  for (int d = 0; d <= dim; ++d) {
    auto ci = cview(u.class_id[d]);
    auto ct = view(cnt);
    LO n = u.nents[d];
    int base = d * K;
    pfor(n, [=] __device__(LO e) {
      int p = ci[e] / kPartStride;
      if (p < 0 || p >= K || (e > 0 && ci[e - 1] / kPartStride > p)) {
        raise_status(st, ST_TOPOLOGY);
        return;
      }
      atomicAdd(&ct[base + p], 1);
    });
  }
  if (c.take_status()) throw Error(10, "split: the mesh is not a union of contiguous parts");
  std::vector<LO> h = to_host(cnt);
  std::vector<std::vector<LO>> start(dim + 1, std::vector<LO>(K + 1, 0));
  for (int d = 0; d <= dim; ++d)
    for (int k = 0; k < K; ++k) start[d][k + 1] = start[d][k] + h[d * K + k];
  // in place: down adjacency entries relative to their part, class ids
  // without the part index
  Arr<LO> d_start = fill<LO>((dim + 1) * (K + 1), 0);
  {
    std::vector<LO> flat;
    for (int d = 0; d <= dim; ++d) flat.insert(flat.end(), start[d].begin(), start[d].end());
    d_start = to_device(flat);
  }
  auto sv = cview(d_start);
  for (int d = 0; d <= dim; ++d) {
    auto ci = view(u.class_id[d]);
    pfor(u.nents[d], [=] __device__(LO e) { ci[e] = ci[e] % kPartStride; });
  }
  // the class ids above lost the part index: recover each high entity's part
  // from its position
  for (int d = 1; d <= dim; ++d) {
    Adj& a = u.adj.at({d, d - 1});
    auto dn = view(a.ab2b);
    int deg = simplex_degree(d, d - 1);
    int hb = d * (K + 1), lb = (d - 1) * (K + 1);
    pfor(u.nents[d] * deg, [=] __device__(LO x) {
      LO hent = x / deg;
      int lo = 0, hi = K;
      while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (sv[hb + mid] <= hent) lo = mid; else hi = mid;
      }
      dn[x] = dn[x] - sv[lb + lo];
    });
  }
  std::vector<Mesh> out(K);
  for (int k = 0; k < K; ++k) {
    Mesh& m = out[k];
    m.metric_comps = u.metric_comps;
    m.parting = u.parting;
    m.rebuilt = u.rebuilt;
    m.class_sets = u.class_sets;
    m.dim = dim;
    LO v0 = start[0][k], nv = start[0][k + 1] - v0;
    m.coords = slice(u.coords, v0 * dim, nv * dim);
    m.metric = slice(u.metric, v0 * mc, nv * mc);
    for (int d = 0; d <= dim; ++d) {
      LO b = start[d][k], n = start[d][k + 1] - b;
      m.nents[d] = n;
      m.class_dim[d] = slice(u.class_dim[d], b, n);
      m.class_id[d] = slice(u.class_id[d], b, n);
    }
    for (int d = 1; d <= dim; ++d) {
      const Adj& a = u.adj.at({d, d - 1});
      int deg = simplex_degree(d, d - 1);
      LO b = start[d][k], n = start[d][k + 1] - b;
      Adj s;
      s.ab2b = slice(a.ab2b, b * deg, n * deg);
      if (a.has_codes) {
        s.codes = slice(a.codes, b * deg, n * deg);
        s.has_codes = true;
      }
      m.set_ents(d, std::move(s));
    }
    if (u.has_length) {
      m.length = slice(u.length, start[1][k], start[1][k + 1] - start[1][k]);
      m.has_length = true;
    }
    if (u.has_quality) {
      m.quality = slice(u.quality, start[dim][k], start[dim][k + 1] - start[dim][k]);
      m.has_quality = true;
    }
  }
  return out;
}

}  // namespace ohg
