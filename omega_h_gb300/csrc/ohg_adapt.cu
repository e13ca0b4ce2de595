// Refine, coarsen and 3D edge-swap operators of one adapt pass, the
// topology rebuild (modify) and field transfer, all on device arrays.
#include <math_constants.h>

#include <cfloat>
#include <set>
#include <cmath>

#include "ohg_adapt.cuh"
#include "ohg_math.cuh"
#include "ohg_screen.cuh"

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

typedef View<const double> RV;
typedef View<const LO> LV;

// FP64 element quality of vertices v with the maxdet metric (mc metric
// components per vertex; 1: isotropic)
__device__ __forceinline__ double elem_quality_v(int dim, RV c, RV mt, int mc, const LO* v) {
  double pts[12];
  const double* ms[4];
  for (int i = 0; i <= dim; ++i) {
    for (int j = 0; j < dim; ++j) pts[i * dim + j] = c[v[i] * dim + j];
    ms[i] = &mt[v[i] * mc];
  }
  return elem_quality_ms(dim, mc, pts, ms);
}

__device__ __forceinline__ double edge_len_v(int dim, RV c, RV mt, int mc, LO a, LO b) {
  if (mc == 1)
    return dim == 3 ? edge_length_iso3(&c[a * 3], &c[b * 3], mt[a], mt[b])
                    : edge_length_iso2(&c[a * 2], &c[b * 2], mt[a], mt[b]);
  return dim == 3 ? edge_length3(&c[a * 3], &c[b * 3], &mt[a * mc], &mt[b * mc])
                  : edge_length2(&c[a * 2], &c[b * 2], &mt[a * mc], &mt[b * mc]);
}

// ------------------------------------------------------------ screening
VertScreen build_vert_screen(const Arr<double>& coords, const Arr<double>& metric, LO nv,
                             int dim) {
  VertScreen s;
  int mc = nv > 0 ? LO(metric.size() / nv) : (dim == 3 ? 6 : 3);
  s.mc = mc;
  s.xh = Arr<float4>(nv);
  s.xl = Arr<float4>(nv);
  s.ma = Arr<float4>(nv);
  s.mb = Arr<float4>(nv);
  s.dkey = Arr<long long>(nv);
  s.sdet = Arr<double>(nv);
  auto c = cview(coords);
  auto mt = cview(metric);
  auto xh = view(s.xh);
  auto xl = view(s.xl);
  auto ma = view(s.ma);
  auto mb = view(s.mb);
  auto dk = view(s.dkey);
  auto sd = view(s.sdet);
  if (dim == 2) {
    pfor(nv, [=] __device__(LO v) {
      float h[2], l[2];
      for (int j = 0; j < 2; ++j) {
        double x = c[v * 2 + j];
        h[j] = __double2float_rn(x);
        l[j] = __double2float_rn(x - double(h[j]));
      }
      xh[v] = make_float4(h[0], h[1], 0.0f, fmaxf(fabsf(h[0]), fabsf(h[1])));
      xl[v] = make_float4(l[0], l[1], 0.0f, 0.0f);
      if (mc == 1) {  // isotropic: diag(m), size factor m
        double m = mt[v];
        float f = __double2float_rn(m);
        ma[v] = make_float4(f, f, 0.0f, __fmul_ru(2.0f * fabsf(f), 1.0f + 0x1p-20f));
        mb[v] = make_float4(0.0f, 0.0f, 0.0f, __double2float_rn(m));
        dk[v] = order_key(m);
        sd[v] = m;
        return;
      }
      const double* m = &mt[v * 3];
      float f[3];
      for (int j = 0; j < 3; ++j) f[j] = __double2float_rn(m[j]);
      float s0 = __fmul_ru(fabsf(f[0]) + fabsf(f[1]) + 2.0f * fabsf(f[2]), 1.0f + 0x1p-20f);
      double det = det2p(m);
      double sdet = sqrt(det);
      ma[v] = make_float4(f[0], f[1], f[2], s0);
      mb[v] = make_float4(0.0f, 0.0f, 0.0f, __double2float_rn(sdet));
      dk[v] = order_key(det);
      sd[v] = sdet;
    });
    return s;
  }
  pfor(nv, [=] __device__(LO v) {
    float h[3], l[3];
    for (int j = 0; j < 3; ++j) {
      double x = c[v * 3 + j];
      h[j] = __double2float_rn(x);
      l[j] = __double2float_rn(x - double(h[j]));  // x - h is exact in double
    }
    float mxh = fmaxf(fabsf(h[0]), fmaxf(fabsf(h[1]), fabsf(h[2])));
    xh[v] = make_float4(h[0], h[1], h[2], mxh);
    xl[v] = make_float4(l[0], l[1], l[2], 0.0f);
    if (mc == 1) {  // isotropic: diag(m), size factor sqrt(m (m m))
      double m = mt[v];
      float f = __double2float_rn(m);
      double sf = iso_size_factor(3, m);
      ma[v] = make_float4(f, f, f, 0.0f);
      mb[v] = make_float4(0.0f, 0.0f, __fmul_ru(3.0f * fabsf(f), 1.0f + 0x1p-20f),
                          __double2float_rn(sf));
      dk[v] = order_key(m);
      sd[v] = sf;
      return;
    }
    const double* m = &mt[v * 6];
    float f[6];
    for (int j = 0; j < 6; ++j) f[j] = __double2float_rn(m[j]);
    float s0 = fabsf(f[0]) + fabsf(f[1]) + fabsf(f[2]) +
               2.0f * (fabsf(f[3]) + fabsf(f[4]) + fabsf(f[5]));
    s0 = __fmul_ru(s0, 1.0f + 0x1p-20f);
    double det = det3(symm3(m));
    double sdet = sqrt(det);
    ma[v] = make_float4(f[0], f[1], f[2], f[3]);
    mb[v] = make_float4(f[4], f[5], s0, __double2float_rn(sdet));
    dk[v] = order_key(det);
    sd[v] = sdet;
  });
  return s;
}

// the mesh's screening data, built once per coords and metric
const VertScreen& mesh_screen(Mesh& m) {
  if (!m.screen)
    m.screen = std::make_shared<VertScreen>(build_vert_screen(m.coords, m.metric, m.nverts(), m.dim));
  return *m.screen;
}

void screen_tets(Mesh& m, const LO* tv2v_p, LO n, float* lo_p, float* hi_p, double* ex_p) {
  int dim = m.dim, nvv = dim + 1;
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto tv = cview(tv2v_p, n * nvv);
  auto lo = view(lo_p, n);
  auto hi = view(hi_p, n);
  auto ex = view(ex_p, n);
  pfor(n, [=] __device__(LO i) {
    LO vv[4] = {0, 0, 0, 0};
    for (int k = 0; k < nvv; ++k) vv[k] = tv[i * nvv + k];
    FIv b = elem_quality_bounds(dim, sv, vv);
    lo[i] = b.lo;
    hi[i] = b.hi;
    ex[i] = elem_quality_exact(dim, sv, c, mt, vv);
  });
}

// The per-face route of the collapse screen: each tet's quality interval
// (cubed: the interval of its cube) from its face opposite slot k
// (invariants made once) and the vertex at slot k, with the exact FP64
// value beside it
void screen_tets_face(Mesh& m, const LO* tv2v_p, LO n, int k, bool cubed, float* lo_p,
                      float* hi_p, double* ex_p) {
  if (m.dim != 3 || k < 0 || k > 3) throw Error(1, "screen_tets_face: a 3D mesh and a slot 0..3");
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto tv = cview(tv2v_p, n * 4);
  auto lo = view(lo_p, n);
  auto hi = view(hi_p, n);
  auto ex = view(ex_p, n);
  pfor(n, [=] __device__(LO i) {
    LO vv[4];
    for (int j = 0; j < 4; ++j) vv[j] = tv[i * 4 + j];
    float4 hf[3], lf[3];
    int nf = 0;
    for (int j = 0; j < 4; ++j) {
      if (j == k) continue;
      hf[nf] = sv.xh[vv[j]];
      lf[nf] = sv.xl[vv[j]];
      ++nf;
    }
    int mi = maxdet_vertex(sv, vv);
    TetFaceInv f = tet_face_invariants(hf, lf, k);
    FIv b = cubed ? tet_face_bounds<true>(f, hf, lf, sv.xh[vv[k]], sv.xl[vv[k]], sv.ma[vv[mi]],
                                          sv.mb[vv[mi]])
                  : tet_face_bounds<false>(f, hf, lf, sv.xh[vv[k]], sv.xl[vv[k]], sv.ma[vv[mi]],
                                           sv.mb[vv[mi]]);
    lo[i] = b.lo;
    hi[i] = b.hi;
    ex[i] = tet_quality_exact(sv, c, mt, vv);
  });
}

void screen_edges(Mesh& m, const LO* ev2v_p, LO n, float* lo_p, float* hi_p, double* ex_p) {
  int dim = m.dim, mc = m.mcomp();
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto ev = cview(ev2v_p, n * 2);
  auto lo = view(lo_p, n);
  auto hi = view(hi_p, n);
  auto ex = view(ex_p, n);
  pfor(n, [=] __device__(LO i) {
    FIv b = edge_len_bounds_d(dim, sv, ev[i * 2], ev[i * 2 + 1]);
    lo[i] = b.lo;
    hi[i] = b.hi;
    ex[i] = edge_len_v(dim, c, mt, mc, ev[i * 2], ev[i * 2 + 1]);
  });
}

// adds v over the calling warp's active lanes to *p with one atomic
__device__ __forceinline__ void warp_count(unsigned long long* p, unsigned v) {
  unsigned mask = __activemask();
  unsigned tot = __reduce_add_sync(mask, v);
  if (int(threadIdx.x & 31) == __ffs(mask) - 1 && tot) atomicAdd(p, (unsigned long long)tot);
}

// warp_count for code that every lane of the warp reaches
__device__ __forceinline__ void warp_count_full(unsigned long long* p, unsigned v) {
  unsigned tot = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31u) == 0u && tot) atomicAdd(p, (unsigned long long)tot);
}

// f(i) for every i below a count that is on the device (*n_dev, at most
// bound), in a grid-stride loop over a grid of resident size: the count
// needs no host wait
template <class F>
__global__ void k_for_dev_count(const LO* n_dev, F f) {
  LO n = *n_dev;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    f(LO(i));
}
template <class F>
static void pfor_dev_count(const LO* n_dev, LO bound, F f) {
  if (bound <= 0) return;
  Ctx& c = ctx();
  long long full = (long long)c.num_sms * (2048 / kBlock);
  long long need = ((long long)bound + kBlock - 1) / kBlock;
  k_for_dev_count<<<unsigned(need < full ? need : full), kBlock, 0, c.stream>>>(n_dev, f);
  ++c.launches;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
}

// lanes per collapse direction in the cavity screens (both directions of a
// candidate must fit in one warp: at most 16)
constexpr int kCavityLanes = 8;
static_assert(kCavityLanes <= 16, "two directions per warp");

// smallest float >= x, for comparing floats against a double threshold
static float float_at_or_above(double x) {
  float f = float(x);
  if (double(f) < x) f = std::nextafter(f, INFINITY);
  return f;
}
// largest float <= x
static float float_at_or_below(double x) {
  float f = float(x);
  if (double(f) > x) f = std::nextafter(f, -INFINITY);
  return f;
}

// ------------------------------------------------------------ indset
enum { NOT_IN = 0, IN = 1, UNKNOWN = 2 };
// a sweeping thread that has not settled its vertices after this long gives
// up and raises ST_STALL (with all blocks resident, the highest-ranked
// undecided vertex settles at its owner's next sweep, so this is a guard)
constexpr unsigned long long kIndsetLimitNs = 2000000000ull;
constexpr int kIndsetBlock = 256;
// in-place rounds over all vertices, one thread each, before the sweep
constexpr int kIndsetRounds = 2;
// undecided vertices a sweeping thread keeps in its own list
constexpr int kIndsetPending = 16;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// find_indset (src/Omega_h_indset.cpp:5-34; its rounds, local_iteration,
// src/Omega_h_indset_inline.hpp:14-43, and their driver, lines 53-76):
// a candidate joins when no neighbour has joined and every neighbour not yet
// excluded ranks below it by (quality, index); it is excluded once a
// neighbour has joined.  The set these rules settle on is unique: the greedy
// set by decreasing rank.  A state only ever moves from UNKNOWN to IN or
// NOT_IN, and a lower-ranked neighbour cannot join while a higher-ranked one
// is UNKNOWN, so a read that misses a neighbour's decision can only postpone
// a decision, never change one: the rules may be applied in any order, with
// any staleness, and settle on the same set.  Each neighbour's state is read
// once per decision; the reads of a row are independent (no early exit), so
// their latencies overlap.  first: the state array has not been initialised
// (all UNKNOWN), so a neighbour that is no candidate counts as NOT_IN.
// Eight neighbours u[0..8) (-1: none) folded into a decision: their states,
// then the qualities of the undecided ones, each group of loads issued
// together.  first: the state array has not been initialised (all UNKNOWN),
// so a neighbour that is no candidate counts as NOT_IN.
template <bool first>
__device__ __forceinline__ void indset_fold(LO v, double qv, const LO u[8],
                                            const double* __restrict__ q,
                                            const I8* __restrict__ cands, volatile I8* s,
                                            bool& joined, bool& top) {
  int su[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    su[t] = NOT_IN;
    if (u[t] >= 0 && (!first || cands[u[t]])) su[t] = s[u[t]];
  }
  double qu[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) qu[t] = su[t] == UNKNOWN ? q[u[t]] : 0.0;
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    if (su[t] == IN) joined = true;
    else if (su[t] == UNKNOWN) top = top && ((qu[t] != qv) ? (qu[t] < qv) : (u[t] < v));
  }
}

// A conflict graph given by rows (CSR)
struct CsrGraph {
  const LO* xa;
  const LO* xb;
  template <bool first>
  __device__ __forceinline__ int decide(LO v, const double* __restrict__ q,
                                        const I8* __restrict__ cands, volatile I8* s) const {
    LO beg = xa[v], end = xa[v + 1];
    double qv = q[v];
    bool joined = false, top = true;
    for (LO j = beg; j < end; j += 8) {
      LO u[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) u[t] = j + t < end ? xb[j + t] : -1;
      indset_fold<first>(v, qv, u, q, cands, s, joined, top);
    }
    return joined ? NOT_IN : (top ? IN : UNKNOWN);
  }
};

// Edges that share an element (the star of an edge, src/Omega_h_star.cpp),
// walked through the edge's elements and their edges: no graph is built.
// An edge shared by several of the elements is read once per element, which
// does not change a decision.
struct EdgeStarGraph {
  const LO* ea;   // edge -> element rows
  const LO* eb;
  const LO* le;   // element -> edges, nle per element
  int nle;
  template <bool first>
  __device__ __forceinline__ int decide(LO v, const double* __restrict__ q,
                                        const I8* __restrict__ cands, volatile I8* s) const {
    LO beg = ea[v], end = ea[v + 1];
    double qv = q[v];
    bool joined = false, top = true;
    for (LO x = beg; x < end; ++x) {
      LO el = eb[x];
      LO u[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        LO f = t < nle ? le[el * nle + t] : -1;
        u[t] = f == v ? -1 : f;
      }
      indset_fold<first>(v, qv, u, q, cands, s, joined, top);
    }
    return joined ? NOT_IN : (top ? IN : UNKNOWN);
  }
};

// The rounds before the sweep: one thread per vertex, plain launches, in
// decreasing vertex order.  Among equal qualities the higher index ranks
// first, so decisions spread from high to low indices; with threads in
// decreasing order, a round's later blocks see what its earlier blocks
// decided, and a chain of ties advances by more than one step per round.
template <bool first, class G>
static void indset_round(const G& g, LO n, const Arr<double>& quality, const Arr<I8>& cands,
                         I8* st) {
  auto q = quality.data();
  auto cd = cands.data();
  G gr = g;
  pfor(n, [=] __device__(LO i) {
    LO v = n - 1 - i;
    volatile I8* s = st;
    if (first) {
      if (!cd[v]) {
        s[v] = NOT_IN;
        return;
      }
    } else if (s[v] != UNKNOWN) {
      return;
    }
    int d = gr.template decide<first>(v, q, cd, s);
    if (d != UNKNOWN) s[v] = I8(d);
  });
}

// The sweep that settles the rest: one cooperative launch (all blocks
// resident).  Each thread owns the vertices first, first + stride, ...; it
// keeps up to kIndsetPending of its undecided ones in a list and decides
// what the states it reads allow, sweep after sweep, refilling the list from
// its vertices when it empties, until all of them are decided.  What is
// left after the rounds is chains of decisions that wait on one another;
// one step of a chain costs a sweep of the thread that owns it, so threads
// own few vertices and a sweep is a few rounds of memory latency.  Since the
// highest-ranked undecided vertex can always be decided, every sweep of its
// owner makes progress somewhere.  Threads without progress back off
// briefly with __nanosleep.  sweeps_acc receives the largest sweep count of
// any thread.
template <class G>
__global__ void __launch_bounds__(kIndsetBlock, 4)
    k_indset_sweep(G g, const double* __restrict__ q, const I8* __restrict__ cands, I8* st,
                   LO n, int* status, int* sweeps_acc, unsigned* blocks_done, int* call_max) {
  volatile I8* s = st;
  LO stride = LO(gridDim.x) * kIndsetBlock;
  LO scan = LO(blockIdx.x) * kIndsetBlock + LO(threadIdx.x);  // next owned vertex to look at
  unsigned long long t0 = globaltimer_ns();
  int sweeps = 0;
  unsigned nap = 32;
  LO pend[kIndsetPending];
  int np = 0;
  bool stalled = false;
  for (;;) {
    // refill the list from the owned vertices, eight state reads at a time
    while (np < kIndsetPending && scan < n) {
      I8 sv[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        long long v = (long long)scan + (long long)t * stride;
        sv[t] = v < n ? s[v] : I8(NOT_IN);
      }
      int t = 0;
      for (; t < 8 && np < kIndsetPending; ++t)
        if (sv[t] == UNKNOWN) pend[np++] = scan + LO(t) * stride;
      long long next = (long long)scan + (long long)t * stride;
      scan = next < n ? LO(next) : n;
    }
    if (np == 0) break;
    bool progress = false;
    int keep = 0;
    for (int i = 0; i < np; ++i) {
      LO v = pend[i];
      int d = g.template decide<false>(v, q, cands, s);
      if (d == UNKNOWN) {
        pend[keep++] = v;
      } else {
        s[v] = I8(d);
        progress = true;
      }
    }
    np = keep;
    ++sweeps;
    if (progress) {
      nap = 32;
    } else {
      __nanosleep(nap);
      if (nap < 256) nap *= 2;
    }
    if ((sweeps & 15) == 0 && globaltimer_ns() - t0 > kIndsetLimitNs) {
      stalled = true;
      break;
    }
  }
  if (stalled) raise_status(status, ST_STALL);
  // the call's largest sweep count, added to the accumulator by the last
  // block to finish
  int m = __reduce_max_sync(0xffffffffu, sweeps);
  if ((threadIdx.x & 31u) == 0u) atomicMax(call_max, m);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned prev = atomicAdd(blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      atomicAdd(sweeps_acc, atomicAdd(call_max, 0) + kIndsetRounds);
    }
  }
}

template <class G>
static Arr<I8> find_indset_on(const G& g, LO n, const Arr<double>& quality, const Arr<I8>& cands) {
  Ctx& c = ctx();
  Arr<I8> a(n);
  if (n == 0) return a;
  OHG_CUDA(cudaMemsetAsync(a.data(), UNKNOWN, size_t(n), c.stream));
  indset_round<true>(g, n, quality, cands, a.data());
  for (int r = 1; r < kIndsetRounds; ++r) indset_round<false>(g, n, quality, cands, a.data());
  // blocks_done and the call's sweep maximum
  Arr<unsigned> scratch(2);
  OHG_CUDA(cudaMemsetAsync(scratch.data(), 0, 2 * sizeof(unsigned), c.stream));
  static thread_local int per_sm = 0;  // per host thread and graph type: no locking
  if (per_sm == 0) {
    OHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_indset_sweep<G>,
                                                           kIndsetBlock, 0));
    if (per_sm < 1) per_sm = 1;
  }
  long long full = (long long)per_sm * c.num_sms;
  long long need = (n + kIndsetBlock - 1) / kIndsetBlock;
  unsigned blocks = unsigned(need < full ? need : full);
  G gr = g;
  const double* q = quality.data();
  const I8* cd = cands.data();
  I8* st = a.data();
  int* status = c.d_status;
  int* acc = c.d_indset_sweeps;
  unsigned* done = scratch.data();
  int* cmax = reinterpret_cast<int*>(scratch.data() + 1);
  void* args[] = {(void*)&gr, (void*)&q,      (void*)&cd,  (void*)&st,   (void*)&n,
                  (void*)&status, (void*)&acc, (void*)&done, (void*)&cmax};
  OHG_CUDA(cudaLaunchCooperativeKernel((const void*)k_indset_sweep<G>, dim3(blocks),
                                       dim3(kIndsetBlock), args, 0, c.stream));
  ++c.launches;
  return a;
}

Arr<I8> find_indset(const Adj& g, LO n, const Arr<double>& quality, const Arr<I8>& cands) {
  return find_indset_on(CsrGraph{g.a2ab.data(), g.ab2b.data()}, n, quality, cands);
}
Arr<I8> find_indset(Mesh& m, int d, const Arr<double>& q, const Arr<I8>& cands) {
  if (d == m.dim) return cands;
  if (d == EDGE) {
    // edges sharing an element, walked through the elements: the edge graph
    // (tens of entries per edge) is not built
    const Adj& e2el = m.ask_up_any_order(EDGE, m.dim);  // membership only: row order is free
    EdgeStarGraph g{e2el.a2ab.data(), e2el.ab2b.data(), m.ask_down(m.dim, EDGE).ab2b.data(),
                    simplex_degree(m.dim, EDGE)};
    return find_indset_on(g, m.nents[EDGE], q, cands);
  }
  return find_indset(m.ask_adj(d, d), m.nents[d], q, cands);
}

// ------------------------------------------------------------ marks
static Arr<I8> mark_up(Mesh& m, int ld, int hd, const Arr<I8>& lm) {
  Arr<I8> out(m.nents[hd]);
  auto l = cview(lm);
  auto o = view(out);
  if (ld == VERT && hd == FACE && !m.adj.count({FACE, VERT})) {
    // through the face's edges: the face-vertex list is not derived for it
    auto fe = cview(m.ask_down(FACE, EDGE).ab2b);
    auto ev = cview(m.ask_verts_of(EDGE));
    pfor(m.nents[FACE], [=] __device__(LO f) {
      I8 r = 0;
      for (int k = 0; k < 3; ++k) {
        LO e = fe[f * 3 + k];
        if (l[ev[e * 2]] || l[ev[e * 2 + 1]]) r = 1;
      }
      o[f] = r;
    });
    return out;
  }
  auto hl = cview(m.ask_down(hd, ld).ab2b);
  int deg = simplex_degree(hd, ld);
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
  auto a = cview(l2h.a2ab);
  auto b = cview(l2h.ab2b);
  auto h = cview(hm);
  Arr<I8> out(m.nents[ld]);
  auto o = view(out);
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
// one device, so the local numbering is the global numbering.
//
// In two phases: plan_modify finds the kept entities, the representatives
// and the new numbering's offsets on the device; the three sizes it needs
// (kept, new, products) are the last elements of three of its arrays, so an
// operator plans every dimension first and reads all their sizes with one
// host wait (plan_sizes); apply_modify then builds the dimension.
struct ModifyPlan {
  bool some_mod = false;
  Arr<I8> same;
  Arr<LO> same_offs, reps, offs;
  LO sizes[3] = {0, 0, 0};  // kept, new, products
};
// key_marks, if given, is mark_image(keys2kds, om.nents[key_dim]): the same
// for every dimension of one rebuild, so its caller makes it once
static ModifyPlan plan_modify(Mesh& om, int ent_dim, int key_dim, const Arr<LO>& keys2kds,
                              const Arr<LO>& keys2prods, const Arr<I8>* key_marks = nullptr) {
  LO nkeys = keys2kds.size();
  ModifyPlan pl;
  LO nold = om.nents[ent_dim];
  // entities kept as they are (0/1 marks and their offsets)
  bool some_mod = ent_dim >= key_dim;
  pl.some_mod = some_mod;
  Arr<I8> km;
  Arr<I8>& same = pl.same;
  Arr<LO>& same_offs = pl.same_offs;
  // get_rep_counts (src/Omega_h_modify.cpp:210-243) starts from the kept
  // marks (1 each without modified entities); the keys' products are added
  // below
  Arr<LO> counts(nold);
  if (some_mod) {
    km = key_marks ? *key_marks : mark_image(keys2kds, om.nents[key_dim]);
    Arr<I8> mods_ent = ent_dim == key_dim ? km : mark_up(om, key_dim, ent_dim, km);
    same = Arr<I8>(nold);
    auto me = cview(mods_ent);
    auto sm = view(same);
    auto ct = view(counts);
    pfor(nold, [=] __device__(LO e) {
      I8 k = !me[e];
      sm[e] = k;
      ct[e] = LO(k);
    });
    same_offs = offset_scan(same);
  } else {
    auto ct = view(counts);
    pfor(nold, [=] __device__(LO e) { ct[e] = 1; });
  }
  // representatives (get_mods2reps, src/Omega_h_modify.cpp:163-195)
  Arr<LO>& reps = pl.reps;
  if (key_dim == ent_dim) {
    reps = keys2kds;
  } else {
    reps = Arr<LO>(nkeys);
    auto kd = cview(keys2kds);
    auto r = view(reps);
    if (ent_dim > key_dim && key_dim == VERT && !om.adj.count({VERT, ent_dim})) {
      // The representative is the first entry of the key vertex's upward
      // row, which lists entities in increasing order: the smallest entity
      // index containing the vertex.  Without the rows at hand that is an
      // atomic minimum over the entities' vertices (faces through their
      // edges, so no face-vertex list is derived either).
      LO nv = om.nverts(), nent = om.nents[ent_dim];
      Arr<unsigned> vmin(nv);
      OHG_CUDA(cudaMemsetAsync(vmin.data(), 0xff, size_t(nv) * sizeof(unsigned), ctx().stream));
      auto vm = view(vmin);
      auto kmv = cview(km);
      if (ent_dim == FACE && !om.adj.count({FACE, VERT})) {
        auto fe = cview(om.ask_down(FACE, EDGE).ab2b);
        auto ev = cview(om.ask_verts_of(EDGE));
        pfor(nent, [=] __device__(LO f) {
          for (int k = 0; k < 3; ++k) {
            LO e = fe[f * 3 + k];
            for (int j = 0; j < 2; ++j) {
              LO v = ev[e * 2 + j];
              if (kmv[v]) atomicMin(&vm[v], unsigned(f));
            }
          }
        });
      } else {
        auto hv = cview(om.ask_verts_of(ent_dim));
        int nvh = ent_dim + 1;
        pfor(nent, [=] __device__(LO h) {
          for (int k = 0; k < nvh; ++k) {
            LO v = hv[h * nvh + k];
            if (kmv[v]) atomicMin(&vm[v], unsigned(h));
          }
        });
      }
      int* stw = ctx().d_status;
      pfor(nkeys, [=] __device__(LO k) {
        unsigned b = vm[kd[k]];
        if (b == 0xffffffffu) {
          raise_status(stw, ST_TOPOLOGY);
          r[k] = 0;
        } else {
          r[k] = LO(b);
        }
      });
    } else if (ent_dim == FACE && key_dim == EDGE && om.dim == 3 &&
               !om.adj.count({EDGE, FACE}) && !om.adj_any_order.count({EDGE, FACE})) {
      // the faces containing a key edge are, in each tet around it, the two
      // tet faces that hold both of the edge's vertices: the representative,
      // the smallest such face, without inverting the face-to-edge lists
      const Adj& e2t = om.ask_up_any_order(EDGE, REGION);
      auto ea = cview(e2t.a2ab);
      auto eb = cview(e2t.ab2b);
      auto ec = cview(e2t.codes);
      auto tf = cview(om.ask_down(REGION, FACE).ab2b);
      int* stw = ctx().d_status;
      pfor(nkeys, [=] __device__(LO k) {
        LO e = kd[k];
        LO mn = -1;
        for (LO x = ea[e]; x < ea[e + 1]; ++x) {
          LO t = eb[x];
          int j = code_which_down(ec[x]);
          int va = down_template(3, 1, j, 0), vb = down_template(3, 1, j, 1);
          for (int f = 0; f < 4; ++f) {
            bool ha = false, hb = false;
            for (int q = 0; q < 3; ++q) {
              int fv = down_template(3, 2, f, q);
              ha = ha || fv == va;
              hb = hb || fv == vb;
            }
            if (ha && hb) {
              LO face = tf[t * 4 + f];
              if (mn < 0 || face < mn) mn = face;
            }
          }
        }
        if (mn < 0) {
          raise_status(stw, ST_TOPOLOGY);
          mn = 0;
        }
        r[k] = mn;
      });
    } else if (ent_dim > key_dim) {
      // the first entry of an upward row sorted by high entity is the row's
      // smallest entity: its minimum over the row in any order, so the rows
      // need no sort for this
      const Adj& up = om.ask_up_any_order(key_dim, ent_dim);
      auto ua = cview(up.a2ab);
      auto ub = cview(up.ab2b);
      int* stw = ctx().d_status;
      pfor(nkeys, [=] __device__(LO k) {
        LO b = ua[kd[k]], e = ua[kd[k] + 1];
        if (b == e) {
          raise_status(stw, ST_TOPOLOGY);
          r[k] = 0;
        } else {
          LO mn = ub[b];
          for (LO x = b + 1; x < e; ++x) mn = min(mn, ub[x]);
          r[k] = mn;
        }
      });
    } else {
      auto dn = cview(om.ask_down(key_dim, ent_dim).ab2b);
      int deg = simplex_degree(key_dim, ent_dim);
      pfor(nkeys, [=] __device__(LO k) { r[k] = dn[kd[k] * deg]; });
    }
  }
  // the keys' products onto their representatives: integer sums, so the
  // atomics give a deterministic result
  {
    auto ct = view(counts);
    auto r = cview(reps);
    auto kp = cview(keys2prods);
    pfor(nkeys, [=] __device__(LO k) { atomicAdd(&ct[r[k]], kp[k + 1] - kp[k]); });
  }
  pl.offs = offset_scan(counts);
  pl.sizes[0] = nold;
  return pl;
}

// the sizes of several plans with one host wait (keys2prods[i] belongs to
// plans[i]); status, if given, receives the device status word read in the
// same wait (not cleared)
static void plan_sizes(const std::vector<ModifyPlan*>& plans,
                       const std::vector<const Arr<LO>*>& keys2prods, int* status = nullptr) {
  std::vector<const Arr<LO>*> arrs;
  std::vector<LO*> dst;
  for (size_t i = 0; i < plans.size(); ++i) {
    ModifyPlan& pl = *plans[i];
    if (pl.some_mod) {
      arrs.push_back(&pl.same_offs);
      dst.push_back(&pl.sizes[0]);
    }
    arrs.push_back(&pl.offs);
    dst.push_back(&pl.sizes[1]);
    arrs.push_back(keys2prods[i]);
    dst.push_back(&pl.sizes[2]);
  }
  std::vector<LO> got(arrs.size());
  read_lasts(arrs, got.data(), status);
  for (size_t i = 0; i < arrs.size(); ++i) *dst[i] = got[i];
}

static ModifyOut apply_modify(Mesh& om, Mesh& nm, int ent_dim, int key_dim, const ModifyPlan& pl,
                              const Arr<LO>& keys2kds, const Arr<LO>& keys2prods,
                              const Arr<LO>& prod_verts2verts,
                              const Arr<LO>& old_lows2new_lows) {
  LO nkeys = keys2kds.size();
  ModifyOut out;
  LO nold = om.nents[ent_dim];
  bool some_mod = pl.some_mod;
  const Arr<I8>& same = pl.same;
  const Arr<LO>& same_offs = pl.same_offs;
  const Arr<LO>& reps = pl.reps;
  const Arr<LO>& offs = pl.offs;
  const LO* sizes = pl.sizes;
  LO nnew = sizes[1];
  // the kept entities' old and new numbers and the old-to-new map, in one
  // launch (collect_marked_offs, unmap and map_onto of the same marks)
  {
    LO nsame = some_mod ? sizes[0] : nold;
    out.same2old = Arr<LO>(nsame);
    out.same2new = Arr<LO>(nsame);
    out.old2new = Arr<LO>(nold);
    auto sm = cview(same);
    auto so = cview(same_offs);
    auto of = cview(offs);
    auto s2o = view(out.same2old);
    auto s2n = view(out.same2new);
    auto o2n = view(out.old2new);
    pfor(nold, [=] __device__(LO e) {
      bool kept = !some_mod || sm[e];
      if (!kept) {
        o2n[e] = -1;
        return;
      }
      LO i = some_mod ? so[e] : e;
      LO q = of[e];
      s2o[i] = e;
      s2n[i] = q;
      o2n[e] = q;
    });
  }
  bool has_order = key_dim > ent_dim;
  Arr<LO> order;
  if (has_order) {
    // get_rep2md_order (src/Omega_h_modify.cpp:283-338)
    order = fill<LO>(om.nents[key_dim], -1);
    Arr<LO> md2mod = fill<LO>(om.nents[key_dim], -1);
    auto m2m = view(md2mod);
    auto kd = cview(keys2kds);
    pfor(nkeys, [=] __device__(LO k) { m2m[kd[k]] = k; });
    const Adj& r2m = om.ask_up(ent_dim, key_dim);
    auto ra = cview(r2m.a2ab);
    auto rb = cview(r2m.ab2b);
    auto rc = cview(r2m.codes);
    auto kp = cview(keys2prods);
    auto ord = view(order);
    auto m2mc = cview(md2mod);
    pfor(nold, [=] __device__(LO rep) {
      LO offset = 0;
      for (LO x = ra[rep]; x < ra[rep + 1]; ++x) {
        LO md = rb[x];
        LO mod = m2mc[md];
        if (mod >= 0 && code_which_down(rc[x]) == 0) {
          ord[md] = offset;
          offset += kp[mod + 1] - kp[mod];
        }
      }
    });
  }
  out.prods2new = Arr<LO>(sizes[2]);
  {
    auto of = cview(offs);
    auto r = cview(reps);
    auto kp = cview(keys2prods);
    auto kd = cview(keys2kds);
    auto ord = cview(order);
    auto p2n = view(out.prods2new);
    int self = has_order ? 1 : 0;
    pfor(nkeys, [=] __device__(LO k) {
      LO offset = of[r[k]] + self;
      if (has_order) offset += ord[kd[k]];
      for (LO p = kp[k]; p < kp[k + 1]; ++p) p2n[p] = offset++;
    });
  }
  if (ent_dim == VERT) {
    nm.nents[0] = nnew;
    return out;
  }
  // modify_conn (src/Omega_h_modify.cpp:20-70)
  int ld = ent_dim - 1;
  int deg = simplex_degree(ent_dim, ld);
  const Adj& od = om.ask_down(ent_dim, ld);
  Adj nd;
  // zero-filled so that every slot holds a valid index even if a caller's
  // keys were not independent (the writes below would then overlap)
  nd.ab2b = Arr<LO>(nnew * deg);  // every entry written below
  LO nprods = out.prods2new.size();
  Adj pd;
  if (ld > VERT) {
    // the products' sides among the new mesh's entities of dimension ld:
    // by a hash of their vertex tuples, so the new mesh's vertex-to-ld
    // upward lists (otherwise built for this alone) are not derived
    if (nm.nents[ld] < (LO(1) << 29)) {
      pd = reflect_down_hashed(prod_verts2verts, nprods, nm.ask_verts_of(ld), nm.nents[ld],
                               ent_dim, ld);
    } else {  // the table size would pass the index range: upward lists
      pd = reflect_down(prod_verts2verts, nprods, nm.ask_verts_of(ld), nm.ask_up(VERT, ld),
                        ent_dim, ld);
    }
  } else {
    pd.ab2b = prod_verts2verts;
  }
  // the new down adjacency and its codes in one launch: every new entity is
  // a product (its sides and codes as found) or a kept entity (its old
  // sides renumbered, its old codes)
  bool codes = ld > VERT;
  if (codes) {
    nd.codes = Arr<I8>(nnew * deg);
    nd.has_codes = true;
  }
  {
    LO np = out.prods2new.size(), ns = out.same2old.size();
    auto p2n = cview(out.prods2new);
    auto pb = cview(pd.ab2b);
    auto pc = cview(pd.codes);
    auto s2o = cview(out.same2old);
    auto s2n = cview(out.same2new);
    auto ob = cview(od.ab2b);
    auto oc = cview(od.codes);
    auto l2n = cview(old_lows2new_lows);
    auto nb = view(nd.ab2b);
    auto nc = view(nd.codes);
    int* stw = ctx().d_status;
    pfor(np + ns, [=] __device__(LO i) {
      if (i < np) {
        LO q = p2n[i];
        for (int k = 0; k < deg; ++k) {
          nb[q * deg + k] = pb[i * deg + k];
          if (codes) nc[q * deg + k] = pc[i * deg + k];
        }
        return;
      }
      LO j = i - np, o = s2o[j], q = s2n[j];
      for (int k = 0; k < deg; ++k) {
        LO l = l2n[ob[o * deg + k]];
        if (l < 0) {
          raise_status(stw, ST_TOPOLOGY);
          l = 0;
        }
        nb[q * deg + k] = l;
        if (codes) nc[q * deg + k] = oc[o * deg + k];
      }
    });
  }
  nm.set_ents(ent_dim, std::move(nd));
  return out;
}

static ModifyOut modify_ents_adapt(Mesh& om, Mesh& nm, int ent_dim, int key_dim,
                                   const Arr<LO>& keys2kds, const Arr<LO>& keys2prods,
                                   const Arr<LO>& prod_verts2verts,
                                   const Arr<LO>& old_lows2new_lows) {
  ModifyPlan pl = plan_modify(om, ent_dim, key_dim, keys2kds, keys2prods);
  plan_sizes({&pl}, {&keys2prods});
  return apply_modify(om, nm, ent_dim, key_dim, pl, keys2kds, keys2prods, prod_verts2verts,
                      old_lows2new_lows);
}

// transfer_common (src/Omega_h_transfer.cpp:160-180)
template <class T>
static Arr<T> xfer(const Arr<T>& old, const ModifyOut& mo, LO nnew, const Arr<T>& prod, int w) {
  Arr<T> nd(nnew * w);
  // one launch: the products' values first, then the kept entities'
  LO np = prod.size() ? mo.prods2new.size() : 0;
  auto p2n = cview(mo.prods2new);
  auto pv = cview(prod);
  auto s2o = cview(mo.same2old);
  auto s2n = cview(mo.same2new);
  auto o = cview(old);
  auto d = view(nd);
  pfor(np + mo.same2old.size(), [=] __device__(LO i) {
    if (i < np) {
      for (int j = 0; j < w; ++j) d[p2n[i] * w + j] = pv[i * w + j];
    } else {
      LO k = i - np;
      for (int j = 0; j < w; ++j) d[s2n[k] * w + j] = o[s2o[k] * w + j];
    }
  });
  return nd;
}

// class_dim and class_id of dimension d together, as xfer does for each:
// products take their values (pcd/pci, or those of the old entities kd2d),
// kept entities their old ones; one launch for both arrays
static void xfer_class(Mesh& om, Mesh& nm, int d, const ModifyOut& mo, LO nnew, const I8* pcd,
                       const LO* pci, const LO* kd2d) {
  Arr<I8> cd(nnew);
  Arr<LO> ci(nnew);
  auto ocd = cview(om.class_dim[d]);
  auto oci = cview(om.class_id[d]);
  auto ncd = view(cd);
  auto nci = view(ci);
  LO np = mo.prods2new.size();
  auto p2n = cview(mo.prods2new);
  auto kd = cview(kd2d, kd2d ? np : 0);
  auto pd = cview(pcd, pcd ? np : 0);
  auto pi = cview(pci, pci ? np : 0);
  bool gather = kd2d != nullptr;
  auto s2o = cview(mo.same2old);
  auto s2n = cview(mo.same2new);
  pfor(np + mo.same2old.size(), [=] __device__(LO i) {
    if (i < np) {
      LO q = p2n[i];
      if (gather) {
        ncd[q] = ocd[kd[i]];
        nci[q] = oci[kd[i]];
      } else {
        ncd[q] = pd[i];
        nci[q] = pi[i];
      }
    } else {
      LO k = i - np;
      ncd[s2n[k]] = ocd[s2o[k]];
      nci[s2n[k]] = oci[s2o[k]];
    }
  });
  nm.class_dim[d] = cd;
  nm.class_id[d] = ci;
}

// pv2v: the products' vertex tuples in the new numbering, if at hand (the
// products' qualities are then measured from them, without deriving the new
// mesh's element-to-vertex list)
static void xfer_lengths_qualities(Mesh& om, Mesh& nm, int d, const ModifyOut& mo,
                                   const Arr<LO>* pv2v = nullptr) {
  LO np = mo.prods2new.size();
  if (d == EDGE && om.has_length) {
    Arr<double> pl(np);
    measure_edges_metric(nm, mo.prods2new.data(), np, pl.data());
    nm.length = xfer(om.length, mo, nm.nents[1], pl, 1);
    nm.has_length = true;
  }
  if (d == om.dim && om.has_quality) {
    Arr<double> pq(np);
    if (pv2v && pv2v->size() >= np * (d + 1))
      measure_qualities_tuples(nm, pv2v->data(), np, pq.data());
    else
      measure_qualities(nm, mo.prods2new.data(), np, pq.data());
    nm.quality = xfer(om.quality, mo, nm.nents[d], pq, 1);
    nm.has_quality = true;
  }
}

// ------------------------------------------------------------ refine
// refine_qualities_tmpl (src/Omega_h_refine_qualities.cpp:34-86): one thread
// per candidate edge, two child simplices per adjacent element
void refine_qualities(Mesh& m, const LO* c2e_p, LO n, const double* mid_p, double* out_p) {
  int dim = m.dim, mc = m.mcomp();
  auto ev = cview(m.ask_verts_of(1));
  auto cv = cview(m.ask_verts_of(dim));
  const Adj& e2c = m.ask_up_any_order(1, dim);  // a minimum over the row
  auto ea = cview(e2c.a2ab);
  auto eb = cview(e2c.ab2b);
  auto ec = cview(e2c.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto mid = cview(mid_p, n * mc);
  auto out = view(out_p, n);
  // 8 lanes per candidate over its (element, child) pairs, then the minimum
  // across the lanes (a minimum does not depend on the order: no child
  // quality is NaN or -0)
  constexpr int G = 8;
  group_for(G, n, kBlock, [=] __device__(LO cand, int gl, unsigned gm) {
    if (cand < 0) return;
    LO e = c2e[cand];
    LO v0 = ev[e * 2], v1 = ev[e * 2 + 1];
    double midp[3];
    for (int j = 0; j < dim; ++j) midp[j] = (c[v0 * dim + j] + c[v1 * dim + j]) / 2.;
    double minq = 1.0;
    LO np = 2 * (ea[e + 1] - ea[e]);
    for (LO pi = gl; pi < np; pi += G) {
      LO x = ea[e] + pi / 2;
      LO el = eb[x];
      I8 code = ec[x];
      int cce = code_which_down(code), rot = code_rotation(code);
      {
        int eev = int(pi & 1);
        int ccv = down_template(dim, 1, cce, eev ^ rot);
        int ccs = opposite_template(dim, 0, ccv);
        LO sv[3];
        for (int k = 0; k < dim; ++k) sv[k] = cv[el * (dim + 1) + down_template(dim, dim - 1, ccs, k)];
        // the child: the face opposite the endpoint plus the midpoint (in
        // 3D with the face's last two vertices swapped, flip_new_elem)
        if (dim == 3) {
          LO t = sv[1];
          sv[1] = sv[2];
          sv[2] = t;
        }
        double pts[12];
        const double* ms[4];
        for (int i = 0; i < dim; ++i) {
          for (int j = 0; j < dim; ++j) pts[i * dim + j] = c[sv[i] * dim + j];
          ms[i] = &mt[sv[i] * mc];
        }
        for (int j = 0; j < dim; ++j) pts[dim * dim + j] = midp[j];
        ms[dim] = &mid[cand * mc];
        double q = elem_quality_ms(dim, mc, pts, ms);
        minq = min2d(minq, q);
      }
    }
#pragma unroll
    for (int j = G / 2; j > 0; j >>= 1) minq = min2d(minq, __shfl_xor_sync(gm, minq, j, G));
    if (gl == 0) out[cand] = minq;
  });
}

// refine_products (src/Omega_h_refine_topology.cpp:13-205): per key, the two
// halves of every adjacent d-entity ("pairs"), then the (d+1)-entities'
// mid-cuts ("cuts")
static void refine_products(Mesh& m, int ed, const Arr<LO>& k2e, const Arr<LO>& k2mid,
                            const Arr<LO>& ov2nv, Arr<LO>& k2p, Arr<LO>& pv2v) {
  int dim = m.dim;
  LO nkeys = k2e.size();
  auto ke = cview(k2e);
  auto km = cview(k2mid);
  auto o2n = cview(ov2nv);
  auto ev = cview(m.ask_verts_of(1));
  LV pa = {nullptr, 0}, pb = {nullptr, 0}, ca = {nullptr, 0}, cb = {nullptr, 0};
  LV pdv = {nullptr, 0}, cdv = {nullptr, 0};
  View<const I8> pc = {nullptr, 0}, cc = {nullptr, 0};
  if (ed > EDGE) {
    const Adj& e2d = m.ask_up(1, ed);
    pa = cview(e2d.a2ab);
    pb = cview(e2d.ab2b);
    pc = cview(e2d.codes);
    pdv = cview(m.ask_verts_of(ed));
  }
  int cd = ed + 1;
  bool cuts = ed < dim;
  if (cuts) {
    const Adj& e2c = m.ask_up(1, cd);
    ca = cview(e2c.a2ab);
    cb = cview(e2c.ab2b);
    cc = cview(e2c.codes);
    cdv = cview(m.ask_verts_of(cd));
  }
  Arr<LO> cnt(nkeys);
  auto ct = view(cnt);
  pfor(nkeys, [=] __device__(LO k) {
    LO e = ke[k];
    LO np = ed == EDGE ? 2 : 2 * (pa[e + 1] - pa[e]);
    if (cuts) np += ca[e + 1] - ca[e];
    ct[k] = np;
  });
  k2p = offset_scan(cnt);
  int nppv = ed + 1;
  pv2v = Arr<LO>(last(k2p) * nppv);
  auto kp = cview(k2p);
  auto pv = view(pv2v);
  pfor(nkeys, [=] __device__(LO k) {
    LO e = ke[k];
    LO prod = kp[k];
    LO mid = km[k];
    if (ed == EDGE) {
      LO b = prod * 2;
      pv[b + 0] = o2n[ev[e * 2]];
      pv[b + 1] = mid;
      pv[b + 2] = mid;
      pv[b + 3] = o2n[ev[e * 2 + 1]];
      prod += 2;
    } else {
      for (LO x = pa[e]; x < pa[e + 1]; ++x) {
        LO dom = pb[x];
        int dde = code_which_down(pc[x]), rot = code_rotation(pc[x]);
        for (int eev = 0; eev < 2; ++eev) {
          int ddv = down_template(ed, 1, dde, eev ^ rot);
          int dds = opposite_template(ed, 0, ddv);
          LO tmp[4];
          for (int k2 = 0; k2 < ed; ++k2)
            tmp[k2] = o2n[pdv[dom * (ed + 1) + down_template(ed, ed - 1, dds, k2)]];
          tmp[ed] = mid;
          if (ed == 3) {
            LO t = tmp[1];
            tmp[1] = tmp[2];
            tmp[2] = t;
          }
          for (int k2 = 0; k2 <= ed; ++k2) pv[prod * nppv + k2] = tmp[k2];
          ++prod;
        }
      }
    }
    if (cuts) {
      for (LO x = ca[e]; x < ca[e + 1]; ++x) {
        LO dom = cb[x];
        int ddt = opposite_template(cd, 1, code_which_down(cc[x]));
        for (int k2 = 0; k2 < cd - 1; ++k2)
          pv[prod * nppv + k2] = o2n[cdv[dom * (cd + 1) + down_template(cd, cd - 2, ddt, k2)]];
        pv[prod * nppv + cd - 1] = mid;
        ++prod;
      }
    }
  });
}

// class tags: pairs inherit their split d-entity, cuts their (d+1)-entity
// (transfer_inherit_refine, src/Omega_h_transfer.cpp:213-263)
template <class T>
static void inherit_refine(Mesh& m, int d, const Arr<LO>& k2e, const Arr<LO>& k2p,
                           const Arr<T>* data, Arr<T>& prod) {
  int dim = m.dim;
  LO nkeys = k2e.size();
  auto ke = cview(k2e);
  auto kp = cview(k2p);
  LV pa = {nullptr, 0}, pb = {nullptr, 0}, ca = {nullptr, 0}, cb = {nullptr, 0};
  if (d > EDGE) {
    const Adj& a = m.ask_up(1, d);
    pa = cview(a.a2ab);
    pb = cview(a.ab2b);
  }
  bool cuts = d < dim, cut_is_edge = d + 1 == EDGE;
  if (cuts && !cut_is_edge) {
    const Adj& a = m.ask_up(1, d + 1);
    ca = cview(a.a2ab);
    cb = cview(a.ab2b);
  }
  View<const T> pdat = {nullptr, 0}, cdat = {nullptr, 0};
  if (d > VERT) pdat = cview(data[d]);
  if (cuts) cdat = cview(data[d + 1]);
  auto edat = cview(data[1]);
  auto o = view(prod);
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
    if (cuts) {
      if (cut_is_edge) {
        o[p++] = cdat[e];
      } else {
        for (LO x = ca[e]; x < ca[e + 1]; ++x) o[p++] = cdat[cb[x]];
      }
    }
  });
}

static bool refine(Mesh& m, const AdaptOpts& o, const Arr<LO>& c2e, PassStats* st) {
  m.parting = 1;  // ghosted (src/Omega_h_refine.cpp:85)
  int dim = m.dim, mc = m.mcomp();
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
    auto ce = cview(c2e);
    auto q = cview(cq);
    auto in = view(initial);
    auto e = view(eq);
    auto ag = view(anyg);
    double mqa = o.min_quality_allowed;
    pfor(nc, [=] __device__(LO i) {
      bool g = q[i] >= mqa;
      in[ce[i]] = g;
      e[ce[i]] = q[i];
      if (g) ag[0] = 1;
    });
  }
  if (!get_elem(anyg, 0)) return false;
  Arr<I8> keys = find_indset(m, EDGE, eq, initial);
  Arr<LO> k2e = collect_marked(keys);
  LO nkeys = k2e.size();
  st->refine_keys = nkeys;
  Mesh nm;
  nm.dim = dim;
  nm.rebuilt = true;  // element-based partitioning after a rebuild
  nm.metric_comps = m.metric_comps;
  nm.class_sets = m.class_sets;
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
    xfer_class(m, nm, d, mo, nnew, pcd.data(), pci.data(), nullptr);
    if (d == VERT) {
      Arr<double> pc(nkeys * dim);
      auto ev = cview(m.ask_verts_of(1));
      auto ke = cview(k2e);
      auto c = cview(m.coords);
      auto p = view(pc);
      pfor(nkeys, [=] __device__(LO k) {
        LO e = ke[k];
        for (int j = 0; j < dim; ++j) {
          double comp = 0;
          comp += c[ev[e * 2] * dim + j];
          comp += c[ev[e * 2 + 1] * dim + j];
          comp /= 2;
          p[k * dim + j] = comp;
        }
      });
      nm.coords = xfer(m.coords, mo, nnew, pc, dim);
      Arr<double> pm(nkeys * mc);
      mident_metrics(m, k2e.data(), nkeys, pm.data());
      nm.metric = xfer(m.metric, mo, nnew, pm, mc);
    }
    xfer_lengths_qualities(m, nm, d, mo, &pv2v);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

bool refine_by_size(Mesh& m, const AdaptOpts& o, PassStats* st) {
  const Arr<double>& len = m.ask_lengths();
  Arr<I8> cands(len.size());
  auto l = cview(len);
  auto c = view(cands);
  double mx = o.max_length_desired;
  pfor(len.size(), [=] __device__(LO i) { c[i] = l[i] > mx; });
  Arr<LO> c2e = collect_marked(cands);
  if (c2e.size() == 0) return false;
  return refine(m, o, c2e, st);
}

// ------------------------------------------------------------ coarsen
__device__ __forceinline__ bool collapses(I8 code, int v) { return (code & (1 << v)) != 0; }
__device__ __forceinline__ I8 dont_collapse(I8 code, int v) { return I8(code & ~(1 << v)); }

// check_collapse_class (src/Omega_h_check_collapse.cpp:10-45)
void check_collapse_class(Mesh& m, const LO* c2e_p, LO n, const I8* ci_p, I8* co_p) {
  auto ev = cview(m.ask_verts_of(1));
  auto vcd = cview(m.class_dim[0]);
  auto ecd = cview(m.class_dim[1]);
  auto c2e = cview(c2e_p, n);
  auto ci = cview(ci_p, n);
  auto co = view(co_p, n);
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

// The tet's local edge between local vertices a and b, as 4 bits at
// 4 * (a * 4 + b) of the returned word (from the edge template)
static unsigned long long tet_edge_lookup() {
  unsigned long long t = 0;
  for (int j = 0; j < 6; ++j) {
    int a = down_template(3, 1, j, 0), b = down_template(3, 1, j, 1);
    t |= (unsigned long long)j << (4 * (a * 4 + b));
    t |= (unsigned long long)j << (4 * (b * 4 + a));
  }
  return t;
}
__device__ __forceinline__ int tet_edge_between(unsigned long long lut, int a, int b) {
  return int((lut >> (4 * (a * 4 + b))) & 15u);
}

// check_collapse_exposure (src/Omega_h_check_collapse.cpp:69-119)
void check_collapse_exposure(Mesh& m, const LO* c2e_p, LO n, const I8* ci_p, I8* co_p) {
  auto c2e = cview(c2e_p, n);
  if (m.dim == 3) {
    // Both steps in one walk of the edge's tets.  The faces around the edge
    // are, in each tet around it, the two tet faces that hold the edge: face
    // {col, onto, w} is the one opposite the tet's fourth vertex, and its
    // side opposite onto is the tet edge {col, w}.  A face shared by two
    // tets is checked twice, with the same outcome; the steps only clear
    // bits, so their order does not change the result.
    const Adj& e2t = m.ask_up_any_order(EDGE, REGION);
    auto ea = cview(e2t.a2ab);
    auto eb = cview(e2t.ab2b);
    auto ecc = cview(e2t.codes);
    auto tf = cview(m.ask_down(REGION, FACE).ab2b);
    auto te = cview(m.ask_down(REGION, EDGE).ab2b);
    auto edim = cview(m.class_dim[EDGE]);
    auto fdim = cview(m.class_dim[FACE]);
    auto tdim = cview(m.class_dim[REGION]);
    auto in = cview(ci_p, n);
    auto out = view(co_p, n);
    unsigned long long lut = tet_edge_lookup();
    pfor(n, [=] __device__(LO c) {
      I8 code = in[c];
      if (!code) {
        out[c] = 0;
        return;
      }
      LO e = c2e[c];
      for (LO x = ea[e]; x < ea[e + 1]; ++x) {
        LO t = eb[x];
        int cce = code_which_down(ecc[x]), rot = code_rotation(ecc[x]);
        int l0 = down_template(3, 1, cce, rot), l1 = down_template(3, 1, cce, rot ^ 1);
        // the tet's two other vertices, and each one's face with the edge
        int w0 = -1, w1 = -1;
        for (int k = 0; k < 4; ++k)
          if (k != l0 && k != l1) (w0 < 0 ? w0 : w1) = k;
        int tcd = tdim[t];
        int fw0 = fdim[tf[t * 4 + opposite_template(3, 0, w1)]];  // {l0, l1, w0}
        int fw1 = fdim[tf[t * 4 + opposite_template(3, 0, w0)]];  // {l0, l1, w1}
        for (int col = 0; col < 2; ++col) {
          if (!collapses(code, col)) continue;
          int lc = col ? l1 : l0, lo = col ? l0 : l1;
          bool bad = fdim[tf[t * 4 + opposite_template(3, 0, lo)]] != tcd ||
                     edim[te[t * 6 + tet_edge_between(lut, lc, w0)]] != fw0 ||
                     edim[te[t * 6 + tet_edge_between(lut, lc, w1)]] != fw1;
          if (bad) code = dont_collapse(code, col);
        }
      }
      out[c] = code;
    });
    return;
  }
  Arr<I8> tmp(n);
  View<const I8> in = cview(ci_p, n);
  for (int cd = 2; cd <= m.dim; ++cd) {
    View<I8> out = cd == m.dim ? view(co_p, n) : view(tmp);
    const Adj& e2c = m.ask_up_any_order(1, cd);  // flags only: row order is free
    auto ea = cview(e2c.a2ab);
    auto eb = cview(e2c.ab2b);
    auto ecc = cview(e2c.codes);
    auto cs = cview(m.ask_down(cd, cd - 1).ab2b);
    auto cdim = cview(m.class_dim[cd]);
    auto sdim = cview(m.class_dim[cd - 1]);
    int nccs = simplex_degree(cd, cd - 1);
    pfor(n, [=] __device__(LO c) {
      I8 code = in[c];
      if (!code) {
        out[c] = 0;
        return;
      }
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
    in = {out.p, out.n};
  }
}

// The cavity of collapsing v_col onto v_onto: the elements around v_col that
// do not contain v_onto, with v_col replaced by v_onto.  Returns false for an
// element that dies in the collapse.
__device__ __forceinline__ bool collapse_elem(LV cv, int dim, LO el, int ccv_col, LO v_onto,
                                              LO vv[4]) {
  for (int k = 0; k <= dim; ++k) vv[k] = cv[el * (dim + 1) + k];
  for (int k = 0; k <= dim; ++k)
    if (k != ccv_col && vv[k] == v_onto) return false;
  vv[ccv_col & 3] = v_onto;
  return true;
}

constexpr int kMaxScreenCavity = 64;

// coarsen_qualities_tmpl (src/Omega_h_coarsen_qualities.cpp:15-63) with FP32
// screening: every cavity tet gets an enclosure [lo, hi] of its FP64 quality;
// only tets with lo <= min(1, min hi) can hold the cavity minimum, and only
// those are evaluated in FP64 (the same operations as the reference's), so
// the minimum is the reference's minimum.
static void coarsen_qualities_screened(Mesh& m, const LO* c2e_p, LO n, const I8* codes_p,
                                       double* q2_p) {
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto ev = cview(m.ask_verts_of(1));
  auto cv = cview(m.ask_verts_of(3));
  const Adj& v2c = m.ask_up(0, 3);
  auto va = cview(v2c.a2ab);
  auto vb = cview(v2c.ab2b);
  auto vc = cview(v2c.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto codes = cview(codes_p, n);
  auto q2 = view(q2_p, n * 2);
  unsigned long long* cnt = ctx().d_screen_counts;
  pfor(n, [=] __device__(LO cand) {
    LO e = c2e[cand];
    I8 code = codes[cand];
    unsigned nscreen = 0, nexact = 0;
    for (int col = 0; col < 2; ++col) {
      q2[cand * 2 + col] = -1.0;
      if (!collapses(code, col)) continue;
      LO v_col = ev[e * 2 + col], v_onto = ev[e * 2 + (1 - col)];
      LO x0 = va[v_col], x1 = va[v_col + 1];
      float lo[kMaxScreenCavity];
      float min_hi = 1.0f;
      int k = 0;
      for (LO x = x0; x < x1; ++x) {
        LO vv[4];
        if (!collapse_elem(cv, 3, vb[x], code_which_down(vc[x]), v_onto, vv)) continue;
        FIv b = tet_quality_bounds(sv, vv);
        if (k < kMaxScreenCavity) lo[k] = b.lo;
        ++k;
        min_hi = fminf(min_hi, b.hi);
      }
      bool all = k > kMaxScreenCavity;
      double minq = 1.0;
      int j = 0;
      for (LO x = x0; x < x1; ++x) {
        LO vv[4];
        if (!collapse_elem(cv, 3, vb[x], code_which_down(vc[x]), v_onto, vv)) continue;
        if (all || lo[j] <= min_hi) {
          minq = min2d(minq, tet_quality_exact(sv, c, mt, vv));
          ++nexact;
        }
        ++j;
      }
      nscreen += k;
      q2[cand * 2 + col] = minq;
    }
    warp_count(&cnt[0], nscreen);
    warp_count(&cnt[1], nexact);
  });
}

// coarsen_qualities_tmpl (src/Omega_h_coarsen_qualities.cpp:15-63)
void coarsen_qualities(Mesh& m, const LO* c2e_p, LO n, const I8* codes_p, double* q2_p) {
  int mc = m.mcomp();  // metric components per vertex (1: isotropic)
  int dim = m.dim;
  if (dim == 3 && ctx().screening) {
    coarsen_qualities_screened(m, c2e_p, n, codes_p, q2_p);
    return;
  }
  auto ev = cview(m.ask_verts_of(1));
  auto cv = cview(m.ask_verts_of(dim));
  const Adj& v2c = m.ask_up(0, dim);
  auto va = cview(v2c.a2ab);
  auto vb = cview(v2c.ab2b);
  auto vc = cview(v2c.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto codes = cview(codes_p, n);
  auto q2 = view(q2_p, n * 2);
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
        vv[ccv_col & 3] = v_onto;
        minq = min2d(minq, elem_quality_v(dim, c, mt, mc, vv));
      }
      q2[cand * 2 + col] = minq;
    }
  });
}

// choose_rails (src/Omega_h_collapse_rail.cpp:15-67)
void choose_rails(Mesh& m, const LO* c2e_p, LO n, const I8* codes_p, const double* quals2_p,
                  I8* vcand_p, double* vqual_p, GO* vrail_p) {
  LO nv = m.nverts();
  Arr<LO> e2c = fill<LO>(m.nedges(), -1);
  auto c2e = cview(c2e_p, n);
  {
    auto ec = view(e2c);
    pfor(n, [=] __device__(LO i) { ec[c2e[i]] = i; });
  }
  const Adj& v2e = m.ask_up(0, 1);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto vc = cview(v2e.codes);
  auto len = cview(m.ask_lengths());
  auto ec = cview(e2c);
  auto codes = cview(codes_p, n);
  auto quals2 = cview(quals2_p, n * 2);
  auto vcand = view(vcand_p, nv);
  auto vqual = view(vqual_p, nv);
  auto vrail = view(vrail_p, nv);
  pfor(nv, [=] __device__(LO v) {
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

// Exact FP64 minimum quality of the cavity of collapsing v_col onto v_onto,
// min(1, tet qualities): enclosures first, then FP64 only for the tets whose
// lower bound does not exceed the smallest upper bound.
template <int dim>
__device__ double collapse_min_exact(const ScreenView& sv, RV c, RV mt, LV cv, LV va, LV vb,
                                     View<const I8> vc, LO v_col, LO v_onto, unsigned* nexact) {
  LO x0 = va[v_col], x1 = va[v_col + 1];
  float min_hi = 1.0f;
  for (LO x = x0; x < x1; ++x) {
    LO vv[4];
    if (!collapse_elem(cv, dim, vb[x], code_which_down(vc[x]), v_onto, vv)) continue;
    min_hi = fminf(min_hi, elem_quality_bounds(dim, sv, vv).hi);
  }
  double minq = 1.0;
  for (LO x = x0; x < x1; ++x) {
    LO vv[4];
    if (!collapse_elem(cv, dim, vb[x], code_which_down(vc[x]), v_onto, vv)) continue;
    if (elem_quality_bounds(dim, sv, vv).lo <= min_hi) {
      minq = min2d(minq, elem_quality_exact(dim, sv, c, mt, vv));
      ++*nexact;
    }
  }
  return minq;
}

// ------------------------------------------------------------ vertex-centric screen
// The same screen, one warp per collapsing vertex v_col.  Every direction
// that collapses v_col screens the same star of elements with v_col moved
// onto another neighbour, so the warp stages the star once in shared memory:
// the neighbours' screening records (local index k+1 for the k-th edge of v's
// row, 0 for v), each star element as local indices, and one slot per
// direction.  Lanes then spread over the (direction, element) pairs and
// reduce each direction's bounds by shared atomic minima of order keys.  A
// direction's outcome is the sequential one's: it fails when the smallest
// upper bound is below the threshold, passes when the smallest lower bound
// reaches it, and is sent to the FP64 list otherwise.  Stars that do not fit
// the staging arrays are screened direction by direction from global memory.
// blocks of the vertex-centric screen: 128 threads, so that the 3D kernel's
// per-element invariants fit the static shared memory of a block
constexpr int kVsBlock = 128;
constexpr int kVsWarps = kVsBlock / 32;
constexpr int kVsMaxLocal = 32, kVsMaxElems = 64;
// 3D stars staged with their per-element invariants: at most 48 elements
// (larger stars take the per-direction path), so that six blocks fit an SM
constexpr int kVsMaxElems3 = 48;

struct CoarsenVertexArgs {
  LO nverts;
  int chunk;
  ScreenView sv;
  LV ev, cv, va, vb, ea, eb;
  View<const I8> vc, ec;
  View<const LO> e2cand;
  View<const I8> codes;
  View<double> q2;
  float mqa_f;
  // cubes of the threshold, rounded down and up (3D screens the cube of the
  // quality)
  float mqa3_dn, mqa3_up;
  // prevent_coarsen_overshoot in the same kernel (overshoot): a direction
  // whose new edges reach max_length gets q2 = -1 and is not screened
  bool overshoot;
  double max_length;
  RV elen;  // FP64 edge lengths (the rail choice's order)
  float ov_thr, ov_tdn;
  RV c, mt;
  int mc;
  unsigned long long* queue;  // [0] next vertex, [1] directions in the FP64 list
  LO* amb_dir;
  float* amb_mhi;
  unsigned long long* cnt;
};

// order-preserving int key of a float, and back
__device__ __forceinline__ int fkey(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// cubed: lo and hi bound the cube of the quality; the FP64 list takes the
// upper bound of the quality itself (a cube root rounded up)
__device__ __forceinline__ void screen_outcome(const CoarsenVertexArgs& a, LO d, float lo, float hi,
                                               bool cubed) {
  if (cubed ? hi < a.mqa3_dn : hi < a.mqa_f) {
    a.q2[d] = -1.0;  // fails
  } else if (cubed ? lo >= a.mqa3_up : lo >= a.mqa_f) {
    a.q2[d] = CUDART_NAN;  // passes on its enclosure
  } else {
    LO k = LO(atomicAdd(&a.queue[1], 1ULL));
    a.amb_dir[k] = d;
    a.amb_mhi[k] = cubed ? __fmul_ru(cbrtf(hi), 1.0f + 0x1p-20f) : hi;
    a.q2[d] = -1.0;  // replaced by the FP64 minimum
  }
}

template <int D>
__global__ void __launch_bounds__(kVsBlock, 7) k_coarsen_screen_v(CoarsenVertexArgs a) {
  constexpr int NV = D + 1;
  // 3D: per star element, the invariants of its face opposite the
  // collapsing vertex (tet_face_invariants), the slot of that vertex and the
  // face's first maxdet slot
  constexpr int kMaxE = D == 3 ? kVsMaxElems3 : kVsMaxElems;
  constexpr int kInv = D == 3 ? kVsMaxElems3 : 1;
  __shared__ TetFaceInv s_inv[kVsWarps][kInv];
  __shared__ unsigned char s_slot[kVsWarps][kInv];  // slot | first maxdet face slot << 4
  // (element, direction) pairs queued for screening: element * 32 + direction
  __shared__ unsigned short s_q[kVsWarps][64];
  __shared__ float4 s_h[kVsWarps][kVsMaxLocal], s_l[kVsWarps][kVsMaxLocal];
  __shared__ float4 s_ma[kVsWarps][kVsMaxLocal], s_mb[kVsWarps][kVsMaxLocal];
  __shared__ long long s_key[kVsWarps][kVsMaxLocal];
  __shared__ LO s_gid[kVsWarps][kVsMaxLocal];
  __shared__ LO s_dir[kVsWarps][kVsMaxLocal];  // direction of local vertex k as v_onto, or -1
  __shared__ int s_lo[kVsWarps][kVsMaxLocal], s_hi[kVsWarps][kVsMaxLocal];
  __shared__ unsigned char s_dk[kVsWarps][kVsMaxLocal];  // local indices of the directions
  __shared__ unsigned s_elem[kVsWarps][kMaxE];     // NV local indices, 8 bits each
  // per local vertex: which end of its edge with v is v (the new edge to the
  // vertex moved onto keeps the edge's orientation), and whether the
  // direction onto it overshoots
  __shared__ unsigned char s_end[kVsWarps][kVsMaxLocal], s_over[kVsWarps][kVsMaxLocal];
  // direction index of each local vertex, and the current length group's
  // directions (local indices)
  __shared__ unsigned char s_dt[kVsWarps][kVsMaxLocal], s_gk[kVsWarps][kVsMaxLocal];
  const unsigned full = 0xffffffffu;
  const int w = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31u);
  unsigned nscreen = 0;
  LO next = 0, end = 0;
  for (;;) {
    if (next >= end) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&a.queue[0], (unsigned long long)a.chunk);
      base = __shfl_sync(full, base, 0);
      if (base >= (unsigned long long)a.nverts) break;
      next = LO(base);
      end = next + a.chunk < a.nverts ? next + a.chunk : a.nverts;
    }
    const LO v = next++;
    const LO e0 = a.ea[v], ne = a.ea[v + 1] - e0;
    // the directions with v as v_col; non-collapsing directions of candidate
    // edges fail outright
    bool fits = ne + 1 <= kVsMaxLocal;
    unsigned any = 0;
    for (LO kb = 0; kb < ne; kb += 32) {
      LO k = kb + lane;
      LO dir = -1;
      if (k < ne) {
        LO e = a.eb[e0 + k];
        LO cand = a.e2cand[e];
        if (cand >= 0) {
          int col = code_which_down(a.ec[e0 + k]);
          LO d = cand * 2 + col;
          if (collapses(a.codes[cand], col)) dir = d;
          else a.q2[d] = -1.0;
        }
        if (fits) s_dir[w][k + 1] = dir;
      }
      any |= __ballot_sync(full, dir >= 0);
    }
    if (!any) continue;
    const LO s0 = a.va[v], S = a.va[v + 1] - s0;
    fits = fits && S <= kMaxE;
    if (fits) {
      // stage the local vertices and the star's elements
      for (LO k = lane; k <= ne; k += 32) {
        LO u = v;
        if (k > 0) {
          LO e = a.eb[e0 + k - 1];
          u = a.ev[e * 2 + (1 - code_which_down(a.ec[e0 + k - 1]))];
        }
        s_gid[w][k] = u;
        s_h[w][k] = a.sv.xh[u];
        s_l[w][k] = a.sv.xl[u];
        s_ma[w][k] = a.sv.ma[u];
        s_mb[w][k] = a.sv.mb[u];
        s_key[w][k] = a.sv.dkey[u];
        s_lo[w][k] = fkey(1.0f);
        s_hi[w][k] = fkey(1.0f);
        s_end[w][k] = k > 0 ? (unsigned char)code_which_down(a.ec[e0 + k - 1]) : 0;
        s_over[w][k] = 0;
      }
      __syncwarp();
      bool found = true;
      for (LO x = lane; x < S; x += 32) {
        LO el = a.vb[s0 + x];
        int pos = code_which_down(a.vc[s0 + x]);
        unsigned packed = 0;
        bool here = true;
        // the element's other vertices among the local ones: one pass over
        // the local list for all of them (v itself, slot pos, is local 0)
        LO u[NV];
        unsigned li[NV];
        for (int j = 0; j < NV; ++j) {
          u[j] = j != pos ? a.cv[el * NV + j] : LO(-1);
          li[j] = j != pos ? 255u : 0u;
        }
        for (LO k = 1; k <= ne; ++k) {
          LO g = s_gid[w][k];
          for (int j = 0; j < NV; ++j)
            if (u[j] == g) li[j] = unsigned(k);
        }
        for (int j = 0; j < NV; ++j) {
          if (li[j] == 255u) here = false;
          packed |= li[j] << (8 * j);
        }
        s_elem[w][x] = packed;
        found = found && here;
        if constexpr (D == 3) {
          if (here) {
            // the face's slots in order, without the collapsing vertex's
            int j0 = pos == 0 ? 1 : 0, j1 = pos <= 1 ? 2 : 1, j2 = pos <= 2 ? 3 : 2;
            int f0 = int((packed >> (8 * j0)) & 255u), f1 = int((packed >> (8 * j1)) & 255u),
                f2 = int((packed >> (8 * j2)) & 255u);
            float4 hf[3] = {s_h[w][f0], s_h[w][f1], s_h[w][f2]};
            float4 lf[3] = {s_l[w][f0], s_l[w][f1], s_l[w][f2]};
            long long k0 = s_key[w][f0], k1 = s_key[w][f1], k2 = s_key[w][f2];
            int fb = j0;
            long long kb = k0;
            if (k1 > kb) {
              fb = j1;
              kb = k1;
            }
            if (k2 > kb) fb = j2;
            s_inv[w][x] = tet_face_invariants(hf, lf, pos);
            s_slot[w][x] = (unsigned char)(pos | (fb << 4));
          }
        }
      }
      fits = __all_sync(full, found);
      __syncwarp();
    }
    if (!fits) {
      // direction by direction, each lane one direction, from global memory
      for (LO kb = 0; kb < ne; kb += 32) {
        LO k = kb + lane;
        LO d = -1, v_onto = 0;
        if (k < ne) {
          LO e = a.eb[e0 + k];
          LO cand = a.e2cand[e];
          int col = code_which_down(a.ec[e0 + k]);
          if (cand >= 0 && collapses(a.codes[cand], col)) {
            d = cand * 2 + col;
            v_onto = a.ev[e * 2 + (1 - col)];
          }
        }
        if (d >= 0 && a.overshoot) {
          // prevent_coarsen_overshoot for this direction, as the separate
          // kernel decides it
          LenCut cut = len_cut(a.ov_tdn, a.ov_thr);
          unsigned nl = 0, nx = 0;
          for (LO x = e0; x < e0 + ne; ++x) {
            LO e2 = a.eb[x];
            int ein = code_which_down(a.ec[x]), eout = 1 - ein;
            LO nv[2];
            nv[ein] = v_onto;
            nv[eout] = a.ev[e2 * 2 + eout];
            if (nv[eout] == v_onto) continue;  // the collapsing edge
            float qlo[2], qhi[2];
            bool qok = edge_q_bounds_d(D, a.sv, nv[0], nv[1], qlo, qhi);
            int side = len_cut_side(qlo, qhi, qok, cut);
            ++nl;
            bool over;
            if (side != 0) {
              over = side > 0;
            } else {
              FIv L = qok ? len_from_q(qlo, qhi) : widen_all();
              if (L.lo >= a.ov_thr) {
                over = true;
              } else if (L.hi < a.ov_thr) {
                over = false;
              } else {
                over = edge_len_v(D, a.c, a.mt, a.mc, nv[0], nv[1]) >= a.max_length;
                ++nx;
              }
            }
            if (over) {
              a.q2[d] = -1.0;
              d = -1;
              break;
            }
          }
          atomicAdd(&a.cnt[2], (unsigned long long)nl);
          if (nx) atomicAdd(&a.cnt[3], (unsigned long long)nx);
        }
        if (d >= 0) {
          float lo = 1.0f, hi = 1.0f;
          for (LO x = s0; x < s0 + S && !(hi < a.mqa_f); ++x) {
            LO vv[4];
            if (collapse_elem(a.cv, D, a.vb[x], code_which_down(a.vc[x]), v_onto, vv)) {
              FIv b = elem_quality_bounds(D, a.sv, vv);
              lo = fminf(lo, b.lo);
              hi = fminf(hi, b.hi);
              ++nscreen;
            }
          }
          screen_outcome(a, d, lo, hi, false);
        }
      }
      __syncwarp();
      continue;
    }
    // the directions' local indices, in order
    int nd = 0;
    for (LO kb = 1; kb <= ne; kb += 32) {
      LO k = kb + lane;
      bool is = k <= ne && s_dir[w][k] >= 0;
      unsigned m = __ballot_sync(full, is);
      if (is) {
        int t = nd + __popc(m & ((1u << lane) - 1u));
        s_dk[w][t] = (unsigned char)k;
        s_dt[w][k] = (unsigned char)t;
      }
      nd += __popc(m);
    }
    __syncwarp();
    // (element, direction) pairs, element by element: pair p = x * nd + t
    // is direction t on element x.  A pair whose element contains the vertex
    // moved onto is not in the direction's cavity.  Every direction walks
    // its cavity in element order, and one whose upper bound fell below the
    // threshold skips the rest (its minimum only falls, as the sequential
    // screen stops at its first failing element); a direction that is not
    // skipped is screened in full, so its bounds do not depend on the
    // schedule.  The warp scans the pairs 32 at a time and queues the ones
    // to screen in shared memory (ballot compaction); it screens 32 queued
    // pairs at a time, one per lane.
    constexpr bool cubed = D == 3;
    const float fail_below = cubed ? a.mqa3_dn : a.mqa_f;
    const float pass_from = cubed ? a.mqa3_up : a.mqa_f;
    // choose_rails (src/Omega_h_collapse_rail.cpp:19-77) takes at each vertex
    // the shortest edge whose collapse passes (ties by quality), so the
    // directions are screened in groups of equal length, shortest first:
    // once a group holds a direction that surely passes (its lower bound
    // clears the threshold and it does not overshoot), no longer direction
    // can be the rail, and those are not screened (q2 = -1: they do not
    // collapse, which leaves the rail choice as it is).  A group whose
    // directions only straddle the threshold does not end the search: their
    // FP64 minima decide later.
    // The first two groups go one at a time and the rest together: each
    // round costs its own pass over the star, and the search ends within
    // the first two groups at most vertices.
    double mylen = INFINITY;
    if (lane < nd) mylen = a.elen[a.eb[e0 + s_dk[w][lane] - 1]];
    unsigned todo = nd >= 32 ? full : ((1u << nd) - 1u), skipped = 0u;
    for (int round = 0; todo; ++round) {
      double ml = ((todo >> lane) & 1u) ? mylen : INFINITY;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ml = fmin(ml, __shfl_xor_sync(full, ml, o));
      const unsigned grp =
          round < 2 ? __ballot_sync(full, ((todo >> lane) & 1u) && mylen == ml) : todo;
      todo &= ~grp;
      const int ng = __popc(grp);
      if ((grp >> lane) & 1u) s_gk[w][__popc(grp & ((1u << lane) - 1u))] = s_dk[w][lane];
      __syncwarp();
      const int npairs = S * ng;
      const float rnd = 1.0f / float(ng);
      int p0 = 0, qn = 0;
      for (;;) {
        while (qn < 32 && p0 < npairs) {
          int p = p0 + lane;
          bool take = false;
          int x = 0, t = 0;
          if (p < npairs) {
            x = int((float(p) + 0.5f) * rnd);  // p / ng: exact for p < 2^12, ng <= 32
            t = p - x * ng;
            int k = s_gk[w][t];
            take = __vcmpeq4(s_elem[w][x], unsigned(k) * 0x01010101u) == 0u &&  // not v_onto's
                   !(fkey_inv(s_hi[w][k]) < fail_below);
          }
          unsigned m = __ballot_sync(full, take);
          if (take) s_q[w][qn + __popc(m & ((1u << lane) - 1u))] = (unsigned short)(x * 32 + t);
          qn += __popc(m);
          p0 += 32;
        }
        if (qn == 0) break;
        __syncwarp();
        const int nq = qn < 32 ? qn : 32;
        if (lane < nq) {
          unsigned qe = s_q[w][lane];
          int x = int(qe >> 5), t = int(qe & 31u);
          int k = s_gk[w][t];
          if (!(fkey_inv(s_hi[w][k]) < fail_below)) {
            unsigned packed = s_elem[w][x];
            FIv b;
            if constexpr (D == 3) {
              // the face's vertices in slot order, the vertex moved onto at the
              // collapsing vertex's slot; maxdet as in slot order: the face's
              // first maximum against k, k first on a tie if its slot comes first
              unsigned sl = s_slot[w][x];
              int pos = int(sl & 15u), fb = int(sl >> 4);
              int j0 = pos == 0 ? 1 : 0, j1 = pos <= 1 ? 2 : 1, j2 = pos <= 2 ? 3 : 2;
              int f0 = int((packed >> (8 * j0)) & 255u), f1 = int((packed >> (8 * j1)) & 255u),
                  f2 = int((packed >> (8 * j2)) & 255u);
              float4 hf[3] = {s_h[w][f0], s_h[w][f1], s_h[w][f2]};
              float4 lf[3] = {s_l[w][f0], s_l[w][f1], s_l[w][f2]};
              int lfb = int((packed >> (8 * fb)) & 255u);
              long long kf = s_key[w][lfb], kp = s_key[w][k];
              int best = (kp > kf || (kp == kf && pos < fb)) ? k : lfb;
              b = tet_face_bounds<true>(s_inv[w][x], hf, lf, s_h[w][k], s_l[w][k], s_ma[w][best],
                                        s_mb[w][best]);
            } else {
              int li[NV];
              for (int jj = 0; jj < NV; ++jj) {
                li[jj] = int((packed >> (8 * jj)) & 255u);
                if (li[jj] == 0) li[jj] = k;  // v_col moved onto v_onto
              }
              int best = 0;
              long long bk = s_key[w][li[0]];
              for (int jj = 1; jj < NV; ++jj) {
                long long kk = s_key[w][li[jj]];
                if (kk > bk) {
                  best = jj;
                  bk = kk;
                }
              }
              float4 h[NV], l[NV];
              for (int jj = 0; jj < NV; ++jj) {
                h[jj] = s_h[w][li[jj]];
                l[jj] = s_l[w][li[jj]];
              }
              b = tri_quality_bounds_of(h, l, s_ma[w][li[best]], s_mb[w][li[best]]);
            }
            atomicMin(&s_lo[w][k], fkey(b.lo));
            atomicMin(&s_hi[w][k], fkey(b.hi));
            ++nscreen;
          }
        }
        __syncwarp();
        // move the rest of the queue (fewer than 32) to its front
        const int rest = qn - nq;
        unsigned short mv = lane < rest ? s_q[w][nq + lane] : (unsigned short)0;
        __syncwarp();
        if (lane < rest) s_q[w][lane] = mv;
        qn = rest;
        __syncwarp();
      }
      if (a.overshoot) {
        // prevent_coarsen_overshoot (src/Omega_h_coarsen_overshoot.cpp:11-49)
        // for the directions the quality screen has not failed: the new edges
        // from each direction's vertex moved onto to v's other neighbours,
        // (direction, neighbour) pairs over the lanes; a direction with a new
        // edge at or above max_length does not collapse.  The two checks are
        // both required of a direction, so either order gives the same
        // decisions; this order skips the edges of the many directions that
        // fail on quality.  Its outcome does not depend on which over-long
        // edge is found first.
        const LenCut cut = len_cut(a.ov_tdn, a.ov_thr);
        const int npo = ng * ne;
        const float rne = 1.0f / float(ne);
        unsigned nl = 0, nx = 0;
        for (int p = lane; p < npo; p += 32) {
          int t = int((float(p) + 0.5f) * rne);  // p / ne: exact for p < 2^12, ne <= 31
          int wl = p - t * ne + 1;
          int k = s_gk[w][t];
          if (wl == k || s_over[w][k] || fkey_inv(s_hi[w][k]) < fail_below) continue;
          // the new edge keeps the orientation of v's edge to wl, with k for v
          int ein = s_end[w][wl];
          int ia = ein == 0 ? k : wl, ib = ein == 0 ? wl : k;
          float qlo[2], qhi[2];
          bool qok = edge_q_bounds_rec<D>(s_h[w][ia], s_l[w][ia], s_ma[w][ia], s_mb[w][ia],
                                          s_h[w][ib], s_l[w][ib], s_ma[w][ib], s_mb[w][ib], qlo, qhi);
          int side = len_cut_side(qlo, qhi, qok, cut);
          ++nl;
          bool over;
          if (side != 0) {
            over = side > 0;
          } else {
            FIv L = qok ? len_from_q(qlo, qhi) : widen_all();
            if (L.lo >= a.ov_thr) {
              over = true;
            } else if (L.hi < a.ov_thr) {
              over = false;
            } else {
              over = edge_len_v(D, a.c, a.mt, a.mc, s_gid[w][ia], s_gid[w][ib]) >= a.max_length;
              ++nx;
            }
          }
          if (over) s_over[w][k] = 1;
        }
        warp_count_full(&a.cnt[2], nl);
        warp_count_full(&a.cnt[3], nx);
        __syncwarp();
      }
      // a surely passing direction ends the search
      bool sure = false;
      if (lane < ng) {
        int k = s_gk[w][lane];
        sure = !s_over[w][k] && fkey_inv(s_lo[w][k]) >= pass_from;
      }
      if (__any_sync(full, sure)) {
        skipped = todo;
        break;
      }
    }
    for (LO k = 1 + lane; k <= ne; k += 32) {
      LO d = s_dir[w][k];
      if (d < 0) continue;
      if ((skipped >> s_dt[w][k]) & 1u) {
        a.q2[d] = -1.0;  // longer than a surely passing direction: not the rail
      } else if (s_over[w][k]) {
        a.q2[d] = -1.0;  // overshoots: does not collapse
      } else {
        screen_outcome(a, d, fkey_inv(s_lo[w][k]), fkey_inv(s_hi[w][k]), cubed);
      }
    }
    __syncwarp();
  }
  warp_count_full(a.cnt, nscreen);
}

// grid of a persistent kernel: as many blocks of the given size as stay
// resident on the device, and no more than the work needs
template <class K>
static unsigned persistent_blocks(K kernel, int block, long long work_warps) {
  thread_local std::map<int, int> per_sm_of;  // per host thread: no locking
  int& per_sm = per_sm_of[block];
  if (per_sm == 0) {
    OHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0));
    if (per_sm < 1) per_sm = 1;
  }
  long long full = (long long)per_sm * ctx().num_sms;
  long long need = (work_warps * 32 + block - 1) / block;
  long long b = need < full ? need : full;
  return unsigned(b < 1 ? 1 : b);
}

// prevent_coarsen_overshoot with FP32 screening of the new edge lengths:
// an enclosure of each FP64 length settles "length >= max_length" unless the
// threshold lies inside it; those lengths are computed in FP64.
template <int D>
static void prevent_coarsen_overshoot_screened_d(Mesh& m, double max_length, const LO* c2e_p,
                                                 LO n, const I8* ci_p, I8* co_p) {
  constexpr int dim = D, mc = D == 3 ? 6 : 3;
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto ev = cview(m.ask_verts_of(1));
  const Adj& v2e = m.ask_up(0, 1);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto vc = cview(v2e.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto ci = cview(ci_p, n);
  auto co = view(co_p, n);
  float thr = float_at_or_above(max_length);  // for float x: x >= max_length <=> x >= thr
  float tdn = float_at_or_below(max_length);
  unsigned long long* cnt = ctx().d_screen_counts;
  pfor(n, [=] __device__(LO cand) {
    LO e = c2e[cand];
    I8 code = ci[cand];
    unsigned nscreen = 0, nexact = 0;
    LenCut cut = len_cut(tdn, thr);
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
        float qlo[2], qhi[2];
        bool qok = edge_q_bounds_d(dim, sv, nv[0], nv[1], qlo, qhi);
        int side = len_cut_side(qlo, qhi, qok, cut);
        ++nscreen;
        bool over;
        if (side != 0) {
          over = side > 0;
        } else {
          FIv L = qok ? len_from_q(qlo, qhi) : widen_all();
          if (L.lo >= thr) {
            over = true;
          } else if (L.hi < thr) {
            over = false;
          } else {
            over = edge_len_v(dim, c, mt, mc, nv[0], nv[1]) >= max_length;
            ++nexact;
          }
        }
        if (over) {
          code = dont_collapse(code, col);
          break;
        }
      }
    }
    co[cand] = code;
    warp_count(&cnt[2], nscreen);
    warp_count(&cnt[3], nexact);
  });
}
static void prevent_coarsen_overshoot_screened(Mesh& m, double max_length, const LO* c2e_p,
                                               LO n, const I8* ci_p, I8* co_p) {
  if (m.dim == 3)
    prevent_coarsen_overshoot_screened_d<3>(m, max_length, c2e_p, n, ci_p, co_p);
  else
    prevent_coarsen_overshoot_screened_d<2>(m, max_length, c2e_p, n, ci_p, co_p);
}

// prevent_coarsen_overshoot (src/Omega_h_coarsen_overshoot.cpp:11-49)
void prevent_coarsen_overshoot(Mesh& m, double max_length, const LO* c2e_p, LO n,
                               const I8* ci_p, I8* co_p) {
  if (ctx().screening) {
    prevent_coarsen_overshoot_screened(m, max_length, c2e_p, n, ci_p, co_p);
    return;
  }
  auto ev = cview(m.ask_verts_of(1));
  const Adj& v2e = m.ask_up(0, 1);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto vc = cview(v2e.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  int dim = m.dim, mc = m.mcomp();
  auto c2e = cview(c2e_p, n);
  auto ci = cview(ci_p, n);
  auto co = view(co_p, n);
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
        if (edge_len_v(dim, c, mt, mc, nv[0], nv[1]) >= max_length) {
          code = dont_collapse(code, col);
          break;
        }
      }
    }
    co[cand] = code;
  });
}

// The quality filter of coarsen_by_size (src/Omega_h_coarsen.cpp:29-58 with
// coarsen_qualities and filter_coarsen_min_qual) from enclosures: a
// direction whose enclosure of min(1, cavity qualities) lies on one side of
// min_quality_allowed is decided without FP64; the others get their FP64
// minimum.  q2 holds the FP64 minimum where it was computed and NaN where the
// direction passed on its enclosure (its value is computed later only if
// choose_rails_lazy needs it).
template <int D>
static void coarsen_filter_lazy_d(Mesh& m, const LO* c2e_p, LO n, I8* codes_p, double mqa,
                                  double* q2_p, double max_length) {
  constexpr int dim = D;
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto ev = cview(m.ask_verts_of(1));
  auto cv = cview(m.ask_verts_of(dim));
  const Adj& v2c = m.ask_up(0, dim);
  auto va = cview(v2c.a2ab);
  auto vb = cview(v2c.ab2b);
  auto vc = cview(v2c.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto codes = view(codes_p, n);
  auto q2 = view(q2_p, n * 2);
  unsigned long long* cnt = ctx().d_screen_counts;
  float mqa_f = float_at_or_above(mqa);  // for float x: x >= mqa <=> x >= mqa_f
  // floats below and above the exact cube of mqa (the double product is
  // within 2.1 u_double of it)
  double mqa3 = mqa * mqa * mqa;
  float mqa3_dn = float_at_or_below(mqa3 * (1.0 - 0x1p-50));
  float mqa3_up = float_at_or_above(mqa3 * (1.0 + 0x1p-50));
  // algorithmic bytes: candidates in and codes and q2 out, the candidate
  // edges' vertices, vertex-to-element rows, element vertices and the
  // per-vertex screening data, each read once
  LO nV = m.nverts(), nT = m.nelems();
  double bytes = double(n) * (4 + 1 + 8 + 1 + 16) + double(nV + 1) * 4 +
                 double(v2c.ab2b.size()) * 5 + double(nT) * 4 * (dim + 1) + double(nV) * 80;
  LO ndirs = LO(2LL * n);
  if (2LL * n > 0x7fffffffLL) throw Error(8, "coarsen filter: too many candidates");
  Arr<unsigned long long> queue = fill<unsigned long long>(2, 0ULL);
  Arr<LO> amb_dir(ndirs);
  Arr<float> amb_mhi(ndirs);
  // candidate index of each edge (-1: not a candidate), for the vertex rows
  const Adj& v2e = m.ask_up(0, 1);
  LO nE = m.nedges();
  Arr<LO> e2cand(nE);
  OHG_CUDA(cudaMemsetAsync(e2cand.data(), 0xff, size_t(nE) * sizeof(LO), ctx().stream));
  {
    auto e2c = view(e2cand);
    pfor(n, [=] __device__(LO cand) { e2c[c2e[cand]] = cand; });
  }
  // tuned launch shape: vertices taken 8 or 4 at a time (the results do not
  // depend on it); blocks of 256 threads
  Ctx& cx = ctx();
  int var = cx.tuner.select("coarsen_screen_v", D, nV, 2, 0, cx.stream);
  bool timed = cx.tuner.open >= 0;
  int block = kVsBlock, chunk = (var & 1) ? 4 : 8;
  bool overshoot = max_length >= 0.0;
  float ov_thr = overshoot ? float_at_or_above(max_length) : 0.0f;
  float ov_tdn = overshoot ? float_at_or_below(max_length) : 0.0f;
  CoarsenVertexArgs args{nV,   chunk, sv,   ev,   cv,
                         va,   vb,    cview(v2e.a2ab), cview(v2e.ab2b), vc,
                         cview(v2e.codes), cview(e2cand), cview(codes_p, n), q2, mqa_f,
                         mqa3_dn, mqa3_up, overshoot, max_length, cview(m.ask_lengths()), ov_thr,
                         ov_tdn, c, mt, m.mcomp(), queue.data(), amb_dir.data(), amb_mhi.data(),
                         &cnt[0]};
  // the edge-to-candidate map, the vertex-to-edge rows and the FP64 edge
  // lengths (the rail order)
  bytes += double(nE) * (4 + 8) + double(nV + 1) * 4 + double(v2e.ab2b.size()) * 5;
  {
    KernelTimer timer("coarsen_filter", bytes);
    unsigned nb = persistent_blocks(k_coarsen_screen_v<D>, block, (nV + chunk - 1) / chunk);
    k_coarsen_screen_v<D><<<nb, block, 0, cx.stream>>>(args);
    if (timed) cx.tuner.stop(cx.stream);
    ++cx.launches;
#ifdef OHG_CHECKED
    checked_after_launch(__FILE__, __LINE__);
#endif
  }
  // FP64 minima of the straddling directions: of each one's cavity, the
  // elements whose lower bound does not exceed the smallest upper bound are
  // evaluated in FP64 and reduced to their minimum (the minimum of a set of
  // doubles does not depend on the order of evaluation).  One group of lanes
  // per direction, the directions' number read on the device: no host wait
  // for it.
  {
    const unsigned long long* qn = queue.data() + 1;
    auto ad = cview(amb_dir);
    auto am = cview(amb_mhi);
    constexpr int G = kCavityLanes;
    LO slots = LO(std::min<long long>(ndirs, (long long)cx.num_sms * (2048 / G)));
    group_for(G, slots, kBlock, [=] __device__(LO s, int gl, unsigned gm) {
      if (s < 0) return;
      LO K = LO(*qn);
      unsigned nfp64 = 0;
      for (LO k = s; k < K; k += slots) {
        LO d = ad[k], e = c2e[d >> 1];
        int col = d & 1;
        LO v_col = ev[e * 2 + col], v_onto = ev[e * 2 + (1 - col)];
        float mh = am[k];
        long long best = order_key(1.0);
        LO x1 = va[v_col + 1];
        for (LO xb = va[v_col]; xb < x1; xb += G) {
          LO x = xb + gl;
          LO vv[4];
          if (x < x1 && collapse_elem(cv, dim, vb[x], code_which_down(vc[x]), v_onto, vv) &&
              elem_quality_bounds(dim, sv, vv).lo <= mh) {
            long long q = order_key(elem_quality_exact(dim, sv, c, mt, vv));
            best = q < best ? q : best;
            ++nfp64;
          }
        }
#pragma unroll
        for (int j = G / 2; j > 0; j >>= 1) {
          long long o = __shfl_xor_sync(gm, best, j, G);
          best = o < best ? o : best;
        }
        if (gl == 0) q2[ad[k]] = key_to_double(best);
      }
      warp_count(&cnt[1], nfp64);
    });
  }
  // the decisions: a direction passes on its enclosure (NaN) or on its FP64
  // minimum; -1 marks a failed or non-collapsing direction
  pfor(n, [=] __device__(LO cand) {
    I8 code = codes[cand];
    for (int col = 0; col < 2; ++col) {
      double q = q2[cand * 2 + col];
      if (collapses(code, col) && !(q != q || q >= mqa)) code = dont_collapse(code, col);
    }
    codes[cand] = code;
  });
}
// max_length >= 0: prevent_coarsen_overshoot with that limit in the same
// kernel, before the quality screen (a direction that overshoots gets
// q2 = -1 and loses its collapse bit)
static void coarsen_filter_lazy(Mesh& m, const LO* c2e_p, LO n, I8* codes_p, double mqa,
                                double* q2_p, double max_length = -1.0) {
  if (m.dim == 3)
    coarsen_filter_lazy_d<3>(m, c2e_p, n, codes_p, mqa, q2_p, max_length);
  else
    coarsen_filter_lazy_d<2>(m, c2e_p, n, codes_p, mqa, q2_p, max_length);
}

// FP64 minima min(1, cavity qualities) of K collapse cavities (v_col[k] onto
// v_onto[k]; every v_col distinct), written to out[k].  Enclosures select the
// tets that can hold each minimum; those are gathered into one dense list so
// that the FP64 evaluations run in full warps (GB300's FP64 pipe is narrow,
// and a divergent warp occupies it as long as a full one).
template <int D>
static void collapse_minima_exact_d(Mesh& m, const ScreenView& sv, const Arr<LO>& vcol,
                                    const Arr<LO>& vonto, double* out_p) {
  LO K = vcol.size();
  if (K == 0) return;
  constexpr int dim = D;
  auto cv = cview(m.ask_verts_of(dim));
  const Adj& v2t = m.ask_up(0, dim);
  auto ta = cview(v2t.a2ab);
  auto tb = cview(v2t.ab2b);
  auto tc = cview(v2t.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto vcv = cview(vcol);
  auto vov = cview(vonto);
  Arr<float> lo_at(v2t.ab2b.size());
  Arr<float> mhi(K);
  Arr<LO> cnt(K);
  {
    // kCavityLanes lanes per cavity; in 3D the bounds are of the cube of
    // the quality (no cube root), a monotone scale for the selection
    // lo <= min hi below
    auto lo = view(lo_at);
    auto mh = view(mhi);
    auto ct = view(cnt);
    constexpr int G = kCavityLanes;
    group_for(G, K, kBlock, [=] __device__(LO k, int gl, unsigned gm) {
      if (k < 0) return;
      LO v = vcv[k], onto = vov[k];
      LO x0 = ta[v], x1 = ta[v + 1];
      float min_hi = 1.0f;
      for (LO x = x0 + gl; x < x1; x += G) {
        LO vv[4];
        if (!collapse_elem(cv, dim, tb[x], code_which_down(tc[x]), onto, vv)) {
          lo[x] = INFINITY;
          continue;
        }
        FIv b = D == 3 ? tet_quality_bounds<true>(sv, vv) : elem_quality_bounds(dim, sv, vv);
        lo[x] = b.lo;
        min_hi = fminf(min_hi, b.hi);
      }
#pragma unroll
      for (int j = G / 2; j > 0; j >>= 1) min_hi = fminf(min_hi, __shfl_xor_sync(gm, min_hi, j, G));
      __syncwarp(gm);
      LO n = 0;
      for (LO x = x0 + gl; x < x1; x += G) n += lo[x] <= min_hi;
#pragma unroll
      for (int j = G / 2; j > 0; j >>= 1) n += __shfl_xor_sync(gm, n, j, G);
      if (gl == 0) {
        mh[k] = min_hi;
        ct[k] = n;
      }
    });
  }
  Arr<LO> offs = offset_scan(cnt);
  LO ntot = last(offs);
  Arr<LO> tets(ntot * 4);  // dim + 1 vertices per entry, stride 4
  {
    auto lo = cview(lo_at);
    auto mh = cview(mhi);
    auto of = cview(offs);
    auto tt = view(tets);
    pfor(K, [=] __device__(LO k) {
      LO v = vcv[k], onto = vov[k];
      LO j = of[k];
      for (LO x = ta[v]; x < ta[v + 1]; ++x) {
        if (!(lo[x] <= mh[k])) continue;
        LO vv[4] = {0, 0, 0, 0};
        collapse_elem(cv, dim, tb[x], code_which_down(tc[x]), onto, vv);
        for (int q = 0; q < 4; ++q) tt[j * 4 + q] = vv[q];
        ++j;
      }
    });
  }
  Arr<double> eq(ntot);
  {
    auto tt = cview(tets);
    auto q = view(eq);
    pfor(ntot, [=] __device__(LO j) {
      LO vv[4] = {tt[j * 4], tt[j * 4 + 1], tt[j * 4 + 2], tt[j * 4 + 3]};
      q[j] = elem_quality_exact(dim, sv, c, mt, vv);
    });
  }
  unsigned long long* counts = ctx().d_screen_counts;
  {
    auto of = cview(offs);
    auto q = cview(eq);
    auto out = view(out_p, K);
    pfor(K, [=] __device__(LO k) {
      double minq = 1.0;
      for (LO j = of[k]; j < of[k + 1]; ++j) minq = min2d(minq, q[j]);
      out[k] = minq;
      warp_count(&counts[1], unsigned(of[k + 1] - of[k]));
    });
  }
}
static void collapse_minima_exact(Mesh& m, const ScreenView& sv, const Arr<LO>& vcol,
                                  const Arr<LO>& vonto, double* out_p) {
  if (m.dim == 3)
    collapse_minima_exact_d<3>(m, sv, vcol, vonto, out_p);
  else
    collapse_minima_exact_d<2>(m, sv, vcol, vonto, out_p);
}

// choose_rails (src/Omega_h_collapse_rail.cpp:15-67) on lazily known
// qualities.  The reference keeps, per vertex, the shortest candidate edge
// that collapses the vertex, the higher quality on equal lengths and the
// earlier edge on equal both: that is the first edge of minimal length, or,
// when several share the minimal length, the first of those with the largest
// quality.  Qualities are computed in FP64 only for the chosen edges (in one
// compacted pass) and for edges tied on length.
template <int D>
static void choose_rails_lazy_d(Mesh& m, const LO* c2e_p, LO n, const I8* codes_p,
                                const double* quals2_p, I8* vcand_p, double* vqual_p,
                                GO* vrail_p) {
  LO nv = m.nverts();
  constexpr int dim = D;
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  Arr<LO> e2c = fill<LO>(m.nedges(), -1);
  auto c2e = cview(c2e_p, n);
  {
    auto ec = view(e2c);
    pfor(n, [=] __device__(LO i) { ec[c2e[i]] = i; });
  }
  const Adj& v2e = m.ask_up(0, 1);
  auto va = cview(v2e.a2ab);
  auto vb = cview(v2e.ab2b);
  auto vc = cview(v2e.codes);
  auto ev = cview(m.ask_verts_of(1));
  auto cv = cview(m.ask_verts_of(dim));
  const Adj& v2t = m.ask_up(0, dim);
  auto ta = cview(v2t.a2ab);
  auto tb = cview(v2t.ab2b);
  auto tc = cview(v2t.codes);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto len = cview(m.ask_lengths());
  auto ec = cview(e2c);
  auto codes = cview(codes_p, n);
  auto quals2 = cview(quals2_p, n * 2);
  auto vcand = view(vcand_p, nv);
  auto vqual = view(vqual_p, nv);
  auto vrail = view(vrail_p, nv);
  Arr<LO> vonto(nv);
  Arr<I8> needm(nv);
  auto von = view(vonto);
  auto nm = view(needm);
  unsigned long long* cnt = ctx().d_screen_counts;
  pfor(nv, [=] __device__(LO v) {
    unsigned nexact = 0;
    // the shortest length and how many eligible edges have it
    double best_l = 0;
    int ntie = 0;
    LO first = -1;
    for (LO x = va[v]; x < va[v + 1]; ++x) {
      LO e = vb[x];
      LO cand = ec[e];
      if (cand == -1) continue;
      if (!collapses(codes[cand], code_which_down(vc[x]))) continue;
      double l = len[e];
      if (first == -1 || l < best_l) {
        first = x;
        best_l = l;
        ntie = 1;
      } else if (l == best_l) {
        ++ntie;
      }
    }
    von[v] = -1;
    nm[v] = 0;
    if (first == -1) {
      vcand[v] = 0;
      vqual[v] = -1.0;
      vrail[v] = -1;
      return;
    }
    LO chosen = -1;
    double best_q = -1;
    if (ntie == 1) {
      LO e = vb[first];
      int eev = code_which_down(vc[first]);
      chosen = e;
      best_q = quals2[ec[e] * 2 + eev];
      if (best_q != best_q) {  // computed below
        von[v] = ev[e * 2 + (1 - eev)];
        nm[v] = 1;
      }
    } else {
      for (LO x = first; x < va[v + 1]; ++x) {
        LO e = vb[x];
        LO cand = ec[e];
        if (cand == -1) continue;
        int eev = code_which_down(vc[x]);
        if (!collapses(codes[cand], eev)) continue;
        if (!(len[e] == best_l)) continue;
        double q = quals2[cand * 2 + eev];
        if (q != q) q = collapse_min_exact<dim>(sv, c, mt, cv, ta, tb, tc, v, ev[e * 2 + (1 - eev)], &nexact);
        if (chosen == -1 || q > best_q) {
          chosen = e;
          best_q = q;
        }
      }
    }
    vcand[v] = 1;
    vqual[v] = best_q;
    vrail[v] = chosen;
    warp_count(&cnt[1], nexact);
  });
  // the FP64 quality of each chosen rail not known yet
  Arr<LO> need = collect_marked(needm);
  LO K = need.size();
  if (K == 0) return;
  Arr<LO> kv = need;
  Arr<LO> ko(K);
  {
    auto nd = cview(need);
    auto o = view(ko);
    auto vo = cview(vonto);
    pfor(K, [=] __device__(LO k) { o[k] = vo[nd[k]]; });
  }
  Arr<double> kq(K);
  collapse_minima_exact(m, sv, kv, ko, kq.data());
  {
    auto nd = cview(need);
    auto q = cview(kq);
    pfor(K, [=] __device__(LO k) { vqual[nd[k]] = q[k]; });
  }
}
static void choose_rails_lazy(Mesh& m, const LO* c2e_p, LO n, const I8* codes_p,
                              const double* quals2_p, I8* vcand_p, double* vqual_p, GO* vrail_p) {
  if (m.dim == 3)
    choose_rails_lazy_d<3>(m, c2e_p, n, codes_p, quals2_p, vcand_p, vqual_p, vrail_p);
  else
    choose_rails_lazy_d<2>(m, c2e_p, n, codes_p, quals2_p, vcand_p, vqual_p, vrail_p);
}

static void filter_cands(Arr<LO>& c2e, Arr<I8>& codes, Arr<double>* q2) {
  Arr<LO> keep = collect_marked(codes);
  c2e = unmap(keep, c2e, 1);
  codes = unmap(keep, codes, 1);
  if (q2) *q2 = unmap(keep, *q2, 2);
}

// The faces around a vertex v of a tet mesh, from v's tets: each tet holds v
// in one slot, and its three faces other than the one opposite that slot
// contain v.  Every face around v is found this way, once per tet that holds
// it (one or two).  For rows of up to 32 tets, lane l of a warp takes tet
// beg + l; the face ids go to F (-1 where there is none) and keep[] marks
// each face's first occurrence in (lane, slot) order.
__device__ __forceinline__ void faces_around_lane(LO v, LO beg, LO end, int lane, LV tb,
                                                  View<const I8> tc, LV tf, LO F[3],
                                                  bool keep[3]) {
  for (int i = 0; i < 3; ++i) F[i] = -1;
  LO x = beg + lane;
  if (x < end) {
    LO t = tb[x];
    int sv = code_which_down(tc[x]);
    int q = 0;
    for (int f = 0; f < 4; ++f) {
      bool has = false;
      for (int j = 0; j < 3; ++j) has = has || down_template(3, 2, f, j) == sv;
      if (has) F[q++] = tf[t * 4 + f];
    }
  }
  for (int i = 0; i < 3; ++i) keep[i] = F[i] >= 0;
  for (int src = 0; src < 32; ++src) {
    for (int j = 0; j < 3; ++j) {
      LO o = __shfl_sync(0xffffffffu, F[j], src);
      for (int i = 0; i < 3; ++i)
        if (o == F[i] && (src < lane || (src == lane && j < i))) keep[i] = false;
    }
  }
}

// coarsen_verts + coarsen (src/Omega_h_coarsen.cpp:29-176): collapse the
// marked vertices along their edges.  allowed: overshoot limit
// max_length_allowed instead of max_length_desired; improve: keep only
// directions whose cavity quality beats the worst element now at the
// collapsing vertex (filter_coarsen_improve,
// src/Omega_h_coarsen_qualities.cpp:111-122).
static bool coarsen_verts(Mesh& m, const AdaptOpts& o, const Arr<I8>& vm, bool allowed,
                          bool improve, PassStats* st) {
  int dim = m.dim;
  LO ne = m.nedges();
  Arr<I8> ecodes(ne);
  {
    auto ev = cview(m.ask_verts_of(1));
    auto v = cview(vm);
    auto ec = view(ecodes);
    pfor(ne, [=] __device__(LO e) { ec[e] = I8((v[ev[e * 2]] ? 1 : 0) | (v[ev[e * 2 + 1]] ? 2 : 0)); });
  }
  Arr<LO> c2e = collect_marked(ecodes);
  if (c2e.size() == 0) return false;
  Arr<I8> codes0 = unmap(c2e, ecodes, 1);
  Arr<I8> codes(c2e.size());
  check_collapse_class(m, c2e.data(), c2e.size(), codes0.data(), codes.data());
  // The exposure and overshoot checks run on the same list: a candidate
  // that failed the class check has code 0, which they pass through at
  // once, so one compaction after the three gives the list the reference
  // gets by compacting after each (src/Omega_h_coarsen.cpp:159-176).  Whether
  // any candidate passed the class check (the mesh is then ghosted) is read
  // with that compaction's count.
  Arr<int> any_class = fill<int>(1, 0);
  {
    auto cd = cview(codes);
    int* ac = any_class.data();
    pfor(c2e.size(), [=] __device__(LO i) {
      if (cd[i]) *ac = 1;
    });
  }
  Arr<I8> codes2(c2e.size());
  check_collapse_exposure(m, c2e.data(), c2e.size(), codes.data(), codes2.data());
  // with screening, prevent_coarsen_overshoot runs inside the quality
  // screen (it stages the same neighbours); otherwise here
  bool lazy = ctx().screening && !improve;
  double max_len = allowed ? o.max_length_allowed : o.max_length_desired;
  if (lazy)
    codes = codes2;
  else
    prevent_coarsen_overshoot(m, max_len, c2e.data(), c2e.size(), codes2.data(), codes.data());
  // With screening the list is not compacted here: the screen and
  // choose_rails_lazy pass over candidates with code 0, and whether any
  // candidate passed the class check is read with the keys' count below.
  int passed_class = 0;
  if (!lazy) {
    Arr<LO> keep = collect_marked(codes, any_class.data(), &passed_class);
    c2e = unmap(keep, c2e, 1);
    codes = unmap(keep, codes, 1);
    if (passed_class) m.parting = 1;  // ghosted once candidates pass the class check
    if (c2e.size() == 0) return false;
  }
  LO nc = c2e.size();
  Arr<double> q2(nc * 2);
  if (lazy) {
    coarsen_filter_lazy(m, c2e.data(), nc, codes.data(), o.min_quality_allowed, q2.data(),
                        max_len);
  } else {
    coarsen_qualities(m, c2e.data(), nc, codes.data(), q2.data());
    // the worst element quality at each vertex now (graph_reduce MIN)
    Arr<double> vold;
    if (improve) {
      const Adj& v2c = m.ask_up(0, dim);
      auto va = cview(v2c.a2ab);
      auto vb = cview(v2c.ab2b);
      auto eq = cview(m.ask_qualities());
      vold = Arr<double>(m.nverts());
      auto vo = view(vold);
      pfor(m.nverts(), [=] __device__(LO v) {
        double mq = DBL_MAX;
        for (LO x = va[v]; x < va[v + 1]; ++x) mq = min2d(mq, eq[vb[x]]);
        vo[v] = mq;
      });
    }
    auto cd = view(codes);
    auto q = cview(q2);
    auto ce = cview(c2e);
    auto ev = cview(m.ask_verts_of(1));
    auto vo = cview(vold);
    double mqa = o.min_quality_allowed;
    pfor(nc, [=] __device__(LO i) {
      I8 code = cd[i];
      for (int d = 0; d < 2; ++d) {
        if (!(q[i * 2 + d] >= mqa)) code = dont_collapse(code, d);
        if (improve && !(q[i * 2 + d] > vo[ev[ce[i] * 2 + d]])) code = dont_collapse(code, d);
      }
      cd[i] = code;
    });
  }
  // choose_rails_lazy skips candidates whose directions all failed (code
  // 0), so with screening the list is not compacted here (no host wait); a
  // pass where none survives then finds no key below
  if (!lazy) {
    filter_cands(c2e, codes, &q2);
    if (c2e.size() == 0) return false;
  }
  LO nv = m.nverts();
  Arr<I8> vc(nv);
  Arr<double> vq(nv);
  Arr<GO> vr(nv);
  if (lazy)
    choose_rails_lazy(m, c2e.data(), c2e.size(), codes.data(), q2.data(), vc.data(), vq.data(),
                      vr.data());
  else
    choose_rails(m, c2e.data(), c2e.size(), codes.data(), q2.data(), vc.data(), vq.data(),
                 vr.data());
  Arr<I8> vkeys = find_indset(m, VERT, vq, vc);
  Arr<LO> k2v = lazy ? collect_marked(vkeys, any_class.data(), &passed_class)
                     : collect_marked(vkeys);
  if (lazy && passed_class) m.parting = 1;
  LO nkeys = k2v.size();
  if (nkeys == 0) return false;  // no candidate survived (the set of any is not empty)
  st->coarsen_keys = nkeys;
  // find_rails (src/Omega_h_collapse_rail.cpp:79-108) and the vertices onto
  Arr<LO> r2e(nkeys);
  Arr<I8> rdir(nkeys);
  Arr<LO> k2onto(nkeys);
  {
    const Adj& v2e = m.ask_up(0, 1);
    auto va = cview(v2e.a2ab);
    auto vb = cview(v2e.ab2b);
    auto vcd = cview(v2e.codes);
    auto kv = cview(k2v);
    auto rail = cview(vr);
    auto ev = cview(m.ask_verts_of(1));
    auto re = view(r2e);
    auto rd = view(rdir);
    auto ko = view(k2onto);
    int* stw = ctx().d_status;
    pfor(nkeys, [=] __device__(LO k) {
      LO v = kv[k];
      LO fe = -1;
      I8 fd = 0;
      for (LO x = va[v]; x < va[v + 1]; ++x)
        if (GO(vb[x]) == rail[v]) {
          fe = vb[x];
          fd = I8(code_which_down(vcd[x]));
          break;
        }
      if (fe < 0) {
        raise_status(stw, ST_TOPOLOGY);
        fe = 0;
        fd = 0;
      }
      re[k] = fe;
      rd[k] = fd;
      ko[k] = ev[fe * 2 + (1 - fd)];
    });
  }
  // mark_dead_ents (src/Omega_h_coarsen_topology.cpp:28-70)
  Arr<I8> dead[4];
  dead[1] = mark_image(r2e, ne);
  for (int d = 2; d <= dim; ++d) dead[d] = fill<I8>(m.nents[d], 0);
  if (dim == 3) {
    // both steps in one walk of the rail's tets: each tet dies with its face
    // opposite onto; of the two faces holding the rail, {col, onto, w}, each
    // dies with its side opposite onto, the tet edge {col, w}
    const Adj& e2t = m.ask_up_any_order(EDGE, REGION);
    auto ea = cview(e2t.a2ab);
    auto eb = cview(e2t.ab2b);
    auto ecc = cview(e2t.codes);
    auto tf = cview(m.ask_down(REGION, FACE).ab2b);
    auto te = cview(m.ask_down(REGION, EDGE).ab2b);
    auto re = cview(r2e);
    auto rd = cview(rdir);
    auto d3 = view(dead[3]);
    auto d2 = view(dead[2]);
    auto d1 = view(dead[1]);
    unsigned long long lut = tet_edge_lookup();
    pfor(nkeys, [=] __device__(LO r) {
      LO e = re[r];
      int onto = 1 - rd[r];
      for (LO x = ea[e]; x < ea[e + 1]; ++x) {
        LO t = eb[x];
        int cce = code_which_down(ecc[x]), rot = code_rotation(ecc[x]);
        int lo = down_template(3, 1, cce, rot ^ onto);
        int lc = down_template(3, 1, cce, rot ^ (1 - onto));
        d3[t] = 1;
        d2[tf[t * 4 + opposite_template(3, 0, lo)]] = 1;
        for (int w = 0; w < 4; ++w) {
          if (w == lo || w == lc) continue;
          d2[tf[t * 4 + opposite_template(3, 0, 6 - lo - lc - w)]] = 1;
          d1[te[t * 6 + tet_edge_between(lut, lc, w)]] = 1;
        }
      }
    });
  }
  for (int cd = dim; cd > EDGE && dim != 3; --cd) {
    const Adj& e2c = m.ask_up_any_order(1, cd);  // marks only: row order is free
    auto ea = cview(e2c.a2ab);
    auto eb = cview(e2c.ab2b);
    auto ecc = cview(e2c.codes);
    auto cs = cview(m.ask_down(cd, cd - 1).ab2b);
    int nccs = simplex_degree(cd, cd - 1);
    auto re = cview(r2e);
    auto rd = cview(rdir);
    auto dc = view(dead[cd]);
    auto ds = view(dead[cd - 1]);
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
  nm.rebuilt = true;  // element-based partitioning after a rebuild
  nm.metric_comps = m.metric_comps;
  nm.class_sets = m.class_sets;
  Arr<LO> ov2nv, old_lows2new;
  // find_coarsen_domains: live d-entities around each key vertex, for every
  // dimension, and every dimension's modify plan, before one host wait for
  // all their sizes
  Arr<LO> k2ps[4];
  ModifyPlan plans[4];
  k2ps[0] = fill<LO>(nkeys + 1, 0);
  // In 3D the faces around a key vertex come from its tets (faces_around_lane)
  // when the vertex-to-face rows are not built: their ascending order is the
  // sorted row's, without inverting and sorting the face-to-vertex lists.
  bool faces_by_tets = dim == 3 && !m.adj.count({VERT, FACE});
  // per key with at most 32 tets, its live faces in ascending order (at
  // most 96), found by the count below and copied out by the fill
  constexpr int kFaceLoc = 96;
  Arr<LO> face_loc(faces_by_tets ? nkeys * kFaceLoc : 0);
  for (int d = 1; d <= dim; ++d) {
    auto dd = cview(dead[d]);
    auto kv = cview(k2v);
    Arr<LO> cnt(nkeys);
    auto ct = view(cnt);
    if (d == FACE && faces_by_tets) {
      const Adj& v2t = m.ask_up(0, 3);
      auto ta = cview(v2t.a2ab);
      auto tb = cview(v2t.ab2b);
      auto tc = cview(v2t.codes);
      auto tf = cview(m.ask_down(3, 2).ab2b);
      auto fl = view(face_loc);
      group_for(32, nkeys, kBlock, [=] __device__(LO k, int gl, unsigned gm) {
        if (k < 0) return;
        LO v = kv[k], beg = ta[v], end = ta[v + 1];
        LO n2 = 0;
        if (end - beg <= 32) {
          LO F[3];
          bool keep[3];
          faces_around_lane(v, beg, end, gl, tb, tc, tf, F, keep);
          // the live faces kept here (-1: none), each placed at its rank
          // among the live faces (the sorted row's order)
          LO L[3];
          for (int i = 0; i < 3; ++i) L[i] = keep[i] && !dd[F[i]] ? F[i] : -1;
          LO rank[3] = {0, 0, 0};
          for (int src = 0; src < 32; ++src)
            for (int j = 0; j < 3; ++j) {
              LO o = __shfl_sync(0xffffffffu, L[j], src);
              for (int i = 0; i < 3; ++i) rank[i] += o >= 0 && o < L[i];
            }
          for (int i = 0; i < 3; ++i) {
            if (L[i] < 0) continue;
            fl[k * kFaceLoc + rank[i]] = L[i];
            ++n2;
          }
          n2 = LO(__reduce_add_sync(gm, unsigned(n2)));
        } else if (gl == 0) {
          // a long row: one lane, each face counted at its first occurrence
          for (LO x = beg; x < end; ++x) {
            LO t = tb[x];
            int sv = code_which_down(tc[x]);
            for (int f = 0; f < 4; ++f) {
              bool has = false;
              for (int j = 0; j < 3; ++j) has = has || down_template(3, 2, f, j) == sv;
              if (!has) continue;
              LO F = tf[t * 4 + f];
              bool first = true;
              for (LO y = beg; y < x && first; ++y)
                for (int g = 0; g < 4; ++g)
                  if (tf[tb[y] * 4 + g] == F) first = false;
              n2 += first && !dd[F];
            }
          }
        }
        if (gl == 0) ct[k] = n2;
      });
    } else {
      const Adj& v2d = m.ask_up(0, d);
      auto va = cview(v2d.a2ab);
      auto vb = cview(v2d.ab2b);
      // one warp per key: the lanes stride the key vertex's row (rows of
      // tens of entries, which one thread would walk alone)
      group_for(32, nkeys, kBlock, [=] __device__(LO k, int gl, unsigned gm) {
        if (k < 0) return;
        LO v = kv[k], n2 = 0;
        for (LO x = va[v] + gl; x < va[v + 1]; x += 32) n2 += !dd[vb[x]];
        n2 = LO(__reduce_add_sync(gm, unsigned(n2)));
        if (gl == 0) ct[k] = n2;
      });
    }
    k2ps[d] = offset_scan(cnt);
  }
  {
    std::vector<ModifyPlan*> pls;
    std::vector<const Arr<LO>*> kps;
    Arr<I8> key_marks = mark_image(k2v, m.nverts());
    for (int d = 0; d <= dim; ++d) {
      plans[d] = plan_modify(m, d, VERT, k2v, k2ps[d], &key_marks);
      pls.push_back(&plans[d]);
      kps.push_back(&k2ps[d]);
    }
    plan_sizes(pls, kps);
  }
  for (int d = 0; d <= dim; ++d) {
    const Arr<LO>& k2p = k2ps[d];
    Arr<LO> pv2v, kd2d;
    if (d == FACE && faces_by_tets) {
      const Adj& v2t = m.ask_up(0, 3);
      auto ta = cview(v2t.a2ab);
      auto tb = cview(v2t.ab2b);
      auto tc = cview(v2t.codes);
      auto tf = cview(m.ask_down(3, 2).ab2b);
      auto dd = cview(dead[d]);
      auto kv = cview(k2v);
      LO nprod = plans[d].sizes[2];
      kd2d = Arr<LO>(nprod);
      pv2v = Arr<LO>(nprod * 3);
      auto kp = cview(k2p);
      auto cv = cview(m.ask_verts_of(2));
      auto ko = cview(k2onto);
      auto o2n = cview(ov2nv);
      auto kd = view(kd2d);
      auto pv = view(pv2v);
      auto fl = cview(face_loc);
      // the live faces in ascending order (the sorted row's order): each
      // one's rank among the live faces gives its product slot
      group_for(32, nkeys, kBlock, [=] __device__(LO k, int gl, unsigned gm) {
        if (k < 0) return;
        LO v = kv[k], beg = ta[v], end = ta[v + 1], p = kp[k];
        auto put = [&](LO q, LO F) {
          kd[q] = F;
          for (int ccv = 0; ccv < 3; ++ccv) {
            LO fv = cv[F * 3 + ccv];
            pv[q * 3 + ccv] = o2n[fv == v ? ko[k] : fv];
          }
        };
        if (end - beg <= 32) {
          // the count placed them in order
          LO nf = kp[k + 1] - p;
          for (LO r = gl; r < nf; r += 32) put(p + r, fl[k * kFaceLoc + r]);
        } else if (gl == 0) {
          // a long row: one lane; a face's slot is the number of live first
          // occurrences with a smaller id
          for (LO x = beg; x < end; ++x) {
            LO t = tb[x];
            int sv = code_which_down(tc[x]);
            for (int f = 0; f < 4; ++f) {
              bool has = false;
              for (int j = 0; j < 3; ++j) has = has || down_template(3, 2, f, j) == sv;
              if (!has) continue;
              LO F = tf[t * 4 + f];
              bool first = true;
              for (LO y = beg; y < x && first; ++y)
                for (int g = 0; g < 4; ++g)
                  if (tf[tb[y] * 4 + g] == F) first = false;
              if (!first || dd[F]) continue;
              LO r = 0;
              for (LO y = beg; y < end; ++y) {
                int sy = code_which_down(tc[y]);
                for (int g = 0; g < 4; ++g) {
                  bool hg = false;
                  for (int j = 0; j < 3; ++j) hg = hg || down_template(3, 2, g, j) == sy;
                  if (!hg) continue;
                  LO G = tf[tb[y] * 4 + g];
                  if (G >= F || dd[G]) continue;
                  bool gfirst = true;
                  for (LO z = beg; z < y && gfirst; ++z)
                    for (int h = 0; h < 4; ++h)
                      if (tf[tb[z] * 4 + h] == G) gfirst = false;
                  r += gfirst;
                }
              }
              put(p + r, F);
            }
          }
        }
      });
    } else if (d != VERT) {
      const Adj& v2d = m.ask_up(0, d);
      auto va = cview(v2d.a2ab);
      auto vb = cview(v2d.ab2b);
      auto vcd = cview(v2d.codes);
      auto dd = cview(dead[d]);
      auto kv = cview(k2v);
      LO nprod = plans[d].sizes[2];
      kd2d = Arr<LO>(nprod);
      int nccv = d + 1;
      pv2v = Arr<LO>(nprod * nccv);
      auto kp = cview(k2p);
      auto cv = cview(m.ask_verts_of(d));
      auto ko = cview(k2onto);
      auto o2n = cview(ov2nv);
      auto kd = view(kd2d);
      auto pv = view(pv2v);
      // the live entries in row order, ranked within each 32-entry step
      // by a ballot: the positions a walk of the row would give them
      group_for(32, nkeys, kBlock, [=] __device__(LO k, int gl, unsigned gm) {
        if (k < 0) return;
        LO v = kv[k], p = kp[k], beg = va[v], end = va[v + 1];
        for (LO x0 = beg; x0 < end; x0 += 32) {
          LO x = x0 + gl;
          LO el = 0;
          bool live = false;
          if (x < end) {
            el = vb[x];
            live = !dd[el];
          }
          unsigned lm = __ballot_sync(gm, live);
          if (live) {
            LO q = p + LO(__popc(lm & ((1u << gl) - 1u)));
            int ccv_col = code_which_down(vcd[x]);
            kd[q] = el;
            for (int ccv = 0; ccv < nccv; ++ccv) {
              LO ov = ccv == ccv_col ? ko[k] : cv[el * nccv + ccv];
              pv[q * nccv + ccv] = o2n[ov];
            }
          }
          p += LO(__popc(lm));
        }
      });
    }
    ModifyOut mo = apply_modify(m, nm, d, VERT, plans[d], k2v, k2p, pv2v, old_lows2new);
    LO nnew = nm.nents[d];
    if (d == VERT) ov2nv = mo.old2new;
    xfer_class(m, nm, d, mo, nnew, nullptr, nullptr, kd2d.data());
    if (d == VERT) {
      nm.coords = xfer(m.coords, mo, nnew, Arr<double>(), dim);
      nm.metric = xfer(m.metric, mo, nnew, Arr<double>(), m.mcomp());
    }
    xfer_lengths_qualities(m, nm, d, mo, &pv2v);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
  return true;
}

// coarsen_by_size (src/Omega_h_coarsen.cpp:198-208): vertices of edges
// shorter than min_length_desired
bool coarsen_by_size(Mesh& m, const AdaptOpts& o, PassStats* st) {
  const Arr<double>& len = m.ask_lengths();
  LO ne = m.nedges();
  Arr<I8> ecand(ne);
  {
    auto l = cview(len);
    auto c = view(ecand);
    double mn = o.min_length_desired;
    pfor(ne, [=] __device__(LO i) { c[i] = l[i] < mn; });
  }
  // no separate count: without candidates the candidate list below is empty
  return coarsen_verts(m, o, mark_down(m, EDGE, VERT, ecand), false, false, st);
}

// coarsen_slivers (src/Omega_h_coarsen.cpp:210-220): vertices of the sliver
// layers, overshoot up to max_length_allowed, local improvement required
bool coarsen_slivers(Mesh& m, const AdaptOpts& o, PassStats* st) {
  m.parting = 1;  // src/Omega_h_coarsen.cpp:212
  Arr<I8> ec = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  return coarsen_verts(m, o, mark_down(m, m.dim, VERT, ec), true, true, st);
}

// ------------------------------------------------------------ swap (3D)
// Edge-swap triangulation tables in device memory: a header of 9 ints per
// loop size n = 0..7 (meshes, triangles per mesh, unique triangles, edges
// per mesh, unique edges, then the offsets of the four tables), followed by
// the flat table of ohg_swap3d_tables.inc.
enum { SW_NMESH, SW_NTRI, SW_NUTRI, SW_NEDGE, SW_NUEDGE, SW_OTRI, SW_OMESH, SW_OUEDGE, SW_OE2U };
constexpr int kSwapHdr = 8 * 9;
constexpr int kMaxUniqTris = 35, kMaxUniqEdges = 26;

// the largest product counts of one key over the 3..7-gons: edges,
// triangles and tets (npe, npt + 2 npe, 2 npt)
static void swap3d_max_products(int out[4]) {
  out[0] = 0;
  out[1] = out[2] = out[3] = 0;
  int p = 0;
  while (p < OHG_SWAP3D_TABLE_LEN) {
    int nm = OHG_SWAP3D_TABLE[p + 1], nt = OHG_SWAP3D_TABLE[p + 2],
        nu = OHG_SWAP3D_TABLE[p + 3];
    p += 4 + nu * 3 + nm * nt;
    int ne = OHG_SWAP3D_TABLE[p], nue = OHG_SWAP3D_TABLE[p + 1];
    p += 2 + nue * 2 + nm * ne;
    out[1] = std::max(out[1], ne);
    out[2] = std::max(out[2], nt + 2 * ne);
    out[3] = std::max(out[3], 2 * nt);
  }
}

static View<const int> swap_tables() {
  Ctx& c = ctx();
  if (!c.d_swap_tables) {
    std::vector<int> h(kSwapHdr + OHG_SWAP3D_TABLE_LEN, 0);
    int p = 0;
    while (p < OHG_SWAP3D_TABLE_LEN) {
      int n = OHG_SWAP3D_TABLE[p], nm = OHG_SWAP3D_TABLE[p + 1], nt = OHG_SWAP3D_TABLE[p + 2],
          nu = OHG_SWAP3D_TABLE[p + 3];
      int* hd = &h[n * 9];
      p += 4;
      hd[SW_NMESH] = nm;
      hd[SW_NTRI] = nt;
      hd[SW_NUTRI] = nu;
      hd[SW_OTRI] = kSwapHdr + p;
      p += nu * 3;
      hd[SW_OMESH] = kSwapHdr + p;
      p += nm * nt;
      int ne = OHG_SWAP3D_TABLE[p], nue = OHG_SWAP3D_TABLE[p + 1];
      p += 2;
      hd[SW_NEDGE] = ne;
      hd[SW_NUEDGE] = nue;
      hd[SW_OUEDGE] = kSwapHdr + p;
      p += nue * 2;
      hd[SW_OE2U] = kSwapHdr + p;
      p += nm * ne;
    }
    for (int i = 0; i < OHG_SWAP3D_TABLE_LEN; ++i) h[kSwapHdr + i] = OHG_SWAP3D_TABLE[i];
    OHG_CUDA(cudaMalloc(&c.d_swap_tables, h.size() * sizeof(int)));
    OHG_CUDA(cudaMemcpy(c.d_swap_tables, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
    c.swap_tables_len = int(h.size());
  }
  return {c.d_swap_tables, c.swap_tables_len};
}

// swap3d::find_loop (src/Omega_h_swap3d_loop.hpp:24-78): the ring of tets
// around each edge, loop vertices ordered to curl around it.  One thread per
// edge; ring sizes outside 3..7 are reported as size 0.
static void swap_loops(Mesh& m, const LO* edges_p, LO n, Arr<int>& lsize, Arr<LO>& lverts,
                       Arr<LO>& leev) {
  const Adj& e2t = m.ask_up(1, 3);
  auto ea = cview(e2t.a2ab);
  auto eb = cview(e2t.ab2b);
  auto ec = cview(e2t.codes);
  auto ev = cview(m.ask_verts_of(1));
  auto tv = cview(m.ask_verts_of(3));
  auto edges = cview(edges_p, n);
  lsize = Arr<int>(n);
  lverts = Arr<LO>(n * 7);
  leev = Arr<LO>(n * 2);
  auto ls = view(lsize);
  auto lv = view(lverts);
  auto le = view(leev);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    LO edge = edges[i];
    LO b = ea[edge];
    int size = ea[edge + 1] - b;
    le[i * 2] = ev[edge * 2];
    le[i * 2 + 1] = ev[edge * 2 + 1];
    for (int k = 0; k < 7; ++k) lv[i * 7 + k] = 0;
    if (size < 3 || size > 7) {
      ls[i] = 0;
      return;
    }
    LO t0[7], t1[7];
    for (int k = 0; k < size; ++k) {
      LO tet = eb[b + k];
      I8 code = ec[b + k];
      int opp = opposite_template(3, 1, code_which_down(code) & 7);
      int rot = code_rotation(code);
      t0[k] = tv[tet * 4 + down_template(3, 1, opp, rot ^ 0)];
      t1[k] = tv[tet * 4 + down_template(3, 1, opp, rot ^ 1)];
    }
    for (int a = 0; a < size - 1; ++a) {
      int j = a + 1;
      while (j < size && t0[j] != t1[a]) ++j;
      if (j >= size) {
        raise_status(st, ST_TOPOLOGY);
        ls[i] = 0;
        return;
      }
      LO x0 = t0[a + 1], x1 = t1[a + 1];
      t0[a + 1] = t0[j];
      t1[a + 1] = t1[j];
      t0[j] = x0;
      t1[j] = x1;
    }
    for (int k = 0; k < size; ++k) lv[i * 7 + k] = t0[k];
    ls[i] = size;
  });
}

// device bytes held by a mesh: every array it references (stored and
// derived adjacencies, fields, cached lengths and qualities, screening data),
// each buffer counted once (the parts of a split union share buffers)
std::size_t mesh_device_bytes(const Mesh& m) {
  std::set<const Buf*> seen;
  std::size_t total = 0;
  auto add = [&](const std::shared_ptr<Buf>& b) {
    if (b && seen.insert(b.get()).second) total += b->bytes;
  };
  add(m.coords.buf);
  add(m.metric.buf);
  add(m.length.buf);
  add(m.quality.buf);
  for (int d = 0; d < 4; ++d) {
    add(m.class_dim[d].buf);
    add(m.class_id[d].buf);
  }
  for (const auto* cache : {&m.adj, &m.adj_any_order})
    for (const auto& kv : *cache) {
      add(kv.second.a2ab.buf);
      add(kv.second.ab2b.buf);
      add(kv.second.codes.buf);
    }
  for (const auto& t : m.extra_tags) add(t.bytes.buf);
  if (m.screen) {
    add(m.screen->xh.buf);
    add(m.screen->xl.buf);
    add(m.screen->ma.buf);
    add(m.screen->mb.buf);
    add(m.screen->dkey.buf);
    add(m.screen->sdet.buf);
  }
  return total;
}

void swap3d_find_loops(Mesh& m, const LO* edges, LO n, int* sizes, LO* eev2v, LO* loop_verts) {
  if (m.dim != 3) throw Error(8, "swap3d loops: the mesh is not 3D");
  if (n == 0) return;
  Arr<int> lsize;
  Arr<LO> lverts, leev;
  swap_loops(m, edges, n, lsize, lverts, leev);
  Ctx& c = ctx();
  OHG_CUDA(cudaMemcpyAsync(sizes, lsize.data(), size_t(n) * sizeof(int), cudaMemcpyDeviceToDevice,
                           c.stream));
  OHG_CUDA(cudaMemcpyAsync(eev2v, leev.data(), size_t(n) * 2 * sizeof(LO),
                           cudaMemcpyDeviceToDevice, c.stream));
  OHG_CUDA(cudaMemcpyAsync(loop_verts, lverts.data(), size_t(n) * 7 * sizeof(LO),
                           cudaMemcpyDeviceToDevice, c.stream));
}

// swap3d_qualities + swap3d::choose (src/Omega_h_swap3d_qualities.cpp:10-58,
// src/Omega_h_swap3d_choice.hpp:15-100).  The reference evaluates unique
// triangles and edges lazily per candidate; here every unique triangle's two
// tets and every unique edge length are evaluated by their own threads into
// global memory, then one thread per candidate walks the triangulations in
// table order with the reference's comparisons (first best wins, a negative
// triangle ends a triangulation, an edge longer than max_length_allowed
// rejects it).  The values are pure functions of the loop, so the choice is
// the same.
// swap3d_qualities with FP32 screening.  The reference picks, in table
// order, the first triangulation with the largest min quality among those
// whose new edges are all within max_len, provided that quality is > 0.  That
// is order independent apart from ties, so it is computed from enclosures:
//  1. every unique triangle gets an enclosure of its FP64 quality (min of 1
//     and its two tets), every unique edge an exact "longer than max_len"
//     flag (screened, FP64 where the threshold is inside the enclosure);
//  2. L* = the largest lower bound of a valid triangulation; only valid
//     triangulations with upper bound >= L* and > 0 can hold the maximum,
//     and in each only triangles with lower bound <= its upper bound can
//     hold its minimum: those triangles are evaluated in FP64;
//  3. the FP64 minima of those triangulations give the reference's choice
//     and quality, the first one winning ties.
// improving_only (the pass): a candidate whose best triangulation's upper
// bound is below the worst current quality around its edge cannot pass
// filter_swap_improve; it gets quality -DBL_MAX and no FP64 work.
static void swap3d_qualities_screened(Mesh& m, double max_len, const LO* c2e_p, LO n,
                                      double* quals_p, I8* configs_p,
                                      bool improving_only = false) {
  int mc = m.mcomp();  // metric components per vertex (1: isotropic)
  auto tab = swap_tables();
  Arr<int> lsize;
  Arr<LO> lverts, leev;
  swap_loops(m, c2e_p, n, lsize, lverts, leev);
  const VertScreen& vs = mesh_screen(m);
  auto sv = screen_view(vs);
  auto ls = cview(lsize);
  auto lv = cview(lverts);
  auto le = cview(leev);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  unsigned long long* cnt = ctx().d_screen_counts;
  Arr<float2> tbnd(n * kMaxUniqTris);
  Arr<I8> over(n * kMaxUniqEdges);
  Arr<unsigned long long> need(n);
  Arr<float> lstar(n);
  Arr<double> tq(n * kMaxUniqTris);
  // The (candidate, unique triangle) and (candidate, unique edge) items of
  // all loops, numbered consecutively: loops of 4 to 6 edges use 4 to 20 of
  // the 35 triangle slots, so a grid over the slots would leave most lanes
  // idle.  titem/eitem map an item back to its candidate; the slots past
  // the last item (the grid still spans n times the table maximum) return.
  Arr<LO> tioff, eioff, titem(n * kMaxUniqTris), eitem(n * kMaxUniqEdges);
  {
    Arr<LO> tcnt(n), ecnt(n);
    auto tc = view(tcnt);
    auto ec = view(ecnt);
    pfor(n, [=] __device__(LO i) {
      int size = ls[i];
      tc[i] = size >= 3 ? tab[size * 9 + SW_NUTRI] : 0;
      ec[i] = size >= 3 ? tab[size * 9 + SW_NUEDGE] : 0;
    });
    tioff = offset_scan(tcnt);
    eioff = offset_scan(ecnt);
    auto to = cview(tioff);
    auto eo = cview(eioff);
    auto ti = view(titem);
    auto ei = view(eitem);
    pfor(n, [=] __device__(LO i) {
      for (LO k = to[i]; k < to[i + 1]; ++k) ti[k] = i;
      for (LO k = eo[i]; k < eo[i + 1]; ++k) ei[k] = i;
    });
  }
  auto to = cview(tioff);
  auto eo = cview(eioff);
  auto ti = cview(titem);
  auto ei = cview(eitem);
  {
    auto tb = view(tbnd);
    // the items up to their count on the device, in a grid of resident size
    pfor_dev_count(tioff.data() + n, n * kMaxUniqTris, [=] __device__(LO item) {
      LO i = ti[item];
      if (i < 0 || i >= n) return;  // unwritten only after a scan tile gave up its wait
      int u = int(item - to[i]);
      LO idx = i * kMaxUniqTris + u;
      int size = ls[i];
      unsigned ns = 0;
      {
        // the triangle's two tets (t0, t1, t2, end 1) and (t0, t2, t1, end 0)
        // share the face opposite slot 3: its invariants once, the second
        // tet's normal the first's negated (its face edges in swapped order);
        // the bounds are of the cube of the quality, a monotone scale for
        // every comparison below
        int otri = tab[size * 9 + SW_OTRI];
        LO f[3];
        for (int k = 0; k < 3; ++k) f[k] = lv[i * 7 + tab[otri + u * 3 + k]];
        float4 hf[3] = {sv.xh[f[0]], sv.xh[f[1]], sv.xh[f[2]]};
        float4 lf[3] = {sv.xl[f[0]], sv.xl[f[1]], sv.xl[f[2]]};
        long long k0 = sv.dkey[f[0]], k1 = sv.dkey[f[1]], k2 = sv.dkey[f[2]];
        TetFaceInv inv = tet_face_invariants(hf, lf, 3);
        float lo = 1.0f, hi = 1.0f;
        for (int tt = 0; tt < 2; ++tt) {
          LO pv = le[i * 2 + (1 - tt)];
          // maxdet in slot order: (f0, f1, f2, p) or (f0, f2, f1, p)
          LO sa = f[0], sb = tt == 0 ? f[1] : f[2], sc = tt == 0 ? f[2] : f[1];
          long long ka = k0, kb = tt == 0 ? k1 : k2, kc = tt == 0 ? k2 : k1, kp = sv.dkey[pv];
          LO best = sa;
          long long bk = ka;
          if (kb > bk) {
            best = sb;
            bk = kb;
          }
          if (kc > bk) {
            best = sc;
            bk = kc;
          }
          if (kp > bk) best = pv;
          FIv b;
          if (tt == 0) {
            b = tet_face_bounds<true>(inv, hf, lf, sv.xh[pv], sv.xl[pv], sv.ma[best],
                                      sv.mb[best]);
          } else {
            TetFaceInv neg = inv;
            neg.a.x = -inv.a.x;
            neg.a.y = -inv.a.y;
            neg.a.z = -inv.a.z;
            float4 hs[3] = {hf[0], hf[2], hf[1]}, ls2[3] = {lf[0], lf[2], lf[1]};
            b = tet_face_bounds<true>(neg, hs, ls2, sv.xh[pv], sv.xl[pv], sv.ma[best],
                                      sv.mb[best]);
          }
          lo = fminf(lo, b.lo);
          hi = fminf(hi, b.hi);
        }
        tb[idx] = make_float2(lo, hi);
        ns = 2;
      }
      warp_count(&cnt[0], ns);
    });
  }
  {
    auto ov = view(over);
    float thr = float_at_or_below(max_len);  // for float x: x > max_len <=> x > thr
    // floats t_dn <= max_len < t_up for the end-length cut (strict above)
    float tup = float_at_or_above(max_len);
    if (double(tup) == max_len) tup = std::nextafter(tup, INFINITY);
    pfor_dev_count(eioff.data() + n, n * kMaxUniqEdges, [=] __device__(LO item) {
      LO i = ei[item];
      if (i < 0 || i >= n) return;  // unwritten only after a scan tile gave up its wait
      int u = int(item - eo[i]);
      LO idx = i * kMaxUniqEdges + u;
      int size = ls[i];
      unsigned ns = 0, nx = 0;
      {
        int oued = tab[size * 9 + SW_OUEDGE];
        LO a = lv[i * 7 + tab[oued + u * 2]], b = lv[i * 7 + tab[oued + u * 2 + 1]];
        float qlo[2], qhi[2];
        bool qok = edge_q_bounds3(sv, a, b, qlo, qhi);
        int side = len_cut_side(qlo, qhi, qok, len_cut(thr, tup));
        bool o;
        if (side != 0) {
          o = side > 0;
        } else {
          FIv L = qok ? len_from_q(qlo, qhi) : widen_all();
          if (L.lo > thr) {
            o = true;
          } else if (L.hi <= thr) {
            o = false;
          } else {
            o = edge_len_v(3, c, mt, mc, a, b) > max_len;
            nx = 1;
          }
        }
        ov[idx] = o;
        ns = 1;
      }
      warp_count(&cnt[2], ns);
      warp_count(&cnt[3], nx);
    });
  }
  auto tb = cview(tbnd);
  auto ov = cview(over);
  // the cube of the worst current quality around each candidate edge,
  // rounded down (improving_only)
  Arr<float> old3;
  if (improving_only) {
    old3 = Arr<float>(n);
    auto o3 = view(old3);
    auto eq = cview(m.ask_qualities());
    const Adj& e2t = m.ask_up_any_order(1, 3);  // a minimum: row order is free
    auto ea = cview(e2t.a2ab);
    auto eb = cview(e2t.ab2b);
    auto ce = cview(c2e_p, n);
    pfor(n, [=] __device__(LO i) {
      LO e = ce[i];
      double old = DBL_MAX;
      for (LO x = ea[e]; x < ea[e + 1]; ++x) old = min2d(old, eq[eb[x]]);
      // largest float at or below old, then its cube rounded down: for a
      // negative old the cube is negative and no candidate is skipped
      float f = float(old);
      if (double(f) > old) f = nextafterf(f, -INFINITY);
      float c3 = f > 0.0f ? __fmul_rd(__fmul_rd(f, f), f) : -INFINITY;
      o3[i] = old >= DBL_MAX ? -INFINITY : c3;
    });
  }
  auto o3 = cview(old3);
  bool improving = improving_only;
  {
    auto nd = view(need);
    auto lst = view(lstar);
    // 8 lanes per candidate over its triangulations; the floats are combined
    // by max, min and or, which do not depend on the order (the bounds are
    // only compared, so the sign of a zero does not matter)
    constexpr int G = 8;
    group_for(G, n, kBlock, [=] __device__(LO i, int gl, unsigned gm) {
      if (i < 0) return;
      int size = ls[i];
      if (size < 3) {
        if (gl == 0) {
          nd[i] = 0;
          lst[i] = INFINITY;
        }
        return;
      }
      const int* h = &tab[size * 9];
      int nmeshes = h[SW_NMESH], ntris = h[SW_NTRI], nedges = h[SW_NEDGE];
      int omsh = h[SW_OMESH], oe2u = h[SW_OE2U];
      float L = -INFINITY;
      for (int mesh = gl; mesh < nmeshes; mesh += G) {
        bool valid = true;
        for (int e = 0; e < nedges; ++e)
          if (ov[i * kMaxUniqEdges + tab[oe2u + mesh * nedges + e]]) valid = false;
        if (!valid) continue;
        float mlo = 1.0f;
        for (int t = 0; t < ntris; ++t)
          mlo = fminf(mlo, tb[i * kMaxUniqTris + tab[omsh + mesh * ntris + t]].x);
        L = fmaxf(L, mlo);
      }
#pragma unroll
      for (int j = G / 2; j > 0; j >>= 1) L = fmaxf(L, __shfl_xor_sync(gm, L, j, G));
      unsigned long long mask = 0;
      float best_hi = -INFINITY;
      for (int mesh = gl; mesh < nmeshes; mesh += G) {
        bool valid = true;
        for (int e = 0; e < nedges; ++e)
          if (ov[i * kMaxUniqEdges + tab[oe2u + mesh * nedges + e]]) valid = false;
        if (!valid) continue;
        float mhi = 1.0f;
        for (int t = 0; t < ntris; ++t)
          mhi = fminf(mhi, tb[i * kMaxUniqTris + tab[omsh + mesh * ntris + t]].y);
        if (!(mhi >= L && mhi > 0.0f)) continue;
        best_hi = fmaxf(best_hi, mhi);
        for (int t = 0; t < ntris; ++t) {
          int u = tab[omsh + mesh * ntris + t];
          if (tb[i * kMaxUniqTris + u].x <= mhi) mask |= 1ull << u;
        }
      }
#pragma unroll
      for (int j = G / 2; j > 0; j >>= 1) {
        best_hi = fmaxf(best_hi, __shfl_xor_sync(gm, best_hi, j, G));
        mask |= __shfl_xor_sync(gm, mask, j, G);
      }
      // cannot beat the worst current quality: no FP64 work (L = +inf
      // marks it for the selection below)
      if (improving && best_hi < o3[i]) {
        mask = 0;
        L = INFINITY;
      }
      if (gl == 0) {
        nd[i] = mask;
        lst[i] = L;
      }
    });
  }
  auto nd = cview(need);
  {
    // the triangles that need FP64, as one dense list (full warps on the
    // narrow FP64 pipe)
    Arr<LO> tcnt(n);
    auto tc = view(tcnt);
    pfor(n, [=] __device__(LO i) { tc[i] = __popcll(nd[i]); });
    // the list is sized by its bound (every unique triangle of every
    // candidate) and walked up to its count on the device: no host wait
    Arr<LO> toff = offset_scan(tcnt);
    LO bound = n * kMaxUniqTris;
    Arr<LO> ent(bound);
    auto of = cview(toff);
    auto en = view(ent);
    pfor(n, [=] __device__(LO i) {
      unsigned long long mbits = nd[i];
      LO j = of[i];
      while (mbits) {
        int u = __ffsll((long long)mbits) - 1;
        mbits &= mbits - 1;
        en[j++] = i * kMaxUniqTris + u;
      }
    });
    auto q = view(tq);
    auto enc = cview(ent);
    pfor_dev_count(toff.data() + n, bound, [=] __device__(LO j) {
      LO idx = enc[j];
      // an entry no tile wrote (only after a scan tile gave up its wait,
      // which the pass reports as an error) is skipped, not followed
      if (idx < 0 || idx >= bound) return;
      LO i = idx / kMaxUniqTris;
      int u = idx % kMaxUniqTris;
      int size = ls[i];
      int otri = tab[size * 9 + SW_OTRI];
      LO tet[4];
      for (int k = 0; k < 3; ++k) tet[k] = lv[i * 7 + tab[otri + u * 3 + k]];
      double tmq = 1.0;
      for (int tt = 0; tt < 2; ++tt) {
        tet[3] = le[i * 2 + (1 - tt)];
        tmq = min2d(tmq, tet_quality_exact(sv, c, mt, tet));
        LO sw = tet[1];
        tet[1] = tet[2];
        tet[2] = sw;
      }
      q[idx] = tmq;
      warp_count(&cnt[1], 2u);
    });
  }
  auto q = cview(tq);
  auto lst = cview(lstar);
  auto quals = view(quals_p, n);
  auto configs = view(configs_p, n);
  pfor(n, [=] __device__(LO i) {
    int size = ls[i];
    int best = -1;
    double bestq = 0.0;
    if (size < 3) {
      quals[i] = -1.0;
      configs[i] = -1;
      return;
    }
    const int* h = &tab[size * 9];
    int nmeshes = h[SW_NMESH], ntris = h[SW_NTRI], nedges = h[SW_NEDGE];
    int omsh = h[SW_OMESH], oe2u = h[SW_OE2U];
    float L = lst[i];
    if (L == INFINITY) {  // cannot improve (improving_only)
      configs[i] = -1;
      quals[i] = -DBL_MAX;
      return;
    }
    for (int mesh = 0; mesh < nmeshes; ++mesh) {
      bool valid = true;
      for (int e = 0; e < nedges; ++e)
        if (ov[i * kMaxUniqEdges + tab[oe2u + mesh * nedges + e]]) valid = false;
      if (!valid) continue;
      float mhi = 1.0f;
      for (int t = 0; t < ntris; ++t)
        mhi = fminf(mhi, tb[i * kMaxUniqTris + tab[omsh + mesh * ntris + t]].y);
      if (!(mhi >= L && mhi > 0.0f)) continue;
      double mq = 1.0;
      for (int t = 0; t < ntris; ++t) {
        int u = tab[omsh + mesh * ntris + t];
        if (tb[i * kMaxUniqTris + u].x <= mhi) mq = min2d(mq, q[i * kMaxUniqTris + u]);
      }
      if (mq > bestq) {
        best = mesh;
        bestq = mq;
      }
    }
    configs[i] = I8(best);
    quals[i] = bestq;
  });
}

void swap3d_qualities(Mesh& m, double max_len, const LO* c2e_p, LO n, double* quals_p,
                      I8* configs_p) {
  int mc = m.mcomp();  // metric components per vertex (1: isotropic)
  if (ctx().screening) {
    swap3d_qualities_screened(m, max_len, c2e_p, n, quals_p, configs_p);
    return;
  }
  auto tab = swap_tables();
  Arr<int> lsize;
  Arr<LO> lverts, leev;
  swap_loops(m, c2e_p, n, lsize, lverts, leev);
  auto ls = cview(lsize);
  auto lv = cview(lverts);
  auto le = cview(leev);
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  Arr<double> tq(n * kMaxUniqTris), el(n * kMaxUniqEdges);
  {
    auto q = view(tq);
    pfor(n * kMaxUniqTris, [=] __device__(LO idx) {
      LO i = idx / kMaxUniqTris;
      int u = idx % kMaxUniqTris;
      int size = ls[i];
      if (size < 3 || u >= tab[size * 9 + SW_NUTRI]) return;
      int otri = tab[size * 9 + SW_OTRI];
      LO tet[4];
      for (int k = 0; k < 3; ++k) tet[k] = lv[i * 7 + tab[otri + u * 3 + k]];
      double tmq = 1.0;
      for (int tt = 0; tt < 2; ++tt) {
        tet[3] = le[i * 2 + (1 - tt)];
        tmq = min2d(tmq, elem_quality_v(3, c, mt, mc, tet));
        LO s = tet[1];
        tet[1] = tet[2];
        tet[2] = s;
      }
      q[idx] = tmq;
    });
  }
  {
    auto l = view(el);
    pfor(n * kMaxUniqEdges, [=] __device__(LO idx) {
      LO i = idx / kMaxUniqEdges;
      int u = idx % kMaxUniqEdges;
      int size = ls[i];
      if (size < 3 || u >= tab[size * 9 + SW_NUEDGE]) return;
      int oued = tab[size * 9 + SW_OUEDGE];
      LO a = lv[i * 7 + tab[oued + u * 2]], b = lv[i * 7 + tab[oued + u * 2 + 1]];
      l[idx] = edge_len_v(3, c, mt, mc, a, b);
    });
  }
  auto q = cview(tq);
  auto l = cview(el);
  auto quals = view(quals_p, n);
  auto configs = view(configs_p, n);
  pfor(n, [=] __device__(LO i) {
    int size = ls[i];
    if (size < 3) {
      quals[i] = -1.0;
      configs[i] = -1;
      return;
    }
    const int* h = &tab[size * 9];
    int nmeshes = h[SW_NMESH], ntris = h[SW_NTRI], nedges = h[SW_NEDGE];
    int omsh = h[SW_OMESH], oe2u = h[SW_OE2U];
    int best = -1;
    double bestq = 0.0;
    for (int mesh = 0; mesh < nmeshes; ++mesh) {
      double mq = 1.0;
      for (int t = 0; t < ntris; ++t) {
        mq = min2d(mq, q[i * kMaxUniqTris + tab[omsh + mesh * ntris + t]]);
        if (mq < 0.0) break;
      }
      if (mq > bestq) {
        bool over = false;
        for (int e = 0; e < nedges; ++e)
          if (l[i * kMaxUniqEdges + tab[oe2u + mesh * nedges + e]] > max_len) {
            over = true;
            break;
          }
        if (!over) {
          best = mesh;
          bestq = mq;
        }
      }
    }
    configs[i] = I8(best);
    quals[i] = bestq;
  });
}

// mark_sliver_layers (src/Omega_h_mark.cpp:190-212): elements below the
// quality ceiling, then nlayers rounds of max over dual-graph neighbours
Arr<I8> mark_sliver_layers(Mesh& m, double ceil, int nlayers) {
  const Arr<double>& q = m.ask_qualities();
  LO ne = m.nelems();
  Arr<I8> a(ne), b(ne);
  {
    auto qq = cview(q);
    auto s = view(a);
    pfor(ne, [=] __device__(LO i) { s[i] = qq[i] < ceil; });
  }
  // the dual graph (elements across their sides) as a fixed-width table:
  // the other element across each side of e, -1 on the boundary (a side of
  // a simplicial mesh has at most two elements), so no sizes are read back
  int nse = m.dim + 1;
  Arr<LO> across(ne * nse);
  {
    auto es = cview(m.ask_down(m.dim, m.dim - 1).ab2b);
    const Adj& s2e = m.ask_up_any_order(m.dim - 1, m.dim);  // a maximum: row order is free
    auto sa = cview(s2e.a2ab);
    auto sb = cview(s2e.ab2b);
    auto ac = view(across);
    pfor(ne, [=] __device__(LO e) {
      for (int k = 0; k < nse; ++k) {
        LO sd = es[e * nse + k], other = -1;
        for (LO x = sa[sd]; x < sa[sd + 1]; ++x)
          if (sb[x] != e) other = sb[x];
        ac[e * nse + k] = other;
      }
    });
  }
  auto ac = cview(across);
  for (int l = 0; l < nlayers; ++l) {
    auto o = cview(a);
    auto nw = view(b);
    pfor(ne, [=] __device__(LO e) {
      int r = -128;
      for (int k = 0; k < nse; ++k) {
        LO f = ac[e * nse + k];
        if (f >= 0) r = max(r, int(o[f]));
      }
      nw[e] = I8(r);
    });
    std::swap(a, b);
  }
  return a;
}

// swap2d cavity (src/Omega_h_swap2d_qualities.cpp:35-46): the vertices
// opposite an interior edge in its two triangles, ordered by the triangles'
// rotation codes
__device__ __forceinline__ bool swap2d_opposite(LV ea, LV eb, View<const I8> ec, LV tv, LO edge,
                                                LO ov[2]) {
  if (ea[edge + 1] - ea[edge] != 2) return false;
  for (int i = 0; i < 2; ++i) {
    LO x = ea[edge] + i;
    I8 code = ec[x];
    int rot = code_rotation(code) & 1;
    ov[rot] = tv[eb[x] * 3 + opposite_template(2, 1, code_which_down(code))];
  }
  return true;
}

// swap2d_qualities_tmpl (src/Omega_h_swap2d_qualities.cpp:15-67): -1 where the
// new diagonal (ov[0], ov[1]) is longer than max_len, else the min of 1 and
// the two new triangles' qualities
void swap2d_qualities(Mesh& m, double max_len, const LO* c2e_p, LO n, double* quals_p) {
  int mc = m.mcomp();  // metric components per vertex (1: isotropic)
  const Adj& e2t = m.ask_up(1, 2);
  auto ea = cview(e2t.a2ab);
  auto eb = cview(e2t.ab2b);
  auto ec = cview(e2t.codes);
  auto tv = cview(m.ask_verts_of(2));
  auto ev = cview(m.ask_verts_of(1));
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto c2e = cview(c2e_p, n);
  auto q = view(quals_p, n);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO cand) {
    LO edge = c2e[cand];
    LO ov[2];
    if (!swap2d_opposite(ea, eb, ec, tv, edge, ov)) {
      raise_status(st, ST_TOPOLOGY);
      q[cand] = -1.0;
      return;
    }
    if (edge_len_v(2, c, mt, mc, ov[0], ov[1]) > max_len) {
      q[cand] = -1.0;
      return;
    }
    LO e0 = ev[edge * 2], e1 = ev[edge * 2 + 1];
    double minq = 1.0;
    for (int i = 0; i < 2; ++i) {
      LO ntv[3] = {i == 0 ? e1 : e0, ov[i], ov[1 - i]};
      minq = min2d(minq, elem_quality_v(2, c, mt, mc, ntv));
    }
    q[cand] = minq;
  });
}

// filter_swap_improve (src/Omega_h_swap.cpp:35-43) and find_indset over the
// kept candidates: the key edges
static Arr<LO> swap_keys(Mesh& m, Arr<LO> c2e, Arr<double> cq, PassStats* st) {
  LO nc = c2e.size();
  LO ne = m.nedges();
  Arr<I8> keep(nc);
  {
    auto eq = cview(m.ask_qualities());
    const Adj& e2t = m.ask_up(1, m.dim);
    auto ea = cview(e2t.a2ab);
    auto eb = cview(e2t.ab2b);
    auto ce = cview(c2e);
    auto q = cview(cq);
    auto kp = view(keep);
    pfor(nc, [=] __device__(LO i) {
      LO e = ce[i];
      double old = DBL_MAX;
      for (LO x = ea[e]; x < ea[e + 1]; ++x) old = min2d(old, eq[eb[x]]);
      kp[i] = q[i] > old;
    });
  }
  // the improving candidates marked on the edges directly (no compaction
  // and no host wait: without any, the independent set is empty)
  Arr<I8> is_cand = fill<I8>(ne, 0);
  Arr<double> edge_q = fill<double>(ne, -1.0);
  {
    auto ce = cview(c2e);
    auto q = cview(cq);
    auto kp = cview(keep);
    auto ic = view(is_cand);
    auto eq = view(edge_q);
    pfor(nc, [=] __device__(LO i) {
      if (kp[i]) {
        ic[ce[i]] = 1;
        eq[ce[i]] = q[i];
      }
    });
  }
  Arr<I8> keys = find_indset(m, EDGE, edge_q, is_cand);
  Arr<LO> k2e = collect_marked(keys);
  st->swap_keys = k2e.size();
  return k2e;
}

// modify + transfer_swap: every product inherits the key edge's
// classification; lengths and qualities of products are re-measured
static void swap_rebuild(Mesh& m, const Arr<LO>& k2e, Arr<LO>* k2p, Arr<LO>* pv2v,
                         bool check_rings) {
  int dim = m.dim;
  LO nkeys = k2e.size();
  Mesh nm;
  nm.dim = dim;
  nm.rebuilt = true;  // element-based partitioning after a rebuild
  nm.metric_comps = m.metric_comps;
  nm.class_sets = m.class_sets;
  nm.nents[0] = m.nverts();
  nm.coords = m.coords;
  nm.metric = m.metric;
  nm.screen = m.screen;  // same vertices, same screening data
  nm.class_dim[0] = m.class_dim[0];
  nm.class_id[0] = m.class_id[0];
  Arr<LO> old_lows2new = iota(m.nverts());
  // every dimension's plan, then one wait for their sizes and the status
  // word (an invalid edge ring raised ST_TOPOLOGY while the products were
  // written)
  ModifyPlan plans[4];
  {
    std::vector<ModifyPlan*> pls;
    std::vector<const Arr<LO>*> kps;
    Arr<I8> key_marks = mark_image(k2e, m.nedges());
    for (int d = 1; d <= dim; ++d) {
      plans[d] = plan_modify(m, d, EDGE, k2e, k2p[d], &key_marks);
      pls.push_back(&plans[d]);
      kps.push_back(&k2p[d]);
    }
    int status = 0;
    plan_sizes(pls, kps, &status);
    if (check_rings && (status & ST_TOPOLOGY)) throw Error(10, "edge swap found an invalid edge ring");
  }
  for (int d = 1; d <= dim; ++d) {
    ModifyOut mo = apply_modify(m, nm, d, EDGE, plans[d], k2e, k2p[d], pv2v[d], old_lows2new);
    LO nnew = nm.nents[d];
    LO np = mo.prods2new.size();
    Arr<I8> pcd(np);
    Arr<LO> pci(np);
    {
      auto ke = cview(k2e);
      auto kp = cview(k2p[d]);
      auto ecd = cview(m.class_dim[1]);
      auto eci = cview(m.class_id[1]);
      auto a = view(pcd);
      auto b = view(pci);
      pfor(nkeys, [=] __device__(LO k) {
        for (LO p = kp[k]; p < kp[k + 1]; ++p) {
          a[p] = ecd[ke[k]];
          b[p] = eci[ke[k]];
        }
      });
    }
    xfer_class(m, nm, d, mo, nnew, pcd.data(), pci.data(), nullptr);
    xfer_lengths_qualities(m, nm, d, mo, &pv2v[d]);
    old_lows2new = mo.old2new;
  }
  m = std::move(nm);
}

// swap_edges_2d (src/Omega_h_swap2d.cpp:14-80) with swap2d_topology
// (src/Omega_h_swap2d_topology.cpp:37-95): per key one new edge
// (ov[0], ov[1]) and two new triangles (ev[1-i], ov[i], ov[1-i])
static bool swap_edges_2d(Mesh& m, const AdaptOpts& o, PassStats* st, Arr<LO> c2e) {
  LO nc = c2e.size();
  Arr<double> cq(nc);
  swap2d_qualities(m, o.max_length_allowed, c2e.data(), nc, cq.data());
  if (ctx().take_status() & ST_TOPOLOGY) throw Error(10, "2D edge swap: an interior edge without two triangles");
  Arr<LO> k2e = swap_keys(m, c2e, cq, st);
  LO nkeys = k2e.size();
  if (nkeys == 0) return false;
  Arr<LO> k2p[4], pv2v[4];
  k2p[1] = iota(nkeys + 1);
  k2p[2] = Arr<LO>(nkeys + 1);
  pv2v[1] = Arr<LO>(nkeys * 2);
  pv2v[2] = Arr<LO>(nkeys * 6);
  {
    const Adj& e2t = m.ask_up(1, 2);
    auto ea = cview(e2t.a2ab);
    auto eb = cview(e2t.ab2b);
    auto ec = cview(e2t.codes);
    auto tv = cview(m.ask_verts_of(2));
    auto ev = cview(m.ask_verts_of(1));
    auto ke = cview(k2e);
    auto p2 = view(k2p[2]);
    auto v1 = view(pv2v[1]);
    auto v2 = view(pv2v[2]);
    pfor(nkeys + 1, [=] __device__(LO k) { p2[k] = 2 * k; });
    pfor(nkeys, [=] __device__(LO k) {
      LO e = ke[k];
      LO ov[2];
      swap2d_opposite(ea, eb, ec, tv, e, ov);
      v1[k * 2] = ov[0];
      v1[k * 2 + 1] = ov[1];
      LO e0 = ev[e * 2], e1 = ev[e * 2 + 1];
      for (int i = 0; i < 2; ++i) {
        LO t = k * 2 + i;
        v2[t * 3] = i == 0 ? e1 : e0;
        v2[t * 3 + 1] = ov[i];
        v2[t * 3 + 2] = ov[1 - i];
      }
    });
  }
  swap_rebuild(m, k2e, k2p, pv2v, false);
  return true;
}

// swap_edges_3d (src/Omega_h_swap3d.cpp:14-84)
static bool swap_edges_3d(Mesh& m, const AdaptOpts& o, PassStats* st, Arr<LO> c2e) {
  LO nc = c2e.size();
  Arr<double> cq(nc);
  Arr<I8> cc(nc);
  if (ctx().screening)
    swap3d_qualities_screened(m, o.max_length_allowed, c2e.data(), nc, cq.data(), cc.data(),
                              true);
  else
    swap3d_qualities(m, o.max_length_allowed, c2e.data(), nc, cq.data(), cc.data());
  LO ne = m.nedges();
  Arr<I8> econfig = map_onto(cc, c2e, ne, I8(-1), 1);
  Arr<LO> k2e = swap_keys(m, c2e, cq, st);
  LO nkeys = k2e.size();
  if (nkeys == 0) return false;
  // swap3d_keys_to_prods + swap3d_topology (src/Omega_h_swap3d_topology.cpp)
  auto tab = swap_tables();
  Arr<int> lsize;
  Arr<LO> lverts, leev;
  swap_loops(m, k2e.data(), nkeys, lsize, lverts, leev);
  Arr<LO> cnt[4], k2p[4], pv2v[4];
  for (int d = 1; d <= 3; ++d) cnt[d] = Arr<LO>(nkeys);
  {
    auto ls = cview(lsize);
    auto c1 = view(cnt[1]);
    auto c2 = view(cnt[2]);
    auto c3 = view(cnt[3]);
    pfor(nkeys, [=] __device__(LO k) {
      int size = ls[k];
      int npt = tab[size * 9 + SW_NTRI], npe = tab[size * 9 + SW_NEDGE];
      c1[k] = npe;
      c2[k] = npt + 2 * npe;
      c3[k] = 2 * npt;
    });
  }
  // products' vertices sized by the tables' largest product counts per key
  // (no host wait; the exact counts come with the rebuild's sizes)
  int maxp[4];
  swap3d_max_products(maxp);
  for (int d = 1; d <= 3; ++d) {
    k2p[d] = offset_scan(cnt[d]);
    long long cap = (long long)nkeys * maxp[d] * (d + 1);
    if (cap > 0x7fffffffLL) throw Error(8, "edge swap: too many products");
    pv2v[d] = Arr<LO>(LO(cap));
  }
  {
    auto ls = cview(lsize);
    auto lv = cview(lverts);
    auto le = cview(leev);
    auto ke = cview(k2e);
    auto cfg = cview(econfig);
    auto p1 = cview(k2p[1]);
    auto p2 = cview(k2p[2]);
    auto p3 = cview(k2p[3]);
    auto v1 = view(pv2v[1]);
    auto v2 = view(pv2v[2]);
    auto v3 = view(pv2v[3]);
    int* stw = ctx().d_status;
    pfor(nkeys, [=] __device__(LO k) {
      int size = ls[k];
      int config = cfg[ke[k]];
      if (size < 3 || config < 0 || config >= tab[size * 9 + SW_NMESH]) {
        // no valid configuration: the key's products get one of its loop
        // vertices (a valid index) and the status word reports the failure
        raise_status(stw, ST_TOPOLOGY);
        LO a = le[k * 2];
        for (LO p = p1[k] * 2; p < p1[k + 1] * 2; ++p) v1[p] = a;
        for (LO p = p2[k] * 3; p < p2[k + 1] * 3; ++p) v2[p] = a;
        for (LO p = p3[k] * 4; p < p3[k + 1] * 4; ++p) v3[p] = a;
        return;
      }
      const int* h = &tab[size * 9];
      int npt = h[SW_NTRI], npe = h[SW_NEDGE];
      int otri = h[SW_OTRI], omsh = h[SW_OMESH], oued = h[SW_OUEDGE], oe2u = h[SW_OE2U];
      for (int pe = 0; pe < npe; ++pe) {
        int ue = tab[oe2u + config * npe + pe];
        LO a = lv[k * 7 + tab[oued + ue * 2]], b = lv[k * 7 + tab[oued + ue * 2 + 1]];
        LO pedge = p1[k] + pe;
        v1[pedge * 2] = a;
        v1[pedge * 2 + 1] = b;
        for (int eev = 0; eev < 2; ++eev) {
          LO ptri = p2[k] + 2 * pe + eev;
          v2[ptri * 3] = a;
          v2[ptri * 3 + 1] = b;
          v2[ptri * 3 + 2] = le[k * 2 + eev];
        }
      }
      for (int pt = 0; pt < npt; ++pt) {
        int ut = tab[omsh + config * npt + pt];
        LO t0 = lv[k * 7 + tab[otri + ut * 3]];
        LO t1 = lv[k * 7 + tab[otri + ut * 3 + 1]];
        LO t2 = lv[k * 7 + tab[otri + ut * 3 + 2]];
        LO ptri = p2[k] + 2 * npe + pt;
        v2[ptri * 3] = t0;
        v2[ptri * 3 + 1] = t1;
        v2[ptri * 3 + 2] = t2;
        for (int eev = 0; eev < 2; ++eev) {
          LO ptet = p3[k] + 2 * pt + eev;
          v3[ptet * 4] = t0;
          v3[ptet * 4 + 1] = eev == 0 ? t2 : t1;
          v3[ptet * 4 + 2] = eev == 0 ? t1 : t2;
          v3[ptet * 4 + 3] = le[k * 2 + eev];
        }
      }
    });
  }
  swap_rebuild(m, k2e, k2p, pv2v, true);
  return true;
}

// swap_edges (src/Omega_h_swap.cpp:45-53) after swap_part1
// (src/Omega_h_swap.cpp:14-27): interior edges of the sliver layers
bool swap_edges(Mesh& m, const AdaptOpts& o, PassStats* st) {
  m.parting = 1;  // swap_part1 (src/Omega_h_swap.cpp:15)
  int dim = m.dim;
  Arr<I8> ec = mark_sliver_layers(m, o.min_quality_desired, o.nsliver_layers);
  Arr<I8> edc = mark_down(m, dim, 1, ec);
  {
    auto e = view(edc);
    auto cd = cview(m.class_dim[1]);
    pfor(m.nedges(), [=] __device__(LO i) { e[i] = e[i] && cd[i] == dim; });
  }
  Arr<LO> c2e = collect_marked(edc);
  if (c2e.size() == 0) return false;
  return dim == 3 ? swap_edges_3d(m, o, st, c2e) : swap_edges_2d(m, o, st, c2e);
}

// ------------------------------------------------------------ adapt()
// Omega_h::adapt (src/Omega_h_adapt.cpp:153-212, 272-288) for meshes without
// conservation tags or a geometry model: nothing to do when qualities and
// lengths already meet the goals; satisfy_lengths (refine and coarsen by
// size until neither changes the mesh); satisfy_quality (edge swaps, else
// sliver collapses, until the worst quality reaches min_quality_desired or
// neither helps).
AdaptResult adapt(Mesh& m, const AdaptOpts& o) {
  AdaptResult r;
  PassStats st;
  auto meets_goals = [&] {
    const Arr<double>& len = m.ask_lengths();
    return min_f64(m.ask_qualities()) >= o.min_quality_desired &&
           min_f64(len) >= o.min_length_desired && max_f64(len) <= o.max_length_desired;
  };
  if (meets_goals()) return r;
  r.did = true;
  // element-based partitioning when adapt() returns (src/Omega_h_adapt.cpp:285)
  struct ElemBasedOnExit {
    Mesh& m;
    ~ElemBasedOnExit() { m.parting = 0; }
  } on_exit{m};
  constexpr int kMaxRounds = 1000;  // a guard; the reference's loops are unbounded
  bool any;
  do {
    any = false;
    if (refine_by_size(m, o, &st)) {
      ++r.refines;
      any = true;
    }
    if (coarsen_by_size(m, o, &st)) {
      ++r.coarsens;
      any = true;
    }
    if (++r.length_rounds > kMaxRounds) throw Error(5, "adapt: lengths did not settle");
  } while (any);
  if (min_f64(m.ask_qualities()) >= o.min_quality_desired) {
    r.quality_satisfied = true;
    return r;
  }
  int rounds = 0;
  do {
    if (++rounds > kMaxRounds) throw Error(5, "adapt: qualities did not settle");
    if (swap_edges(m, o, &st)) {
      ++r.swaps;
      continue;
    }
    if (coarsen_slivers(m, o, &st)) {
      ++r.sliver_coarsens;
      continue;
    }
    return r;  // could not satisfy quality
  } while (min_f64(m.ask_qualities()) < o.min_quality_desired);
  r.quality_satisfied = true;
  return r;
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
  // each operator of the pass runs on a ghosted mesh (partitioning state
  // only: one part has no ghosts to exchange)
  OHG_CUDA(cudaMemsetAsync(c.d_indset_sweeps, 0, sizeof(int), c.stream));
  OHG_CUDA(cudaEventRecord(e0, c.stream));
  m.parting = 1;
  st.did_refine = refine_by_size(m, o, &st);
  OHG_CUDA(cudaEventRecord(e1, c.stream));
  m.parting = 1;
  st.did_coarsen = coarsen_by_size(m, o, &st);
  OHG_CUDA(cudaEventRecord(e2, c.stream));
  m.parting = 1;
  // adapt() swaps only while the worst quality is below min_quality_desired
  // (src/Omega_h_adapt.cpp:196); with none below it, swap_edges finds no
  // candidate (its candidates are the sliver layers of those elements) and
  // changes nothing.  So the worst quality is only reported: it is read at
  // the pass's last host wait, not before the swap.
  Arr<double> minq = min_f64_dev(m.ask_qualities());
  OHG_CUDA(cudaMemcpyAsync(c.h_pass_min, minq.data(), sizeof(double), cudaMemcpyDeviceToHost,
                           c.stream));
  st.did_swap = swap_edges(m, o, &st);
  OHG_CUDA(cudaEventRecord(e3, c.stream));
  OHG_CUDA(cudaMemcpyAsync(c.h_indset_sweeps, c.d_indset_sweeps, sizeof(int),
                           cudaMemcpyDeviceToHost, c.stream));
  c.sync();
  st.min_quality = *c.h_pass_min;
  st.indset_rounds = *c.h_indset_sweeps;
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
