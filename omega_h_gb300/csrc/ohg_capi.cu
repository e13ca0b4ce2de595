// The C ABI (include/ohg.h) over the device mesh and operators.
#include <cstring>
#include <functional>
#include <string>

#include "../../include/ohg.h"
#include "ohg_metric.cuh"
#include "ohg_adapt.cuh"
#include "ohg_batch.cuh"

using namespace ohg;

struct ohg_context {
  Ctx ctx;
  explicit ohg_context(int dev) : ctx(dev) {}
};
struct ohg_mesh {
  ohg_context* owner;
  Mesh mesh;
};

static thread_local std::string g_err;

static int status_to_code(int st) {
  if (st & ST_NO_MATCH) return OHG_ERR_NO_MATCH;
  if (st & ST_LOOP_TOO_BIG) return OHG_ERR_LOOP_TOO_BIG;
  if (st & ST_BOUNDS) return OHG_ERR_BOUNDS;
  if (st & ST_TOPOLOGY) return OHG_ERR_TOPOLOGY;
  if (st & ST_NUMERIC) return OHG_ERR_NUMERIC;
  if (st & ST_STALL) return OHG_ERR_TIMEOUT;
  return OHG_OK;
}

// After a failed call the status bits it raised are cleared, so that they
// are not reported again by the next call on the context.
static void clear_status_after_error(ohg_context* c) {
  try {
    c->ctx.take_status();
  } catch (Error&) {
    cudaGetLastError();
  }
}

// runs f with the context current; converts exceptions and device status
template <class F>
static int guarded(ohg_context* c, F f) {
  if (!c) {
    g_err = "null context";
    return OHG_ERR_INVALID;
  }
  set_ctx(&c->ctx);
  try {
    // every entry point runs with its context's device current, so that
    // launches on the context's stream and device symbol lookups agree
    int cur = -1;
    OHG_CUDA(cudaGetDevice(&cur));
    if (cur != c->ctx.device) OHG_CUDA(cudaSetDevice(c->ctx.device));
    f();
    int st = c->ctx.take_status();
    int code = status_to_code(st);
    if (code != OHG_OK) {
      g_err = "device status word " + std::to_string(st);
      return code;
    }
    return OHG_OK;
  } catch (Error& e) {
    g_err = e.what();
    cudaGetLastError();
    clear_status_after_error(c);
    return e.code;
  } catch (std::exception& e) {
    g_err = e.what();
    clear_status_after_error(c);
    return OHG_ERR_INVALID;
  }
}
#define MESH_GUARD(m) \
  if (!(m)) {         \
    g_err = "null mesh"; \
    return OHG_ERR_INVALID; \
  }

extern "C" {

const char* ohg_last_error(void) { return g_err.c_str(); }

int ohg_context_create(int device, ohg_context** out) {
  try {
    *out = new ohg_context(device);
    return OHG_OK;
  } catch (Error& e) {
    g_err = e.what();
    return e.code;
  }
}
int ohg_context_destroy(ohg_context* c) {
  if (!c) return OHG_OK;
  set_ctx(&c->ctx);
  delete c;
  set_ctx(nullptr);
  return OHG_OK;
}
int ohg_context_launches(ohg_context* c, unsigned long long* out) {
  if (!c) return OHG_ERR_INVALID;
  *out = c->ctx.launches;
  return OHG_OK;
}
int ohg_context_syncs(ohg_context* c, unsigned long long* out) {
  if (!c || !out) return OHG_ERR_INVALID;
  *out = c->ctx.syncs;
  return OHG_OK;
}
int ohg_context_allocations(ohg_context* c, unsigned long long* out) {
  if (!c || !out) return OHG_ERR_INVALID;
  *out = c->ctx.allocs;
  return OHG_OK;
}

int ohg_context_autotune(ohg_context* c, int mode) {
  if (!c || mode < 0 || mode > 2) {
    g_err = "ohg_context_autotune: null context or mode not 0, 1 or 2";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    Ctx& x = ctx();
    x.sync();  // reads the exploration launches still in flight
    x.tuner.mode = mode;
  });
}
int ohg_context_force_variant(ohg_context* c, int force) {
  if (!c) {
    g_err = "null context";
    return OHG_ERR_INVALID;
  }
  c->ctx.tuner.forced = force < 0 ? -1 : force;
  return OHG_OK;
}
int ohg_context_tuning(ohg_context* c, int* counts3) {
  if (!counts3) {
    g_err = "null argument";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    Ctx& x = ctx();
    x.sync();
    int seen = 0, chosen = 0, moved = 0;
    for (auto& kv : x.tuner.sites) {
      ++seen;
      if (kv.second.chosen >= 0) {
        ++chosen;
        if (kv.second.chosen != kv.second.dflt) ++moved;
      }
    }
    counts3[0] = seen;
    counts3[1] = chosen;
    counts3[2] = moved;
  });
}

int ohg_context_set_screening(ohg_context* c, int on) {
  if (!c) {
    g_err = "null context";
    return OHG_ERR_INVALID;
  }
  c->ctx.screening = on ? 1 : 0;
  return OHG_OK;
}
int ohg_context_screen_counts(ohg_context* c, unsigned long long* out4, int reset) {
  if (!out4) {
    g_err = "null output";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    Ctx& x = ctx();
    OHG_CUDA(cudaMemcpyAsync(out4, x.d_screen_counts, 4 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, x.stream));
    if (reset)
      OHG_CUDA(cudaMemsetAsync(x.d_screen_counts, 0, 4 * sizeof(unsigned long long), x.stream));
    x.sync();
  });
}
int ohg_context_time_kernels(ohg_context* c, int on) {
  if (!c) {
    g_err = "null context";
    return OHG_ERR_INVALID;
  }
  c->ctx.time_kernels = on != 0;
  return OHG_OK;
}
int ohg_context_kernel_time(ohg_context* c, const char* name, double* total_ms,
                            double* total_bytes, int* launches, int reset) {
  if (!name || !total_ms || !total_bytes || !launches) {
    g_err = "null argument";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    Ctx& x = ctx();
    x.sync();
    double ms = 0, by = 0;
    int n = 0;
    for (auto& k : x.kernel_launches) {
      if (k.name != name) continue;
      float t = 0;
      OHG_CUDA(cudaEventElapsedTime(&t, k.start, k.stop));
      ms += t;
      by += k.bytes;
      ++n;
    }
    *total_ms = ms;
    *total_bytes = by;
    *launches = n;
    if (reset) {
      for (auto& k : x.kernel_launches) {
        cudaEventDestroy(k.start);
        cudaEventDestroy(k.stop);
      }
      x.kernel_launches.clear();
    }
  });
}
int ohg_context_stream(ohg_context* c, void** out) {
  if (!c) return OHG_ERR_INVALID;
  *out = reinterpret_cast<void*>(c->ctx.stream);
  return OHG_OK;
}

int ohg_mesh_from_arrays(ohg_context* c, int dim, const int* nents, const int* const* down,
                         const signed char* const* codes, const signed char* const* cdim,
                         const int* const* cid, const double* coords, const double* metric,
                         ohg_mesh** out) {
  if ((dim != 2 && dim != 3) || !nents || !down || !cdim || !cid || !coords || !metric) {
    g_err = "ohg_mesh_from_arrays: bad arguments";
    return OHG_ERR_INVALID;
  }
  ohg_mesh* m = new ohg_mesh{c, Mesh()};
  // the arrays may be device or host memory (the copy kind is inferred from
  // each address); the call returns after every copy completed
  int rc = guarded(c, [&] {
    Mesh& me = m->mesh;
    me.dim = dim;
    cudaStream_t s = ctx().stream;
    me.nents[0] = nents[0];
    for (int d = 1; d <= dim; ++d) {
      int deg = simplex_degree(d, d - 1);
      Adj a;
      a.ab2b = Arr<LO>(nents[d] * deg);
      OHG_CUDA(cudaMemcpyAsync(a.ab2b.data(), down[d], size_t(nents[d]) * deg * 4,
                               cudaMemcpyDefault, s));
      if (d >= 2) {
        if (!codes || !codes[d]) throw Error(OHG_ERR_INVALID, "missing alignment codes");
        a.codes = Arr<I8>(nents[d] * deg);
        a.has_codes = true;
        OHG_CUDA(cudaMemcpyAsync(a.codes.data(), codes[d], size_t(nents[d]) * deg,
                                 cudaMemcpyDefault, s));
      }
      me.set_ents(d, std::move(a));
    }
    for (int d = 0; d <= dim; ++d) {
      me.class_dim[d] = Arr<I8>(nents[d]);
      me.class_id[d] = Arr<LO>(nents[d]);
      OHG_CUDA(cudaMemcpyAsync(me.class_dim[d].data(), cdim[d], size_t(nents[d]),
                               cudaMemcpyDefault, s));
      OHG_CUDA(cudaMemcpyAsync(me.class_id[d].data(), cid[d], size_t(nents[d]) * 4,
                               cudaMemcpyDefault, s));
    }
    me.coords = Arr<double>(nents[0] * dim);
    me.metric = Arr<double>(nents[0] * me.mcomp());
    OHG_CUDA(cudaMemcpyAsync(me.coords.data(), coords, size_t(nents[0]) * dim * 8,
                             cudaMemcpyDefault, s));
    OHG_CUDA(cudaMemcpyAsync(me.metric.data(), metric, size_t(nents[0]) * me.mcomp() * 8,
                             cudaMemcpyDefault, s));
  });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

static void clone_mesh(const Mesh& a, Mesh& b) {
  b.dim = a.dim;
  for (int d = 0; d < 4; ++d) b.nents[d] = a.nents[d];
  for (int d = 1; d <= a.dim; ++d) {
    const Adj& x = a.adj.at({d, d - 1});
    Adj y;
    y.ab2b = copy_arr(x.ab2b);
    if (x.has_codes) {
      y.codes = copy_arr(x.codes);
      y.has_codes = true;
    }
    b.adj[{d, d - 1}] = std::move(y);
  }
  for (int d = 0; d <= a.dim; ++d) {
    b.class_dim[d] = copy_arr(a.class_dim[d]);
    b.class_id[d] = copy_arr(a.class_id[d]);
  }
  b.coords = copy_arr(a.coords);
  b.metric = copy_arr(a.metric);
  // the state written to .osh files (lengths and qualities are not copied:
  // a clone measures them afresh)
  b.metric_comps = a.metric_comps;
  b.parting = a.parting;
  b.rebuilt = a.rebuilt;
  b.class_sets = a.class_sets;
  for (const Mesh::Tag& t : a.extra_tags) b.extra_tags.push_back({t.dim, t.ncomps, t.type, t.name, copy_arr(t.bytes)});
  for (int d = 0; d < 4; ++d) b.tag_order[d] = a.tag_order[d];
}

int ohg_mesh_clone(ohg_mesh* src, ohg_mesh** out) {
  MESH_GUARD(src);
  ohg_mesh* m = new ohg_mesh{src->owner, Mesh()};
  int rc = guarded(src->owner, [&] { clone_mesh(src->mesh, m->mesh); });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

int ohg_mesh_clone_to(ohg_mesh* src, ohg_context* c, ohg_mesh** out) {
  MESH_GUARD(src);
  if (!c || !out) {
    g_err = "ohg_mesh_clone_to: null context or output";
    return OHG_ERR_INVALID;
  }
  // the source's arrays are complete once its context's stream is idle;
  // the copies then run on the target context's stream
  int rc = guarded(src->owner, [&] { ctx().sync(); });
  if (rc != OHG_OK) return rc;
  ohg_mesh* m = new ohg_mesh{c, Mesh()};
  rc = guarded(c, [&] { clone_mesh(src->mesh, m->mesh); });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

int ohg_mesh_write_osh(ohg_mesh* m, const char* path, int compress) {
  MESH_GUARD(m);
  if (!path) {
    g_err = "ohg_mesh_write_osh: null path";
    return OHG_ERR_INVALID;
  }
  return guarded(m->owner, [&] { write_osh(m->mesh, path, compress != 0); });
}

int ohg_mesh_read_osh(ohg_context* c, const char* path, ohg_mesh** out) {
  if (!c || !path || !out) {
    g_err = "ohg_mesh_read_osh: null argument";
    return OHG_ERR_INVALID;
  }
  ohg_mesh* m = new ohg_mesh{c, Mesh()};
  int rc = guarded(c, [&] { m->mesh = read_osh(path); });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

int ohg_osh_zlib(int* available) {
  if (!available) return OHG_ERR_INVALID;
  *available = zlib_available() ? 1 : 0;
  return OHG_OK;
}

int ohg_build_box(ohg_context* c, int dim, int n, ohg_mesh** out) {
  if ((dim != 2 && dim != 3) || n < 1) {
    g_err = "ohg_build_box: dim must be 2 or 3 and n >= 1";
    return OHG_ERR_INVALID;
  }
  ohg_mesh* m = new ohg_mesh{c, Mesh()};
  int rc = guarded(c, [&] { m->mesh = build_box(dim, n); });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

int ohg_mesh_apply_workload(ohg_mesh* m, int n, unsigned long long seed, int kind) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { apply_workload(m->mesh, n, seed, kind); });
}

int ohg_mesh_from_elems(ohg_context* c, int dim, int nverts, int nelems, const int* ev2v,
                        const double* coords, const double* metric, ohg_mesh** out) {
  ohg_mesh* m = new ohg_mesh{c, Mesh()};
  int rc = guarded(c, [&] {
    Mesh& me = m->mesh;
    me.dim = dim;
    me.nents[0] = nverts;
    Arr<LO> ev(nelems * (dim + 1));
    OHG_CUDA(cudaMemcpyAsync(ev.data(), ev2v, size_t(ev.size()) * sizeof(LO),
                             cudaMemcpyDeviceToDevice, ctx().stream));
    for (int md = 1; md < dim; ++md) {
      Arr<LO> mv = find_unique(ev, nelems, dim, md);
      if (md == 1) {
        Adj a;
        a.ab2b = mv;
        me.set_ents(1, std::move(a));
      } else {
        me.set_ents(md, reflect_down(mv, mv.size() / (md + 1), me.ask_verts_of(md - 1),
                                     me.ask_up(0, md - 1), md, md - 1));
      }
    }
    me.set_ents(dim, reflect_down(ev, nelems, me.ask_verts_of(dim - 1), me.ask_up(0, dim - 1),
                                  dim, dim - 1));
    me.coords = Arr<double>(nverts * dim);
    OHG_CUDA(cudaMemcpyAsync(me.coords.data(), coords, size_t(nverts) * dim * sizeof(double),
                             cudaMemcpyDeviceToDevice, ctx().stream));
    me.metric = Arr<double>(nverts * me.mcomp());
    OHG_CUDA(cudaMemcpyAsync(me.metric.data(), metric, size_t(nverts) * me.mcomp() * sizeof(double),
                             cudaMemcpyDeviceToDevice, ctx().stream));
    for (int d = 0; d <= dim; ++d) {
      me.class_dim[d] = fill<I8>(me.nents[d], I8(dim));
      me.class_id[d] = fill<LO>(me.nents[d], 0);
    }
  });
  if (rc != OHG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return OHG_OK;
}

int ohg_mesh_destroy(ohg_mesh* m) {
  if (!m) return OHG_OK;
  set_ctx(&m->owner->ctx);
  delete m;
  return OHG_OK;
}
int ohg_mesh_dim(ohg_mesh* m, int* out) {
  MESH_GUARD(m);
  *out = m->mesh.dim;
  return OHG_OK;
}
int ohg_mesh_device_bytes(ohg_mesh* m, long long* out) {
  MESH_GUARD(m);
  if (!out) return OHG_ERR_INVALID;
  *out = (long long)mesh_device_bytes(m->mesh);
  return OHG_OK;
}
int ohg_context_pool_bytes(ohg_context* c, int reset_high, long long* used, long long* reserved,
                           long long* used_high) {
  if (!c || !used || !reserved || !used_high) {
    g_err = "ohg_context_pool_bytes: null argument";
    return OHG_ERR_INVALID;
  }
  // a device-level query: it touches neither the context's stream nor its
  // status word, so any thread may call it while others use the context
  cudaMemPool_t pool;
  std::uint64_t u = 0, r = 0, h = 0;
  cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, c->ctx.device);
  if (e == cudaSuccess) e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u);
  if (e == cudaSuccess) e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r);
  if (e == cudaSuccess) e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &h);
  if (e == cudaSuccess && reset_high) {
    std::uint64_t zero = 0;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero);
  }
  if (e != cudaSuccess) {
    g_err = std::string("memory pool query failed: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return OHG_ERR_CUDA;
  }
  // blocks the contexts keep for reuse count as in use, as the pool counts
  // them: the high-water mark, taken by the pool, includes them too
  *used = (long long)u;
  *reserved = (long long)r;
  *used_high = (long long)h;
  return OHG_OK;
}
int ohg_mesh_nents(ohg_mesh* m, int d, int* out) {
  MESH_GUARD(m);
  if (d < 0 || d > m->mesh.dim) return OHG_ERR_INVALID;
  *out = m->mesh.nents[d];
  return OHG_OK;
}

// resolves a named array to (pointer, bytes); derives adjacencies on demand
static bool named_array(Mesh& me, const std::string& name, const void** p, long long* bytes,
                        Arr<GO>* tmp) {
  auto num = [&](size_t pos) { return name[pos] - '0'; };
  auto set = [&](const void* q, long long b) {
    *p = q;
    *bytes = b;
    return true;
  };
  int dim = me.dim;
  if (name == "coords") return set(me.coords.data(), me.coords.size() * 8LL);
  if (name == "metric") return set(me.metric.data(), me.metric.size() * 8LL);
  if (name == "length") {
    const Arr<double>& a = me.ask_lengths();
    return set(a.data(), a.size() * 8LL);
  }
  if (name == "quality") {
    const Arr<double>& a = me.ask_qualities();
    return set(a.data(), a.size() * 8LL);
  }
  auto dvalid = [&](int d) { return d >= 0 && d <= dim; };
  if (name.rfind("ev2v_", 0) == 0 && name.size() == 6 && dvalid(num(5)) && num(5) > 0) {
    const Arr<LO>& a = me.ask_verts_of(num(5));
    return set(a.data(), a.size() * 4LL);
  }
  if (name.rfind("down_", 0) == 0 && name.size() == 6 && dvalid(num(5)) && num(5) > 0) {
    const Adj& a = me.ask_down(num(5), num(5) - 1);
    return set(a.ab2b.data(), a.ab2b.size() * 4LL);
  }
  if (name.rfind("downcodes_", 0) == 0 && name.size() == 11 && dvalid(num(10)) && num(10) > 1) {
    const Adj& a = me.ask_down(num(10), num(10) - 1);
    return set(a.codes.data(), a.codes.size() * 1LL);
  }
  if (name == "down31" || name == "downcodes31") {
    if (dim != 3) return false;
    const Adj& a = me.ask_down(3, 1);
    if (name == "down31") return set(a.ab2b.data(), a.ab2b.size() * 4LL);
    return set(a.codes.data(), a.codes.size() * 1LL);
  }
  if (name.rfind("class_dim_", 0) == 0 && name.size() == 11 && dvalid(num(10)))
    return set(me.class_dim[num(10)].data(), me.class_dim[num(10)].size() * 1LL);
  if (name.rfind("class_id_", 0) == 0 && name.size() == 10 && dvalid(num(9)))
    return set(me.class_id[num(9)].data(), me.class_id[num(9)].size() * 4LL);
  if (name.rfind("global_", 0) == 0 && name.size() == 8 && dvalid(num(7))) {
    LO n = me.nents[num(7)];
    *tmp = Arr<GO>(n);
    GO* g = tmp->data();
    pfor(n, [=] __device__(LO i) { g[i] = i; });
    return set(g, n * 8LL);
  }
  if (name.rfind("up_", 0) == 0 && name.size() >= 10) {
    int lo = num(name.size() - 2), hi = num(name.size() - 1);
    if (!(dvalid(lo) && dvalid(hi) && lo < hi)) return false;
    const Adj& a = me.ask_up(lo, hi);
    std::string kind = name.substr(0, name.size() - 2);
    if (kind == "up_a2ab_") return set(a.a2ab.data(), a.a2ab.size() * 4LL);
    if (kind == "up_ab2b_") return set(a.ab2b.data(), a.ab2b.size() * 4LL);
    if (kind == "up_codes_") return set(a.codes.data(), a.codes.size() * 1LL);
    return false;
  }
  if (name.rfind("star_", 0) == 0 && name.size() == 11) {
    int d = num(10);
    if (d < 0 || d > 1 || d >= dim) return false;
    const Adj& a = me.ask_adj(d, d);
    if (name.substr(0, 10) == "star_a2ab_") return set(a.a2ab.data(), a.a2ab.size() * 4LL);
    if (name.substr(0, 10) == "star_ab2b_") return set(a.ab2b.data(), a.ab2b.size() * 4LL);
    return false;
  }
  if (name == "dual_a2ab" || name == "dual_ab2b") {
    const Adj& a = me.ask_adj(dim, dim);
    if (name == "dual_a2ab") return set(a.a2ab.data(), a.a2ab.size() * 4LL);
    return set(a.ab2b.data(), a.ab2b.size() * 4LL);
  }
  return false;
}

int ohg_mesh_array_bytes(ohg_mesh* m, const char* name, long long* nbytes) {
  MESH_GUARD(m);
  bool ok = false;
  int rc = guarded(m->owner, [&] {
    const void* p;
    Arr<GO> tmp;
    ok = named_array(m->mesh, name, &p, nbytes, &tmp);
  });
  if (rc == OHG_OK && !ok) {
    g_err = std::string("unknown mesh array ") + name;
    return OHG_ERR_INVALID;
  }
  return rc;
}
int ohg_mesh_get_array(ohg_mesh* m, const char* name, void* dst, long long cap) {
  MESH_GUARD(m);
  bool ok = false, fits = true;
  int rc = guarded(m->owner, [&] {
    const void* p;
    long long b;
    Arr<GO> tmp;
    ok = named_array(m->mesh, name, &p, &b, &tmp);
    if (!ok) return;
    if (b > cap) {
      fits = false;
      return;
    }
    // dst may be device memory or host memory (pinned host memory is copied
    // to by DMA); the kind is inferred from the address
    if (b) OHG_CUDA(cudaMemcpyAsync(dst, p, size_t(b), cudaMemcpyDefault, ctx().stream));
    ctx().sync();
  });
  if (rc == OHG_OK && !ok) {
    g_err = std::string("unknown mesh array ") + name;
    return OHG_ERR_INVALID;
  }
  if (rc == OHG_OK && !fits) {
    g_err = std::string("destination too small for ") + name;
    return OHG_ERR_BOUNDS;
  }
  return rc;
}
int ohg_mesh_get_arrays(ohg_mesh* m, int n, const char* const* names, void* const* dsts,
                        const long long* caps) {
  MESH_GUARD(m);
  if (n < 0 || (n > 0 && (!names || !dsts || !caps))) {
    g_err = "ohg_mesh_get_arrays: bad arguments";
    return OHG_ERR_INVALID;
  }
  std::string bad;
  int bad_rc = OHG_OK;
  int rc = guarded(m->owner, [&] {
    std::vector<Arr<GO>> tmps(static_cast<size_t>(n));
    std::vector<const void*> ps(static_cast<size_t>(n));
    std::vector<long long> bs(static_cast<size_t>(n));
    for (int i = 0; i < n && bad_rc == OHG_OK; ++i) {
      if (!names[i] || !named_array(m->mesh, names[i], &ps[i], &bs[i], &tmps[i])) {
        bad = std::string("unknown mesh array ") + (names[i] ? names[i] : "(null)");
        bad_rc = OHG_ERR_INVALID;
      } else if (bs[i] > caps[i]) {
        bad = std::string("destination too small for ") + names[i];
        bad_rc = OHG_ERR_BOUNDS;
      }
    }
    if (bad_rc != OHG_OK) return;
    // every copy queued on the context's stream, one wait for all of them
    for (int i = 0; i < n; ++i)
      if (bs[i])
        OHG_CUDA(cudaMemcpyAsync(dsts[i], ps[i], size_t(bs[i]), cudaMemcpyDefault, ctx().stream));
    ctx().sync();
  });
  if (rc == OHG_OK && bad_rc != OHG_OK) {
    g_err = bad;
    return bad_rc;
  }
  return rc;
}
int ohg_mesh_set_array(ohg_mesh* m, const char* name, const void* src, long long nbytes) {
  MESH_GUARD(m);
  std::string n(name);
  Mesh& me = m->mesh;
  Arr<double>* dst = n == "coords" ? &me.coords : n == "metric" ? &me.metric : nullptr;
  if (!dst) {
    g_err = "only coords and metric can be set";
    return OHG_ERR_INVALID;
  }
  // a metric of one value per vertex is isotropic; of the packed tensor's
  // size, anisotropic
  long long full = (long long)me.nverts() * (me.dim == 3 ? 6 : 3) * 8LL;
  long long iso = (long long)me.nverts() * 8LL;
  bool ok = n == "metric" ? (nbytes == full || nbytes == iso) : nbytes == dst->size() * 8LL;
  if (!ok) {
    g_err = "size mismatch for " + n;
    return OHG_ERR_BOUNDS;
  }
  return guarded(m->owner, [&] {
    if (n == "metric") me.metric_comps = (nbytes == iso && nbytes != full) ? 1 : 0;
    Arr<double> a(LO(nbytes / 8));
    // device or host memory: the copy kind is inferred from the address
    OHG_CUDA(cudaMemcpyAsync(a.data(), src, size_t(nbytes), cudaMemcpyDefault, ctx().stream));
    ctx().sync();
    *dst = a;
    me.has_length = me.has_quality = false;
    me.screen.reset();
  });
}

static AdaptOpts to_opts(int dim, const ohg_adapt_opts* o) {
  AdaptOpts a(dim);
  if (o) {
    a.min_length_desired = o->min_length_desired;
    a.max_length_desired = o->max_length_desired;
    a.max_length_allowed = o->max_length_allowed;
    a.min_quality_allowed = o->min_quality_allowed;
    a.min_quality_desired = o->min_quality_desired;
    a.nsliver_layers = o->nsliver_layers;
  }
  return a;
}

int ohg_adapt_opts_default(int dim, ohg_adapt_opts* out) {
  if (dim != 2 && dim != 3) return OHG_ERR_INVALID;
  AdaptOpts a(dim);
  out->min_length_desired = a.min_length_desired;
  out->max_length_desired = a.max_length_desired;
  out->max_length_allowed = a.max_length_allowed;
  out->min_quality_allowed = a.min_quality_allowed;
  out->min_quality_desired = a.min_quality_desired;
  out->nsliver_layers = a.nsliver_layers;
  return OHG_OK;
}

static void to_stats(const PassStats& s, ohg_pass_stats* out) {
  if (!out) return;
  out->did_refine = s.did_refine;
  out->did_coarsen = s.did_coarsen;
  out->did_swap = s.did_swap;
  out->nelems_in = s.nelems_in;
  out->nelems_out = s.nelems_out;
  out->refine_keys = s.refine_keys;
  out->coarsen_keys = s.coarsen_keys;
  out->swap_keys = s.swap_keys;
  out->indset_rounds = s.indset_rounds;
  out->min_quality = s.min_quality;
  out->ms_refine = s.ms_refine;
  out->ms_coarsen = s.ms_coarsen;
  out->ms_swap = s.ms_swap;
}
int ohg_adapt_pass(ohg_mesh* m, const ohg_adapt_opts* o, ohg_pass_stats* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { to_stats(adapt_pass(m->mesh, to_opts(m->mesh.dim, o)), out); });
}
int ohg_adapt(ohg_mesh* m, const ohg_adapt_opts* o, ohg_adapt_result* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    AdaptResult r = adapt(m->mesh, to_opts(m->mesh.dim, o));
    if (out) {
      out->did = r.did;
      out->quality_satisfied = r.quality_satisfied;
      out->refines = r.refines;
      out->coarsens = r.coarsens;
      out->swaps = r.swaps;
      out->sliver_coarsens = r.sliver_coarsens;
      out->length_rounds = r.length_rounds;
    }
  });
}
int ohg_coarsen_slivers(ohg_mesh* m, const ohg_adapt_opts* o, int* did) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    PassStats s;
    bool d = coarsen_slivers(m->mesh, to_opts(m->mesh.dim, o), &s);
    if (did) *did = d;
  });
}
static int batch_args(ohg_context* c, ohg_mesh* const* ms, int n) {
  if (!c || !ms || n <= 0) {
    g_err = "batch: null context or no meshes";
    return OHG_ERR_INVALID;
  }
  for (int i = 0; i < n; ++i)
    if (!ms[i] || ms[i]->owner != c) {
      g_err = "batch: a null mesh or a mesh of another context";
      return OHG_ERR_INVALID;
    }
  return OHG_OK;
}
int ohg_mesh_concat(ohg_context* c, ohg_mesh* const* ms, int n, ohg_mesh** out) {
  int rc = batch_args(c, ms, n);
  if (rc) return rc;
  ohg_mesh* u = new ohg_mesh{c, Mesh()};
  rc = guarded(c, [&] {
    std::vector<Mesh*> v;
    for (int i = 0; i < n; ++i) v.push_back(&ms[i]->mesh);
    u->mesh = concat_meshes(v);
  });
  if (rc != OHG_OK) {
    delete u;
    return rc;
  }
  *out = u;
  return OHG_OK;
}
int ohg_mesh_split(ohg_mesh* u, int n, ohg_mesh** outs) {
  MESH_GUARD(u);
  if (n <= 0 || !outs) return OHG_ERR_INVALID;
  std::vector<Mesh> parts;
  int rc = guarded(u->owner, [&] { parts = split_mesh(u->mesh, n); });
  if (rc != OHG_OK) return rc;
  for (int i = 0; i < n; ++i) outs[i] = new ohg_mesh{u->owner, std::move(parts[i])};
  return OHG_OK;
}
int ohg_adapt_pass_batch(ohg_context* c, ohg_mesh* const* ms, int n, const ohg_adapt_opts* o,
                         ohg_pass_stats* out) {
  int rc = batch_args(c, ms, n);
  if (rc) return rc;
  return guarded(c, [&] {
    std::vector<Mesh*> v;
    for (int i = 0; i < n; ++i) v.push_back(&ms[i]->mesh);
    Mesh u = concat_meshes(v);
    to_stats(adapt_pass(u, to_opts(u.dim, o)), out);
    std::vector<Mesh> parts = split_mesh(u, n);
    for (int i = 0; i < n; ++i) ms[i]->mesh = std::move(parts[i]);
  });
}
int ohg_refine_by_size(ohg_mesh* m, const ohg_adapt_opts* o, int* did) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    PassStats s;
    *did = refine_by_size(m->mesh, to_opts(m->mesh.dim, o), &s);
  });
}
int ohg_coarsen_by_size(ohg_mesh* m, const ohg_adapt_opts* o, int* did) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    PassStats s;
    *did = coarsen_by_size(m->mesh, to_opts(m->mesh.dim, o), &s);
  });
}
int ohg_swap_edges(ohg_mesh* m, const ohg_adapt_opts* o, int* did) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    PassStats s;
    *did = swap_edges(m->mesh, to_opts(m->mesh.dim, o), &s);
  });
}

int ohg_measure_edges_metric(ohg_mesh* m, const int* a2e, int n, double* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { measure_edges_metric(m->mesh, a2e, n, out); });
}
int ohg_measure_qualities(ohg_mesh* m, const int* a2e, int n, double* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { measure_qualities(m->mesh, a2e, n, out); });
}
int ohg_screen_tet_qualities(ohg_mesh* m, const int* tv2v, int n, float* lo, float* hi,
                             double* exact) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { screen_tets(m->mesh, tv2v, n, lo, hi, exact); });
}
int ohg_screen_tet_qualities_face(ohg_mesh* m, const int* tv2v, int n, int slot, int cubed,
                                  float* lo, float* hi, double* exact) {
  MESH_GUARD(m);
  if (n < 0 || slot < 0 || slot > 3) return OHG_ERR_INVALID;
  return guarded(m->owner,
                 [&] { screen_tets_face(m->mesh, tv2v, n, slot, cubed != 0, lo, hi, exact); });
}
int ohg_screen_edge_lengths(ohg_mesh* m, const int* ev2v, int n, float* lo, float* hi,
                            double* exact) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { screen_edges(m->mesh, ev2v, n, lo, hi, exact); });
}
int ohg_get_mident_metrics(ohg_mesh* m, const int* e, int n, double* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { mident_metrics(m->mesh, e, n, out); });
}
int ohg_refine_qualities(ohg_mesh* m, const int* c2e, int n, double* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    Arr<double> mid(n * m->mesh.mcomp());
    mident_metrics(m->mesh, c2e, n, mid.data());
    refine_qualities(m->mesh, c2e, n, mid.data(), out);
  });
}
int ohg_check_collapse_class(ohg_mesh* m, const int* c2e, int n, const signed char* ci,
                             signed char* co) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { check_collapse_class(m->mesh, c2e, n, ci, co); });
}
int ohg_check_collapse_exposure(ohg_mesh* m, const int* c2e, int n, const signed char* ci,
                                signed char* co) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { check_collapse_exposure(m->mesh, c2e, n, ci, co); });
}
int ohg_prevent_coarsen_overshoot(ohg_mesh* m, double ml, const int* c2e, int n,
                                  const signed char* ci, signed char* co) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { prevent_coarsen_overshoot(m->mesh, ml, c2e, n, ci, co); });
}
int ohg_coarsen_qualities(ohg_mesh* m, const int* c2e, int n, const signed char* codes,
                          double* out2) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] { coarsen_qualities(m->mesh, c2e, n, codes, out2); });
}
int ohg_choose_rails(ohg_mesh* m, const int* c2e, int n, const signed char* codes,
                     const double* q2, signed char* vc, double* vq, long long* vr) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    choose_rails(m->mesh, c2e, n, codes, q2, vc, vq, reinterpret_cast<GO*>(vr));
  });
}
int ohg_mark_sliver_layers(ohg_mesh* m, double ceil, int nlayers, signed char* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    Arr<I8> a = mark_sliver_layers(m->mesh, ceil, nlayers);
    OHG_CUDA(cudaMemcpyAsync(out, a.data(), size_t(a.size()), cudaMemcpyDeviceToDevice, ctx().stream));
  });
}
int ohg_swap2d_qualities(ohg_mesh* m, double ml, const int* c2e, int n, double* q) {
  MESH_GUARD(m);
  if (m->mesh.dim != 2) return OHG_ERR_INVALID;
  return guarded(m->owner, [&] { swap2d_qualities(m->mesh, ml, c2e, n, q); });
}
int ohg_swap3d_qualities(ohg_mesh* m, double ml, const int* c2e, int n, double* q, signed char* cf) {
  MESH_GUARD(m);
  if (m->mesh.dim != 3) return OHG_ERR_INVALID;
  return guarded(m->owner, [&] { swap3d_qualities(m->mesh, ml, c2e, n, q, cf); });
}
int ohg_swap3d_find_loops(ohg_mesh* m, const int* edges, int n, int* sizes, int* eev2v,
                          int* loop_verts) {
  MESH_GUARD(m);
  if (m->mesh.dim != 3 || n < 0 || (n > 0 && (!edges || !sizes || !eev2v || !loop_verts))) {
    g_err = "ohg_swap3d_find_loops: needs a 3D mesh, n >= 0 and non-null arrays";
    return OHG_ERR_INVALID;
  }
  return guarded(m->owner, [&] { swap3d_find_loops(m->mesh, edges, n, sizes, eev2v, loop_verts); });
}
int ohg_find_indset(ohg_mesh* m, int d, const double* q, const signed char* cands,
                    signed char* out, int* rounds) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    LO n = m->mesh.nents[d];
    Ctx& x = ctx();
    OHG_CUDA(cudaMemsetAsync(x.d_indset_sweeps, 0, sizeof(int), x.stream));
    Arr<I8> res = find_indset(m->mesh, d, Arr<double>::wrap(const_cast<double*>(q), n),
                              Arr<I8>::wrap(const_cast<I8*>(cands), n));
    OHG_CUDA(cudaMemcpyAsync(out, res.data(), size_t(n), cudaMemcpyDeviceToDevice, x.stream));
    OHG_CUDA(cudaMemcpyAsync(x.h_indset_sweeps, x.d_indset_sweeps, sizeof(int),
                             cudaMemcpyDeviceToHost, x.stream));
    x.sync();
    if (rounds) *rounds = d == m->mesh.dim ? 0 : *x.h_indset_sweeps;
  });
}

int ohg_fp64_peak(ohg_context* c, int reps, double* gflops) {
  if (!gflops || reps < 1) {
    g_err = "ohg_fp64_peak: reps >= 1 and an output are needed";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] { *gflops = fp64_peak_gflops(reps); });
}
int ohg_time_stage(ohg_mesh* m, const char* stage, int reps, float* avg_ms, double* alg_bytes) {
  MESH_GUARD(m);
  std::string st(stage ? stage : "");
  return guarded(m->owner, [&] {
    Mesh& me = m->mesh;
    int dim = me.dim;
    LO E = me.nedges(), V = me.nverts(), T = me.nelems();
    int mc = me.mcomp();
    Arr<LO> all_e = iota(E);
    Arr<double> out;
    Arr<double> mid;
    Arr<I8> codes;
    double b = 0;
    std::function<void()> launch;
    if (st == "lengths") {
      out = Arr<double>(E);
      me.ask_verts_of(1);
      b = E * (8.0 + 8.0) + V * (8.0 * dim + 8.0 * mc);
      launch = [&] { measure_edges_metric(me, nullptr, E, out.data()); };
    } else if (st == "qualities") {
      out = Arr<double>(T);
      me.ask_verts_of(dim);
      b = T * (4.0 * (dim + 1) + 8.0) + V * (8.0 * dim + 8.0 * mc);
      launch = [&] { measure_qualities(me, nullptr, T, out.data()); };
    } else if (st == "refine_qualities") {
      out = Arr<double>(E);
      mid = Arr<double>(E * mc);
      mident_metrics(me, all_e.data(), E, mid.data());
      const Adj& e2c = me.ask_up(1, dim);
      me.ask_verts_of(dim);
      b = E * (4.0 + 8.0 + 8.0 * mc + 8.0) + (E + 1) * 4.0 + e2c.ab2b.size() * 5.0 +
          T * 4.0 * (dim + 1) + V * (8.0 * dim + 8.0 * mc);
      launch = [&] { refine_qualities(me, all_e.data(), E, mid.data(), out.data()); };
    } else if (st == "coarsen_qualities") {
      out = Arr<double>(E * 2);
      codes = fill<I8>(E, 3);
      const Adj& v2c = me.ask_up(0, dim);
      me.ask_verts_of(dim);
      b = E * (4.0 + 1.0 + 8.0 + 16.0) + (V + 1) * 4.0 + v2c.ab2b.size() * 5.0 +
          T * 4.0 * (dim + 1) + V * (8.0 * dim + 8.0 * mc);
      launch = [&] { coarsen_qualities(me, all_e.data(), E, codes.data(), out.data()); };
    } else {
      throw Error(OHG_ERR_INVALID, "unknown stage " + st);
    }
    Ctx& c = ctx();
    launch();
    Arr<char> flush(256 << 20);
    cudaEvent_t e0, e1;
    OHG_CUDA(cudaEventCreate(&e0));
    OHG_CUDA(cudaEventCreate(&e1));
    double total = 0;
    for (int r = 0; r < reps; ++r) {
      OHG_CUDA(cudaMemsetAsync(flush.data(), r & 0xff, size_t(256) << 20, c.stream));
      OHG_CUDA(cudaEventRecord(e0, c.stream));
      launch();
      OHG_CUDA(cudaEventRecord(e1, c.stream));
      OHG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      OHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *avg_ms = float(total / (reps > 0 ? reps : 1));
    *alg_bytes = b;
  });
}

int ohg_invert_adj(ohg_context* c, const int* hl2l, const signed char* codes, int nhigh, int k,
                   int nlows, int* a2ab, int* ab2b, signed char* codes_out) {
  return guarded(c, [&] {
    Adj down;
    down.ab2b = Arr<LO>::wrap(const_cast<LO*>(hl2l), nhigh * k);
    if (codes) {
      down.codes = Arr<I8>::wrap(const_cast<I8*>(codes), nhigh * k);
      down.has_codes = true;
    }
    Adj up = invert_adj(down, k, nlows);
    Ctx& cc = ctx();
    OHG_CUDA(cudaMemcpyAsync(a2ab, up.a2ab.data(), size_t(nlows + 1) * 4, cudaMemcpyDeviceToDevice, cc.stream));
    OHG_CUDA(cudaMemcpyAsync(ab2b, up.ab2b.data(), size_t(nhigh) * k * 4, cudaMemcpyDeviceToDevice, cc.stream));
    OHG_CUDA(cudaMemcpyAsync(codes_out, up.codes.data(), size_t(nhigh) * k, cudaMemcpyDeviceToDevice, cc.stream));
  });
}
int ohg_reflect_down(ohg_context* c, const int* hv2v, int nhigh, int hd, int ld, const int* lv2v,
                     int nlows, const int* va, const int* vb, const signed char* vc, int nverts,
                     int* hl2l, signed char* codes_out) {
  return guarded(c, [&] {
    Adj v2l;
    v2l.a2ab = Arr<LO>::wrap(const_cast<LO*>(va), nverts + 1);
    LO nvl = nlows * (ld + 1);
    v2l.ab2b = Arr<LO>::wrap(const_cast<LO*>(vb), nvl);
    v2l.codes = Arr<I8>::wrap(const_cast<I8*>(vc), nvl);
    Adj r = reflect_down(Arr<LO>::wrap(const_cast<LO*>(hv2v), nhigh * (hd + 1)), nhigh,
                         Arr<LO>::wrap(const_cast<LO*>(lv2v), nvl), v2l, hd, ld,
                         /*check_unique=*/true);
    LO na = nhigh * simplex_degree(hd, ld);
    OHG_CUDA(cudaMemcpyAsync(hl2l, r.ab2b.data(), size_t(na) * 4, cudaMemcpyDeviceToDevice, ctx().stream));
    if (codes_out && ld > 0)
      OHG_CUDA(cudaMemcpyAsync(codes_out, r.codes.data(), size_t(na), cudaMemcpyDeviceToDevice, ctx().stream));
  });
}
int ohg_find_indset_graph(ohg_context* c, int n, const int* xa, const int* xb, const double* q,
                          const signed char* cands, signed char* out, int* rounds) {
  return guarded(c, [&] {
    Adj g;
    g.a2ab = Arr<LO>::wrap(const_cast<LO*>(xa), n + 1);
    g.ab2b = Arr<LO>::wrap(const_cast<LO*>(xb), 0);
    Ctx& x = ctx();
    OHG_CUDA(cudaMemsetAsync(x.d_indset_sweeps, 0, sizeof(int), x.stream));
    Arr<I8> res = find_indset(g, n, Arr<double>::wrap(const_cast<double*>(q), n),
                              Arr<I8>::wrap(const_cast<I8*>(cands), n));
    OHG_CUDA(cudaMemcpyAsync(out, res.data(), size_t(n), cudaMemcpyDeviceToDevice, x.stream));
    OHG_CUDA(cudaMemcpyAsync(x.h_indset_sweeps, x.d_indset_sweeps, sizeof(int),
                             cudaMemcpyDeviceToHost, x.stream));
    x.sync();
    if (rounds) *rounds = *x.h_indset_sweeps;
  });
}
int ohg_sort_by_keys(ohg_context* c, const void* keys, int n, int width, int kb, int* perm) {
  if (width < 1 || width > 4 || (kb != 4 && kb != 8)) return OHG_ERR_INVALID;
  return guarded(c, [&] {
    Arr<LO> p = kb == 4 ? sort_by_keys(Arr<LO>::wrap((LO*)keys, n * width), width)
                        : sort_by_keys64(Arr<GO>::wrap((GO*)keys, n * width), width);
    OHG_CUDA(cudaMemcpyAsync(perm, p.data(), size_t(n) * 4, cudaMemcpyDeviceToDevice, ctx().stream));
  });
}
int ohg_hilbert_sort(ohg_context* c, const double* coords, int n, int dim, int* perm) {
  return guarded(c, [&] {
    Arr<LO> p = hilbert_sort(Arr<double>::wrap(const_cast<double*>(coords), n * dim), n, dim);
    OHG_CUDA(cudaMemcpyAsync(perm, p.data(), size_t(n) * 4, cudaMemcpyDeviceToDevice, ctx().stream));
  });
}
int ohg_hilbert_transpose(ohg_context* c, const unsigned long long* axes, int n, int dim, int bits,
                          unsigned long long* keys) {
  if (n < 0 || dim < 1 || dim > 3 || bits < 1 || bits > 64 || (n > 0 && (!axes || !keys))) {
    g_err = "ohg_hilbert_transpose: bad arguments";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    hilbert_transpose_keys(reinterpret_cast<const std::uint64_t*>(axes), n, dim, bits,
                           reinterpret_cast<std::uint64_t*>(keys));
  });
}
int ohg_offset_scan(ohg_context* c, const int* counts, int n, int* out) {
  return guarded(c, [&] { offset_scan_into(counts, n, out); });
}
int ohg_collect_marked(ohg_context* c, const signed char* marks, int n, int* out, int* count) {
  if (n < 0 || !count || (n > 0 && (!marks || !out))) {
    g_err = "ohg_collect_marked: bad arguments";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] {
    Arr<LO> r = collect_marked(Arr<I8>::wrap(const_cast<I8*>(marks), n));
    if (r.size())
      OHG_CUDA(cudaMemcpyAsync(out, r.data(), size_t(r.size()) * sizeof(LO),
                               cudaMemcpyDeviceToDevice, ctx().stream));
    *count = r.size();
  });
}
int ohg_selftest_scan_wait_limit(ohg_context* c, const int* counts, int n, int* out) {
  return guarded(c, [&] { scan_wait_limit_selftest(counts, n, out); });
}
int ohg_offset_scan_noalloc(ohg_context* c, const int* counts, int n, int* out) {
  return guarded(c, [&] { offset_scan_fixed_scratch(counts, n, out); });
}
int ohg_offset_scan_noalloc_limit(int* out) {
  if (!out) {
    g_err = "null output";
    return OHG_ERR_INVALID;
  }
  *out = offset_scan_fixed_limit();
  return OHG_OK;
}


// ------------------------------------------------------------ metric tools
static bool metric_args(int dim, int n) {
  if ((dim != 2 && dim != 3) || n < 0) {
    g_err = "metric tools: dim must be 2 or 3 and n >= 0";
    return false;
  }
  return true;
}
int ohg_cubic_roots(ohg_context* c, int n, const double* coeffs, double eps, int* nroots,
                    double* roots, int* mults) {
  if (n < 0 || (n > 0 && (!coeffs || !nroots || !roots || !mults)) || !(eps >= 0.0)) {
    g_err = "ohg_cubic_roots: bad arguments";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] { cubic_roots_batch(n, coeffs, eps, nroots, roots, mults); });
}
int ohg_decompose_eigen(ohg_context* c, int dim, int n, const double* m, double* q, double* l) {
  if ((dim != 2 && dim != 3) || n < 0 || (n > 0 && (!m || !q || !l))) {
    g_err = "ohg_decompose_eigen: dim must be 2 or 3, with n >= 0 and non-null arrays";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] { decompose_eigen_batch(dim, n, m, q, l); });
}
int ohg_intersect_metrics(ohg_context* c, int dim, int n, const double* a, const double* b,
                          double* out) {
  if (!metric_args(dim, n)) return OHG_ERR_INVALID;
  return guarded(c, [&] { intersect_metrics(dim, n, a, b, out); });
}
int ohg_clamp_metrics(ohg_context* c, int dim, int n, const double* m, double h_min, double h_max,
                      double* out) {
  if (!metric_args(dim, n)) return OHG_ERR_INVALID;
  if (!(h_min > 0.0) || !(h_min <= h_max)) {
    g_err = "ohg_clamp_metrics: need 0 < h_min <= h_max";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] { clamp_metrics(dim, n, m, h_min, h_max, out); });
}
int ohg_hessian_metrics(ohg_context* c, int dim, int n, const double* h, double eps, double* out) {
  if (!metric_args(dim, n) || !(eps > 0.0)) {
    g_err = "ohg_hessian_metrics: dim 2 or 3 and eps > 0";
    return OHG_ERR_INVALID;
  }
  return guarded(c, [&] { hessian_metrics(dim, n, h, eps, out); });
}
int ohg_mesh_implied_metrics(ohg_mesh* m, double* out) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    Arr<double> r = implied_metrics(m->mesh);
    OHG_CUDA(cudaMemcpyAsync(out, r.data(), sizeof(double) * size_t(r.size()),
                             cudaMemcpyDeviceToDevice, ctx().stream));
  });
}
int ohg_mesh_limit_metric_gradation(ohg_mesh* m, const double* metrics, double max_rate, double tol,
                                    double* out, int* steps) {
  MESH_GUARD(m);
  return guarded(m->owner, [&] {
    Mesh& me = m->mesh;
    LO n = me.nverts() * me.mcomp();
    Arr<double> in(n);
    OHG_CUDA(cudaMemcpyAsync(in.data(), metrics, sizeof(double) * size_t(n),
                             cudaMemcpyDeviceToDevice, ctx().stream));
    Arr<double> r = limit_metric_gradation(me, in, max_rate, tol, steps);
    OHG_CUDA(cudaMemcpyAsync(out, r.data(), sizeof(double) * size_t(n), cudaMemcpyDeviceToDevice,
                             ctx().stream));
  });
}
int ohg_mesh_expected_nelems(ohg_mesh* m, const double* metrics, double* out) {
  MESH_GUARD(m);
  if (!out) return OHG_ERR_INVALID;
  return guarded(m->owner, [&] { *out = expected_nelems(m->mesh, metrics); });
}
int ohg_metric_input_default(ohg_metric_input* o) {
  if (!o) return OHG_ERR_INVALID;
  MetricInput d;
  *o = ohg_metric_input{};
  o->nsources = 0;
  o->should_limit_lengths = d.limit_lengths;
  o->min_length = d.min_length;
  o->max_length = d.max_length;
  o->should_limit_gradation = d.limit_gradation;
  o->max_gradation_rate = d.max_gradation_rate;
  o->gradation_convergence_tolerance = d.gradation_tol;
  o->should_limit_element_count = d.limit_element_count;
  o->max_element_count = d.max_element_count;
  o->min_element_count = d.min_element_count;
  o->element_count_over_relaxation = d.element_count_over_relaxation;
  o->nsmoothing_steps = d.nsmoothing_steps;
  return OHG_OK;
}
int ohg_mesh_generate_metrics(ohg_mesh* m, const ohg_metric_input* in, double* out, int* niters) {
  MESH_GUARD(m);
  if (!in || !out || in->nsources < 0 || in->nsources > 8) {
    g_err = "ohg_mesh_generate_metrics: null input or output, or more than 8 sources";
    return OHG_ERR_INVALID;
  }
  return guarded(m->owner, [&] {
    MetricInput mi;
    for (int i = 0; i < in->nsources; ++i) {
      const ohg_metric_source& s = in->sources[i];
      mi.sources.push_back({s.type, s.knob, s.isotropy, s.scales, s.given});
    }
    mi.limit_lengths = in->should_limit_lengths != 0;
    mi.min_length = in->min_length;
    mi.max_length = in->max_length;
    mi.limit_gradation = in->should_limit_gradation != 0;
    mi.max_gradation_rate = in->max_gradation_rate;
    mi.gradation_tol = in->gradation_convergence_tolerance;
    mi.limit_element_count = in->should_limit_element_count != 0;
    mi.max_element_count = in->max_element_count;
    mi.min_element_count = in->min_element_count;
    mi.element_count_over_relaxation = in->element_count_over_relaxation;
    mi.nsmoothing_steps = in->nsmoothing_steps;
    Arr<double> r = generate_metrics(m->mesh, mi, niters);
    OHG_CUDA(cudaMemcpyAsync(out, r.data(), sizeof(double) * size_t(r.size()),
                             cudaMemcpyDeviceToDevice, ctx().stream));
  });
}

}  // extern "C"
