// Scan, compaction, reduction and radix-sort kernels.
#include <cfloat>
#include <chrono>
#include <cstdlib>
#include <mutex>

#include "ohg_prims.cuh"

namespace ohg {

// ------------------------------------------------------------ runtime
void cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", int(e),
                cudaGetErrorString(e), what, file, line);
  throw Error(e == cudaErrorMemoryAllocation ? 6 : 1, buf);
}

static thread_local Ctx* g_ctx = nullptr;
Ctx& ctx() {
  if (!g_ctx) throw Error(8, "no current ohg context");
  return *g_ctx;
}
void set_ctx(Ctx* c) { g_ctx = c; }

Ctx::Ctx(int dev) : device(dev) {
  OHG_CUDA(cudaSetDevice(dev));
  OHG_CUDA(cudaStreamCreate(&stream));  // blocking: ordered with the legacy default stream
  cache->stream = stream;
  OHG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  OHG_CUDA(cudaMalloc(&d_status, sizeof(int)));
  OHG_CUDA(cudaMemset(d_status, 0, sizeof(int)));
  OHG_CUDA(cudaMallocHost(&h_pinned, kPinnedInts * sizeof(int)));
  OHG_CUDA(cudaMalloc(&d_screen_counts, 4 * sizeof(unsigned long long)));
  OHG_CUDA(cudaMemset(d_screen_counts, 0, 4 * sizeof(unsigned long long)));
  OHG_CUDA(cudaMalloc(&d_indset_sweeps, sizeof(int)));
  OHG_CUDA(cudaMemset(d_indset_sweeps, 0, sizeof(int)));
  OHG_CUDA(cudaMallocHost(&h_indset_sweeps, sizeof(int)));
  OHG_CUDA(cudaMallocHost(&h_pass_min, sizeof(double)));
  cudaMemPool_t pool;
  OHG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  std::uint64_t thr = ~std::uint64_t(0);
  OHG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  const char* tr = std::getenv("OHG_TRACE_SYNCS");
  trace_syncs = tr && *tr && *tr != '0';
}
Ctx::~Ctx() {
  cudaStreamSynchronize(stream);
  cache->release();
  {
    std::lock_guard<std::mutex> g(cache->mu);
    cache->open = false;  // arrays that outlive the context free to the pool
  }
  cudaStreamSynchronize(stream);
  if (trace_syncs) {
    std::fprintf(stderr, "ohg: host waits by call site (%llu in all)\n",
                 (unsigned long long)syncs);
    for (auto& kv : sync_sites)
      std::fprintf(stderr, "ohg:   %s:%d %llu (%.3f ms blocked, %.3f ms issuing %llu launches before)\n",
                   kv.first.first.c_str(), kv.first.second, (unsigned long long)kv.second,
                   double(sync_wait_ns[kv.first]) * 1e-6, double(sync_issue_ns[kv.first]) * 1e-6,
                   (unsigned long long)sync_issue_launches[kv.first]);
  }
  tuner.release();
  for (auto& k : kernel_launches) {
    cudaEventDestroy(k.start);
    cudaEventDestroy(k.stop);
  }
  cudaFree(d_status);
  cudaFree(d_screen_counts);
  cudaFree(d_indset_sweeps);
  cudaFreeHost(h_indset_sweeps);
  cudaFreeHost(h_pass_min);
  if (d_swap_tables) cudaFree(d_swap_tables);
  cudaFreeHost(h_pinned);
  cudaStreamDestroy(stream);
}
void Ctx::sync(const char* file, int line) {
  ++syncs;
  if (trace_syncs) {
    ++sync_sites[{file, line}];
    auto ns = [] {
      return std::int64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(
                              std::chrono::steady_clock::now().time_since_epoch())
                              .count());
    };
    std::int64_t t0 = ns();
    if (trace_last_ns >= 0) {
      sync_issue_ns[{file, line}] += std::uint64_t(t0 - trace_last_ns);
      sync_issue_launches[{file, line}] += launches - trace_last_launches;
    }
    OHG_CUDA(cudaStreamSynchronize(stream));
    trace_last_ns = ns();
    trace_last_launches = launches;
    sync_wait_ns[{file, line}] += std::uint64_t(trace_last_ns - t0);
  } else {
    OHG_CUDA(cudaStreamSynchronize(stream));
  }
  if (!tuner.pending.empty()) tuner.resolve();
}

// ------------------------------------------------------------ autotuner
int Tuner::select(const char* name, int line, long long n, int nvar, int dflt, cudaStream_t s) {
  open = -1;
  if (nvar <= 1) return 0;
  if (forced >= 0) return forced % nvar;
  if (mode == OFF) return dflt;
  int bucket = 0;
  while ((2LL << bucket) <= n) ++bucket;
  std::uint64_t key = std::uint64_t(reinterpret_cast<std::uintptr_t>(name)) * 0x9E3779B97F4A7C15ULL ^
                      (std::uint64_t(line) << 8) ^ std::uint64_t(bucket);
  Site& st = sites[key];
  if (st.nvar == 0) {
    st.name = name;
    st.line = line;
    st.bucket = bucket;
    st.nvar = nvar;
    st.dflt = dflt;
    st.best.assign(nvar, -1.0f);
    st.launched.assign(nvar, 0);
  }
  int seen = st.seen++;
  if (st.chosen >= 0) return st.chosen;
  if (mode != EXPLORE) {
    // frozen: the fastest variant timed so far, else the default
    int b = -1;
    for (int v = 0; v < nvar; ++v)
      if (st.best[v] >= 0.0f && (b < 0 || st.best[v] < st.best[b])) b = v;
    return b >= 0 ? b : dflt;
  }
  // the site's first launch is not timed (it may load the kernel); then
  // each variant once
  if (seen == 0) return dflt;
  int v = -1;
  for (int k = 0; k < nvar; ++k) {
    int c = (dflt + k) % nvar;
    if (!st.launched[c]) {
      v = c;
      break;
    }
  }
  if (v < 0) return dflt;  // all timed, waiting for the events
  st.launched[v] = 1;
  Pending p{&st, v, nullptr, nullptr};
  for (cudaEvent_t* e : {&p.a, &p.b}) {
    if (!spare.empty()) {
      *e = spare.back();
      spare.pop_back();
    } else {
      OHG_CUDA(cudaEventCreate(e));
    }
  }
  OHG_CUDA(cudaEventRecord(p.a, s));
  pending.push_back(p);
  open = int(pending.size()) - 1;
  return v;
}

void Tuner::stop(cudaStream_t s) {
  if (open >= 0) OHG_CUDA(cudaEventRecord(pending[open].b, s));
  open = -1;
}

void Tuner::resolve() {
  for (Pending& p : pending) {
    float ms = -1.0f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) != cudaSuccess) {
      cudaGetLastError();
      ms = -1.0f;
    }
    Site& st = *p.site;
    if (ms >= 0.0f && (st.best[p.var] < 0.0f || ms < st.best[p.var])) st.best[p.var] = ms;
    spare.push_back(p.a);
    spare.push_back(p.b);
    bool all = true;
    int b = 0;
    for (int v = 0; v < st.nvar; ++v) {
      if (st.best[v] < 0.0f) all = false;
      else if (st.best[v] < st.best[b] || st.best[b] < 0.0f) b = v;
    }
    if (all) st.chosen = b;
  }
  pending.clear();
}

void Tuner::release() {
  for (Pending& p : pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  pending.clear();
  for (cudaEvent_t e : spare) cudaEventDestroy(e);
  spare.clear();
}
int Ctx::take_status() {
  OHG_CUDA(cudaMemcpyAsync(h_pinned, d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  OHG_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), stream));
  sync();
  return h_pinned[0];
}

// size classes: multiples of 512 bytes up to 4 KiB, then four classes per
// power of two (at most a quarter over the request)
static size_t size_class(size_t b) {
  if (b <= 4096) return (b + 511) & ~size_t(511);
  size_t p = size_t(1) << (63 - __builtin_clzll((unsigned long long)b));
  size_t step = p / 4;
  return (b + step - 1) / step * step;
}
void* DevCache::take(size_t cls) {
  std::lock_guard<std::mutex> g(mu);
  auto it = lists.find(cls);
  if (it == lists.end() || it->second.empty()) return nullptr;
  void* p = it->second.back();
  it->second.pop_back();
  bytes -= cls;
  return p;
}
bool DevCache::put(void* p, size_t cls) {
  std::lock_guard<std::mutex> g(mu);
  if (!open || bytes + cls > cap) return false;
  lists[cls].push_back(p);
  bytes += cls;
  return true;
}
void DevCache::release() {
  std::lock_guard<std::mutex> g(mu);
  for (auto& kv : lists)
    for (void* p : kv.second) cudaFreeAsync(p, stream);
  lists.clear();
  bytes = 0;
}
void* dev_alloc(size_t& bytes) {
  Ctx& c = ctx();
  ++c.allocs;
  bytes = size_class(bytes);
  if (void* q = c.cache->take(bytes)) return q;
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, c.stream);
  if (e != cudaSuccess) {
    // the cached blocks back to the pool, then once more
    cudaGetLastError();
    c.cache->release();
    e = cudaMallocAsync(&p, bytes, c.stream);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(6, "device allocation of " + std::to_string(bytes) + " bytes failed");
  }
  return p;
}
Buf::~Buf() {
  if (!p) return;
  if (cache && cache->put(p, bytes)) return;
  cudaFreeAsync(p, stream);
}

// ------------------------------------------------------------ scan
// Three-phase exclusive scan: tile sums, scan of tile sums, tile scans.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__global__ void k_tile_sums(const T* in, LO n, LO* sums) {
  __shared__ LO warp_sums[kScanThreads / 32];
  LO base = LO(blockIdx.x) * kScanTile;
  LO s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    LO i = base + k * kScanThreads + threadIdx.x;
    if (i < n) s += LO(in[i]);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < kScanThreads / 32 ? warp_sums[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

// exclusive scan of one value per thread across a block of 1024 threads
// (warp shuffles, then a scan of the 32 warp totals); *block_total gets the sum
__device__ __forceinline__ LO block_exclusive_scan_1024(LO v, LO* block_total) {
  __shared__ LO wsum[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  LO incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    LO y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    LO w = wsum[lane];
    LO wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      LO y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    wsum[lane] = wi - w;
    if (lane == 31) *block_total = wi;
  }
  __syncthreads();
  return wsum[warp] + incl - v;
}

// single block of 1024 threads: exclusive scan of nb tile sums in place,
// total into *total
__global__ void k_scan_sums(LO* sums, LO nb, LO* total) {
  __shared__ LO tot;
  LO per = (nb + blockDim.x - 1) / blockDim.x;
  LO b0 = LO(threadIdx.x) * per;
  LO s = 0;
  for (LO k = 0; k < per; ++k)
    if (b0 + k < nb) s += sums[b0 + k];
  LO run = block_exclusive_scan_1024(s, &tot);
  if (threadIdx.x == 0) *total = tot;
  for (LO k = 0; k < per; ++k)
    if (b0 + k < nb) {
      LO v = sums[b0 + k];
      sums[b0 + k] = run;
      run += v;
    }
}

// one block of 1024 threads scans n <= kSmallScan counts directly
constexpr int kSmallScanItems = 4;
constexpr int kSmallScan = 1024 * kSmallScanItems;
template <class T>
__global__ void k_small_scan(const T* in, LO n, LO* out) {
  __shared__ LO tot;
  LO base = LO(threadIdx.x) * kSmallScanItems;
  LO v[kSmallScanItems];
  LO s = 0;
  for (int k = 0; k < kSmallScanItems; ++k) {
    v[k] = base + k < n ? LO(in[base + k]) : 0;
    s += v[k];
  }
  LO run = block_exclusive_scan_1024(s, &tot);
  for (int k = 0; k < kSmallScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) out[n] = tot;
}

template <class T>
__global__ void k_tile_scan(const T* in, LO n, const LO* sums, LO* out, const LO* total) {
  __shared__ LO warp_tot[kScanThreads / 32];
  LO base = LO(blockIdx.x) * kScanTile + LO(threadIdx.x) * kScanItems;
  LO v[kScanItems];
  LO s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    LO i = base + k;
    v[k] = i < n ? LO(in[i]) : 0;
    s += v[k];
  }
  // block-exclusive scan of thread sums
  LO incl = s;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    LO y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    LO w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    LO wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      LO y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;
  }
  __syncthreads();
  LO run = sums[blockIdx.x] + warp_tot[warp] + incl - s;
  for (int k = 0; k < kScanItems; ++k) {
    LO i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = *total;
}

// ------------------------------------------------------------ single-pass scan
// Exclusive scan in one launch by decoupled look-back (D. Merrill and
// M. Garland, "Single-pass Parallel Prefix Scan with Decoupled Look-back",
// NVIDIA technical report NVR-2016-002).  Each block takes the next tile
// number from a ticket counter, so every tile before it belongs to a block
// that is already running; it publishes its tile's sum (flag A), adds the
// published values of the tiles before it back to the first one that holds
// an inclusive prefix (flag P), then publishes its own inclusive prefix.  A
// status word packs the flag (bits 32-33) with the 32-bit value, so one
// 64-bit store publishes both.  Each item is read once and each offset
// written once: half the traffic of the tile-sums-then-scan form.
constexpr unsigned long long kTileAgg = 1ull << 32, kTilePre = 2ull << 32;
// polls of one predecessor's status word before the wait is given up
constexpr int kLookbackPolls = 1 << 20;

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// Exclusive prefix of tile t > 0, by the 32 lanes of one warp, each reading
// one predecessor's status word per step.  A predecessor that has published
// nothing after kLookbackPolls polls raises ST_STALL and counts as an
// inclusive prefix of 0, so the wait always ends (the host then reports the
// status as an error).
__device__ LO tile_lookback(const unsigned long long* st, LO t, int* status) {
  int lane = int(threadIdx.x & 31u);
  LO prefix = 0;
  for (LO top = t - 1;; top -= 32) {
    LO j = top - lane;
    unsigned long long w = kTilePre;  // before tile 0: an inclusive prefix of 0
    if (j >= 0) {
      w = ld_status(&st[j]);
      for (int poll = 0; (w >> 32) == 0; ++poll) {
        if (poll == kLookbackPolls) {
          raise_status(status, ST_STALL);
          w = kTilePre;
          break;
        }
        __nanosleep(32);
        w = ld_status(&st[j]);
      }
    }
    unsigned pre = __ballot_sync(0xffffffffu, (w >> 32) == 2);
    int stop = pre ? __ffs(pre) - 1 : 31;
    LO v = lane <= stop ? LO(unsigned(w)) : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    prefix += v;
    if (pre) return prefix;
  }
}

// One tile of kScanTile items per block.  kCompact = false: out[i] is the
// exclusive prefix of in[i] and out[n] the total.  kCompact = true: in holds
// marks; out (if not null) receives the indices of the nonzero ones in
// increasing order and *count their number.  st holds nb zeroed status
// words followed by the zeroed ticket counter.  vec: in (and out, for
// offsets) are 16-byte aligned, so whole tiles move as 16-byte vectors.
template <class T, bool kCompact>
__global__ void __launch_bounds__(kScanThreads)
    k_scan_lookback(const T* in, LO n, LO* out, unsigned long long* st, LO nb, int* status,
                    bool vec, LO* count) {
  static_assert(kScanItems == 16, "16 items per thread: 4 int4 of LO or one int4 of I8");
  __shared__ LO s_tile, s_prefix;
  __shared__ LO s_warp[kScanThreads / 32];
  if (threadIdx.x == 0) s_tile = LO(atomicAdd(&st[nb], 1ull));
  __syncthreads();
  LO t = s_tile;
  LO base = t * kScanTile + LO(threadIdx.x) * kScanItems;
  LO v[kScanItems];
  if (vec && base + kScanItems <= n) {
    if (sizeof(T) == 1) {
      int4 q = *reinterpret_cast<const int4*>(in + base);
      const T* b = reinterpret_cast<const T*>(&q);
#pragma unroll
      for (int k = 0; k < kScanItems; ++k) v[k] = kCompact ? LO(b[k] != 0) : LO(b[k]);
    } else {
#pragma unroll
      for (int q = 0; q < kScanItems / 4; ++q) {
        int4 w = reinterpret_cast<const int4*>(in + base)[q];
        v[q * 4] = w.x;
        v[q * 4 + 1] = w.y;
        v[q * 4 + 2] = w.z;
        v[q * 4 + 3] = w.w;
      }
      if (kCompact)
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = LO(v[k] != 0);
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      LO i = base + k;
      v[k] = i < n ? (kCompact ? LO(in[i] != 0) : LO(in[i])) : 0;
    }
  }
  LO s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s += v[k];
  int lane = int(threadIdx.x & 31u), warp = int(threadIdx.x >> 5);
  LO incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    LO y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  LO wex = 0, agg = 0;
#pragma unroll
  for (int w = 0; w < kScanThreads / 32; ++w) {
    LO x = s_warp[w];
    if (w < warp) wex += x;
    agg += x;
  }
  if (warp == 0) {
    LO prefix = 0;
    if (t == 0) {
      if (lane == 0) atomicExch(&st[0], kTilePre | unsigned(agg));
    } else {
      if (lane == 0) atomicExch(&st[t], kTileAgg | unsigned(agg));
      prefix = tile_lookback(st, t, status);
      if (lane == 0) atomicExch(&st[t], kTilePre | unsigned(prefix + agg));
    }
    if (lane == 0) {
      s_prefix = prefix;
      if (t == nb - 1) {
        if (kCompact) *count = prefix + agg;
        else out[n] = prefix + agg;
      }
    }
  }
  __syncthreads();
  LO run = s_prefix + wex + incl - s;
  if (kCompact) {
    if (out) {
#pragma unroll
      for (int k = 0; k < kScanItems; ++k)
        if (v[k]) out[run++] = base + k;
    }
  } else if (vec && base + kScanItems <= n) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      int4 w;
      w.x = run;
      run += v[q * 4];
      w.y = run;
      run += v[q * 4 + 1];
      w.z = run;
      run += v[q * 4 + 2];
      w.w = run;
      run += v[q * 4 + 3];
      reinterpret_cast<int4*>(out + base)[q] = w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      LO i = base + k;
      if (i < n) out[i] = run;
      run += v[k];
    }
  }
}

static bool aligned16(const void* p) { return (reinterpret_cast<std::uintptr_t>(p) & 15u) == 0; }

// launches k_scan_lookback over n > 0 items with fresh status words; count
// (compaction) is written into the status array's last slot when null
template <class T, bool kCompact>
static void launch_lookback(const T* in, LO n, LO* out, Arr<unsigned long long>& st, LO** count) {
  Ctx& c = ctx();
  LO nb = (n + kScanTile - 1) / kScanTile;
  st = Arr<unsigned long long>(nb + 2);
  OHG_CUDA(cudaMemsetAsync(st.data(), 0, size_t(nb + 2) * sizeof(unsigned long long), c.stream));
  bool vec = aligned16(in) && (kCompact || aligned16(out));
  LO* cnt = reinterpret_cast<LO*>(st.data() + nb + 1);
  if (count) *count = cnt;
  k_scan_lookback<T, kCompact>
      <<<nb, kScanThreads, 0, c.stream>>>(in, n, out, st.data(), nb, c.d_status, vec, cnt);
  c.launches += 1;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
}

// Self-test of the look-back's wait limit: the scan of n counts (more than
// one tile) with the first tile's ticket withheld, so no block ever
// publishes tile 0 and the other tiles' waits on it run out.  The status
// word then holds ST_STALL; out[i] for i in the first tile is not written.
// The total is then read the way every size is read back from a scan, so
// the read itself must refuse it (Error 5, OHG_ERR_TIMEOUT).
void scan_wait_limit_selftest(const LO* counts, LO n, LO* out) {
  Ctx& c = ctx();
  LO nb = (n + kScanTile - 1) / kScanTile;
  if (nb < 2) throw Error(8, "scan wait-limit self-test: needs at least two tiles");
  Arr<unsigned long long> st(nb + 2);
  OHG_CUDA(cudaMemsetAsync(st.data(), 0, size_t(nb + 2) * sizeof(unsigned long long), c.stream));
  unsigned long long first = 1;  // tickets start at tile 1
  OHG_CUDA(cudaMemcpyAsync(st.data() + nb, &first, sizeof(first), cudaMemcpyHostToDevice,
                           c.stream));
  bool vec = aligned16(counts) && aligned16(out);
  k_scan_lookback<LO, false><<<nb - 1, kScanThreads, 0, c.stream>>>(
      counts, n, out, st.data(), nb, c.d_status, vec, reinterpret_cast<LO*>(st.data() + nb + 1));
  c.launches += 1;
  last(Arr<LO>::wrap(out, n + 1));
}

template <class T>
static void scan_impl(const T* in, LO n, LO* out) {
  Ctx& c = ctx();
  if (n == 0) {
    OHG_CUDA(cudaMemsetAsync(out, 0, sizeof(LO), c.stream));
    return;
  }
  if (n <= kSmallScan) {
    k_small_scan<T><<<1, 1024, 0, c.stream>>>(in, n, out);
    c.launches += 1;
#ifdef OHG_CHECKED
    checked_after_launch(__FILE__, __LINE__);
#endif
    return;
  }
  Arr<unsigned long long> st;
  launch_lookback<T, false>(in, n, out, st, nullptr);
}

void offset_scan_into(const LO* counts, LO n, LO* out) { scan_impl(counts, n, out); }
void offset_scan_into(const I8* counts, LO n, LO* out) { scan_impl(counts, n, out); }
Arr<LO> offset_scan(const Arr<LO>& counts) {
  Arr<LO> out(counts.size() + 1);
  scan_impl(counts.data(), counts.size(), out.data());
  return out;
}
Arr<LO> offset_scan(const Arr<I8>& counts) {
  Arr<LO> out(counts.size() + 1);
  scan_impl(counts.data(), counts.size(), out.data());
  return out;
}

// ------------------------------------------------------------ fixed-scratch scan
// The same three-phase scan with its tile sums in a statically sized device
// array instead of pool memory.  It serves hosts that cannot let a library
// allocate device memory at the moment they need offsets: a host whose
// arena already owns the device memory it may use (the library's pool would
// then grow behind its back), or one recovering from an out-of-memory failure
// that needs offsets to compact its arrays before anything can be freed.
// Limit: kFixedScanMaxTiles tiles of kScanTile counts, 4,194,304 counts.
// Nothing in the scratch has to start at zero: every slot a call reads was
// written earlier in the same call.  There is one scratch per device, so two
// calls in flight on one device at once (other streams, contexts or threads)
// race on it; callers order such calls themselves.
constexpr LO kFixedScanMaxTiles = 1024;
constexpr LO kFixedScanMaxCounts = kFixedScanMaxTiles * kScanTile;
static __device__ __align__(256) LO g_fixed_scan_scratch[kFixedScanMaxTiles + 1];

// Looks up (once per device, with that device current) the device address of
// the scratch array; later calls return the cached address.
static LO* fixed_scan_scratch(int dev) {
  static std::mutex mu;
  static std::map<int, LO*> addrs;
  std::lock_guard<std::mutex> lock(mu);
  auto it = addrs.find(dev);
  if (it != addrs.end()) return it->second;
  int cur = -1;
  OHG_CUDA(cudaGetDevice(&cur));
  if (cur != dev) OHG_CUDA(cudaSetDevice(dev));
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scan_scratch);
  if (cur != dev) cudaSetDevice(cur);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    throw Error(1, std::string("cudaGetSymbolAddress of the fixed scan scratch failed: ") +
                       cudaGetErrorString(e));
  }
  addrs[dev] = static_cast<LO*>(p);
  return static_cast<LO*>(p);
}

LO offset_scan_fixed_limit() { return kFixedScanMaxCounts; }

void offset_scan_fixed_scratch(const LO* counts, LO n, LO* out) {
  if (n < 0) throw Error(8, "offset scan without allocation: negative count " + std::to_string(n));
  if (n > kFixedScanMaxCounts)
    throw Error(8, "offset scan without allocation: " + std::to_string(n) +
                       " counts exceed the fixed scratch limit of " +
                       std::to_string(kFixedScanMaxCounts));
  Ctx& c = ctx();
  LO* sums = fixed_scan_scratch(c.device);
  if (n == 0) {
    OHG_CUDA(cudaMemsetAsync(out, 0, sizeof(LO), c.stream));
    return;
  }
  LO nb = (n + kScanTile - 1) / kScanTile;
  k_tile_sums<LO><<<nb, kScanThreads, 0, c.stream>>>(counts, n, sums);
  k_scan_sums<<<1, 1024, 0, c.stream>>>(sums, nb, sums + nb);
  k_tile_scan<LO><<<nb, kScanThreads, 0, c.stream>>>(counts, n, sums, out, sums + nb);
  c.launches += 3;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
}

// Sizes read back from scans come with the status word, copied in the same
// wait.  A scan tile whose look-back gave up (ST_STALL) wrote offsets from an
// incomplete prefix, so its offsets and the scan's total need not agree; no
// array may then be sized from that total or filled through those offsets.
static void queue_status_read(Ctx& c) {
  OHG_CUDA(cudaMemcpyAsync(c.h_pinned + kPinnedStatusSlot, c.d_status, sizeof(int),
                           cudaMemcpyDeviceToHost, c.stream));
}
static void check_no_stall(const Ctx& c) {
  if (c.h_pinned[kPinnedStatusSlot] & ST_STALL)
    throw Error(5, "a scan tile gave up waiting for its predecessor; its offsets and total "
                   "are not used");
}

LO last(const Arr<LO>& a, const char* file, int line) {
  Ctx& c = ctx();
  OHG_CUDA(cudaMemcpyAsync(c.h_pinned, a.data() + a.size() - 1, sizeof(LO),
                           cudaMemcpyDeviceToHost, c.stream));
  queue_status_read(c);
  c.sync(file, line);
  check_no_stall(c);
  return c.h_pinned[0];
}

void read_lasts(const std::vector<const Arr<LO>*>& arrs, LO* out, int* status, const char* file,
                int line) {
  Ctx& c = ctx();
  int n = int(arrs.size());
  if (n > kPinnedStatusSlot) throw Error(8, "read_lasts: too many arrays");
  for (int i = 0; i < n; ++i)
    OHG_CUDA(cudaMemcpyAsync(c.h_pinned + i, arrs[i]->data() + arrs[i]->size() - 1, sizeof(LO),
                             cudaMemcpyDeviceToHost, c.stream));
  queue_status_read(c);
  c.sync(file, line);
  check_no_stall(c);
  for (int i = 0; i < n; ++i) out[i] = c.h_pinned[i];
  if (status) *status = c.h_pinned[kPinnedStatusSlot];
}

Arr<LO> collect_marked_offs(const Arr<I8>& marks, const Arr<LO>& offs, LO cnt) {
  LO n = marks.size();
  Arr<LO> out(cnt);
  auto m = cview(marks);
  auto o = cview(offs);
  auto d = view(out);
  pfor(n, [=] __device__(LO i) {
    if (m[i]) d[o[i]] = i;
  });
  return out;
}

// indices of the nonzero marks in increasing order: one compaction launch
// and one read of the count; the result keeps its n-slot buffer
Arr<LO> collect_marked(const Arr<I8>& marks, const char* file, int line) {
  return collect_marked(marks, nullptr, nullptr, file, line);
}
Arr<LO> collect_marked(const Arr<I8>& marks, const int* extra_dev, int* extra_host,
                       const char* file, int line) {
  LO n = marks.size();
  Ctx& c = ctx();
  if (n == 0) {
    if (extra_dev) {
      OHG_CUDA(cudaMemcpyAsync(c.h_pinned + 1, extra_dev, sizeof(int), cudaMemcpyDeviceToHost,
                               c.stream));
      c.sync(file, line);
      *extra_host = c.h_pinned[1];
    }
    return Arr<LO>(0);
  }
  Arr<LO> out(n);
  Arr<unsigned long long> st;
  LO* cnt = nullptr;
  launch_lookback<I8, true>(marks.data(), n, out.data(), st, &cnt);
  OHG_CUDA(cudaMemcpyAsync(c.h_pinned, cnt, sizeof(LO), cudaMemcpyDeviceToHost, c.stream));
  if (extra_dev)
    OHG_CUDA(cudaMemcpyAsync(c.h_pinned + 1, extra_dev, sizeof(int), cudaMemcpyDeviceToHost,
                             c.stream));
  queue_status_read(c);
  c.sync(file, line);
  check_no_stall(c);
  out.n = c.h_pinned[0];
  if (extra_dev) *extra_host = c.h_pinned[1];
  return out;
}
LO count_marked(const Arr<I8>& marks, const char* file, int line) {
  LO n = marks.size();
  if (n == 0) return 0;
  Ctx& c = ctx();
  Arr<unsigned long long> st;
  LO* cnt = nullptr;
  launch_lookback<I8, true>(marks.data(), n, nullptr, st, &cnt);
  OHG_CUDA(cudaMemcpyAsync(c.h_pinned, cnt, sizeof(LO), cudaMemcpyDeviceToHost, c.stream));
  queue_status_read(c);
  c.sync(file, line);
  check_no_stall(c);
  return c.h_pinned[0];
}

// ------------------------------------------------------------ FP64 peak
// Eight independent chains of dependent FP64 fused multiply-adds per thread:
// the FP64 pipe's throughput, the ceiling of the FP64-bound kernels (their
// arithmetic keeps the reference's evaluation order in FP64).
__global__ void __launch_bounds__(256) k_dfma_chains(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = double(threadIdx.x) * 1e-9 + double(k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == -1.0) out[blockIdx.x] = s;  // never true; keeps the chains live
}

double fp64_peak_gflops(int reps) {
  Ctx& c = ctx();
  const int block = 256, iters = 4096;
  int grid = c.num_sms * 8;
  Arr<double> sink(grid);
  cudaEvent_t e0, e1;
  OHG_CUDA(cudaEventCreate(&e0));
  OHG_CUDA(cudaEventCreate(&e1));
  float best = -1.0f;
  for (int r = 0; r < reps + 1; ++r) {
    OHG_CUDA(cudaEventRecord(e0, c.stream));
    k_dfma_chains<<<grid, block, 0, c.stream>>>(sink.data(), iters, 0.9999999, 1e-7);
    OHG_CUDA(cudaEventRecord(e1, c.stream));
    OHG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    OHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (r > 0 && (best < 0.0f || ms < best)) best = ms;  // the first launch warms up
  }
  c.launches += unsigned(reps + 1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  double flops = 2.0 * 8.0 * double(iters) * double(grid) * double(block);
  return flops / (double(best) * 1e-3) / 1e9;
}

// ------------------------------------------------------------ reductions
template <class T, class Op>
__global__ void k_reduce(const T* in, LO n, T init, Op op, T* out) {
  __shared__ T sh[kBlock];
  T acc = init;
  for (LO i = LO(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += LO(gridDim.x) * blockDim.x)
    acc = op(acc, in[i]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (int(threadIdx.x) < s) sh[threadIdx.x] = op(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}
// the reduction of a into a one-element device array (no host wait)
template <class T, class Op>
static Arr<T> reduce_dev(const Arr<T>& a, T init, Op op) {
  Ctx& c = ctx();
  LO n = a.size();
  int nb = int(std::min<LO>(1024, (n + kBlock - 1) / kBlock));
  if (nb < 1) nb = 1;
  Arr<T> part(nb);
  k_reduce<<<nb, kBlock, 0, c.stream>>>(a.data(), n, init, op, part.data());
  Arr<T> fin(1);
  k_reduce<<<1, kBlock, 0, c.stream>>>(part.data(), LO(nb), init, op, fin.data());
  c.launches += 2;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
  return fin;
}
template <class T, class Op>
static T reduce(const Arr<T>& a, T init, Op op) {
  return get_elem(reduce_dev(a, init, op), 0);
}
struct MaxOp {
  template <class T>
  __device__ T operator()(T a, T b) const { return (a < b) ? b : a; }
};
struct MinOp {
  template <class T>
  __device__ T operator()(T a, T b) const { return (b < a) ? b : a; }
};
I8 max_i8(const Arr<I8>& a) { return reduce<I8>(a, I8(-128), MaxOp()); }
LO max_lo(const Arr<LO>& a) { return reduce<LO>(a, LO(-2147483647 - 1), MaxOp()); }
double min_f64(const Arr<double>& a) { return reduce<double>(a, DBL_MAX, MinOp()); }
Arr<double> min_f64_dev(const Arr<double>& a) { return reduce_dev<double>(a, DBL_MAX, MinOp()); }
double max_f64(const Arr<double>& a) { return reduce<double>(a, -DBL_MAX, MaxOp()); }

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of (32-bit digit source, value) pairs, 4-bit digits.
// Each block owns a tile of kRsItems consecutive items per thread; ranks
// inside a tile come from per-thread digit counts scanned across threads, so
// equal digits keep their input order.
constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsBins = 16;

__global__ void k_rs_hist(const std::uint32_t* keys, LO n, int shift, LO* hist, LO nb) {
  __shared__ LO h[kRsBins];
  if (threadIdx.x < kRsBins) h[threadIdx.x] = 0;
  __syncthreads();
  LO base = LO(blockIdx.x) * kRsTile + LO(threadIdx.x) * kRsItems;
  for (int k = 0; k < kRsItems; ++k) {
    LO i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRsBins - 1)], 1);
  }
  __syncthreads();
  if (threadIdx.x < kRsBins) hist[LO(threadIdx.x) * nb + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_rs_scatter(const std::uint32_t* keys, const LO* vals, LO n, int shift,
                             const LO* offs, LO nb, std::uint32_t* okeys, LO* ovals) {
  __shared__ LO cnt[kRsBins][kRsThreads + 1];
  LO base = LO(blockIdx.x) * kRsTile + LO(threadIdx.x) * kRsItems;
  LO c[kRsBins];
  for (int d = 0; d < kRsBins; ++d) c[d] = 0;
  for (int k = 0; k < kRsItems; ++k) {
    LO i = base + k;
    if (i < n) c[(keys[i] >> shift) & (kRsBins - 1)]++;
  }
  for (int d = 0; d < kRsBins; ++d) cnt[d][threadIdx.x] = c[d];
  __syncthreads();
  if (threadIdx.x < kRsBins) {
    LO run = offs[LO(threadIdx.x) * nb + blockIdx.x];
    for (int t = 0; t < kRsThreads; ++t) {
      LO v = cnt[threadIdx.x][t];
      cnt[threadIdx.x][t] = run;
      run += v;
    }
  }
  __syncthreads();
  for (int d = 0; d < kRsBins; ++d) c[d] = cnt[d][threadIdx.x];
  for (int k = 0; k < kRsItems; ++k) {
    LO i = base + k;
    if (i < n) {
      std::uint32_t key = keys[i];
      int d = (key >> shift) & (kRsBins - 1);
      LO pos = c[d]++;
      okeys[pos] = key;
      ovals[pos] = vals[i];
    }
  }
}

// sorts vals by keys[0..n) on bits [0, nbits), stably; both arrays permuted
static void radix_pass_pairs(Arr<std::uint32_t>& keys, Arr<LO>& vals, int nbits) {
  Ctx& c = ctx();
  LO n = keys.size();
  if (n <= 1) return;
  LO nb = (n + kRsTile - 1) / kRsTile;
  Arr<LO> hist(kRsBins * nb);
  Arr<LO> offs(kRsBins * nb + 1);
  Arr<std::uint32_t> k2(n);
  Arr<LO> v2(n);
  for (int shift = 0; shift < nbits; shift += 4) {
    k_rs_hist<<<nb, kRsThreads, 0, c.stream>>>(keys.data(), n, shift, hist.data(), nb);
    offset_scan_into(hist.data(), kRsBins * nb, offs.data());
    k_rs_scatter<<<nb, kRsThreads, 0, c.stream>>>(keys.data(), vals.data(), n, shift,
                                                   offs.data(), nb, k2.data(), v2.data());
    c.launches += 2;
#ifdef OHG_CHECKED
    checked_after_launch(__FILE__, __LINE__);
#endif
    std::swap(keys, k2);
    std::swap(vals, v2);
  }
}

static int bits_needed(std::uint64_t maxv) {
  int b = 0;
  while (b < 64 && (maxv >> b) != 0) ++b;
  return b;
}

// LSD over tuple components from last to first; each component gathered
// through the current permutation, sorted stably on its significant bits
Arr<LO> sort_by_keys(const Arr<LO>& keys, int w) {
  LO n = keys.size() / w;
  Arr<LO> perm = iota(n);
  LO mx = max_lo(keys);
  int nbits = bits_needed(std::uint64_t(mx < 0 ? 0xffffffffu : std::uint32_t(mx)));
  if (nbits == 0) return perm;
  for (int comp = w - 1; comp >= 0; --comp) {
    Arr<std::uint32_t> k(n);
    const LO* src = keys.data();
    const LO* p = perm.data();
    std::uint32_t* kd = k.data();
    pfor(n, [=] __device__(LO i) { kd[i] = std::uint32_t(src[LO(p[i]) * w + comp]); });
    radix_pass_pairs(k, perm, nbits);
  }
  return perm;
}

Arr<LO> sort_by_keys64(const Arr<GO>& keys, int w) {
  LO n = keys.size() / w;
  Arr<LO> perm = iota(n);
  for (int comp = w - 1; comp >= 0; --comp) {
    for (int half = 0; half < 2; ++half) {
      Arr<std::uint32_t> k(n);
      const GO* src = keys.data();
      const LO* p = perm.data();
      std::uint32_t* kd = k.data();
      pfor(n, [=] __device__(LO i) {
        std::uint64_t v = std::uint64_t(src[LO(p[i]) * w + comp]);
        kd[i] = half == 0 ? std::uint32_t(v & 0xffffffffu) : std::uint32_t(v >> 32);
      });
      radix_pass_pairs(k, perm, 32);
    }
  }
  return perm;
}

}  // namespace ohg
