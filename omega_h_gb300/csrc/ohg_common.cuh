// Runtime layer of the GB300 adapt-pass library: typed, reference-counted
// device arrays allocated stream-ordered from the device memory pool, a
// per-context stream and device status word, and the element-wise launch
// helper used by the bookkeeping kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace ohg {

typedef std::int32_t LO;
typedef std::int64_t GO;
typedef std::int8_t I8;

enum { VERT = 0, EDGE = 1, FACE = 2, REGION = 3 };

// status bits raised by kernels into the context's device status word
enum StatusBits : int {
  ST_NO_MATCH = 1,      // reflect_down found no (or two) matching entities
  ST_LOOP_TOO_BIG = 2,  // an edge ring had more tets than a kernel's bound
  ST_BOUNDS = 4,        // an index fell outside its array
  ST_NUMERIC = 8,       // a degenerate eigen solve or non-finite value
  ST_TOPOLOGY = 16,     // an edge ring that does not close
  ST_STALL = 32,        // a scan tile waited past its limit for a predecessor
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_fail(cudaError_t e, const char* what, const char* file, int line);
#define OHG_CUDA(call)                                                 \
  do {                                                                 \
    cudaError_t ohg_e_ = (call);                                       \
    if (ohg_e_ != cudaSuccess) ::ohg::cuda_fail(ohg_e_, #call, __FILE__, __LINE__); \
  } while (0)

// Online launch-shape autotuner.  A tuned launch site (a kernel and the
// size class of its launch, log2 of the item count) has a few variants (block
// sizes, queue chunks) that all compute the same results; in explore mode
// the first launches of a site run each variant once, timed by CUDA events
// on the context's stream, and the site then keeps the fastest.  Events are
// read at the next host wait, so tuning adds no synchronisation.  Frozen
// mode uses the choices made so far (the default variant elsewhere); off
// mode uses the defaults.
struct Tuner {
  enum Mode { OFF = 0, EXPLORE = 1, FROZEN = 2 };
  struct Site {
    const char* name = nullptr;
    int line = 0, bucket = 0;
    int nvar = 0, dflt = 0;
    int seen = 0;                // launches of the site
    std::vector<float> best;     // fastest timed launch per variant (ms), < 0 untimed
    std::vector<char> launched;  // variant timed (in flight or read)
    int chosen = -1;
  };
  struct Pending {
    Site* site;
    int var;
    cudaEvent_t a, b;
  };
  int mode = FROZEN;
  int forced = -1;  // every tuned site runs variant (forced mod its count)
  std::unordered_map<std::uint64_t, Site> sites;
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> spare;
  int open = -1;  // pending entry of the launch being issued
  // variant for a launch of n items at site (name, line); brackets it with
  // events when it is an exploration launch (open >= 0: the caller then
  // calls stop after the launch)
  int select(const char* name, int line, long long n, int nvar, int dflt, cudaStream_t s);
  void stop(cudaStream_t s);
  // reads finished events (call after the stream is idle)
  void resolve();
  void release();
};

// pinned host scratch: small reads, with one slot kept for the status word
// read beside scan totals
constexpr int kPinnedInts = 32;
constexpr int kPinnedStatusSlot = kPinnedInts - 1;

// Freed device blocks kept for reuse, by size class: a host-side cache in
// front of the stream-ordered pool, whose allocation calls cost about 3 µs
// of host time each over a pass's few hundred arrays of mixed sizes.  Every
// block belongs to one context and is used on its stream only, so a block
// freed (its last use enqueued) may serve the next allocation at once, as
// the pool itself would.  Blocks past the cap go back to the pool.
struct DevCache {
  std::mutex mu;
  std::unordered_map<size_t, std::vector<void*>> lists;
  size_t bytes = 0;
  size_t cap = size_t(2) << 30;
  bool open = true;
  cudaStream_t stream = nullptr;
  void* take(size_t cls);
  bool put(void* p, size_t cls);
  void release();  // every cached block back to the pool (stream-ordered)
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int* d_status = nullptr;  // device status word
  int* h_pinned = nullptr;  // pinned host scratch for small reads
  int* d_swap_tables = nullptr;  // edge-swap triangulation tables (device copy)
  int swap_tables_len = 0;
  int num_sms = 0;  // streaming multiprocessors of the device
  std::uint64_t launches = 0;
  std::uint64_t syncs = 0;  // host waits on the stream (sizes and flags read back)
  // host waits per source line of the caller, kept when the environment sets
  // OHG_TRACE_SYNCS and printed to stderr when the context is destroyed
  bool trace_syncs = false;
  std::map<std::pair<std::string, int>, std::uint64_t> sync_sites;
  // with the trace: host time blocked in each site's waits (nanoseconds)
  std::map<std::pair<std::string, int>, std::uint64_t> sync_wait_ns;
  // and the host time from the previous wait's return to this one (the
  // host issuing the work in between), with the launches issued in it
  std::map<std::pair<std::string, int>, std::uint64_t> sync_issue_ns, sync_issue_launches;
  std::int64_t trace_last_ns = -1;
  std::uint64_t trace_last_launches = 0;
  std::uint64_t allocs = 0;  // device allocations made through dev_alloc
  // FP32 screening with exact FP64 recheck (1, default) or FP64 throughout (0)
  int screening = 1;
  // screening counters: cavity tets screened, tets recomputed in FP64,
  // edge lengths screened, edge lengths recomputed in FP64
  unsigned long long* d_screen_counts = nullptr;
  // independent-set sweeps (the largest sweep count of any thread, summed
  // over the calls since the counter was last cleared) and its pinned copy
  int* d_indset_sweeps = nullptr;
  int* h_indset_sweeps = nullptr;
  double* h_pass_min = nullptr;  // pinned: a pass's worst quality, read at its end
  std::shared_ptr<DevCache> cache = std::make_shared<DevCache>();
  // opt-in timing of named kernels: CUDA events on the context's stream
  // around each launch, resolved when read (no synchronisation in between)
  bool time_kernels = false;
  struct KernelLaunch {
    std::string name;
    cudaEvent_t start, stop;
    double bytes;
  };
  std::vector<KernelLaunch> kernel_launches;
  Tuner tuner;
  explicit Ctx(int dev);
  ~Ctx();
  Ctx(const Ctx&) = delete;
  Ctx& operator=(const Ctx&) = delete;
  void sync(const char* file = __builtin_FILE(), int line = __builtin_LINE());
  // reads and clears the device status word (synchronises the stream)
  int take_status();
};

// The calling thread's current context; library entry points set it.
Ctx& ctx();
void set_ctx(Ctx* c);

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;  // the block's size class
  cudaStream_t stream = nullptr;
  std::shared_ptr<DevCache> cache;  // the owning context's (kept past its end)
  ~Buf();
};

template <class T>
struct Arr {
  std::shared_ptr<Buf> buf;
  T* ptr = nullptr;
  LO n = 0;
  Arr() = default;
  explicit Arr(LO count) { alloc(count); }
  void alloc(LO count);
  T* data() const { return ptr; }
  LO size() const { return n; }
  bool empty() const { return n == 0; }
  // wraps memory owned by someone else (no free)
  static Arr wrap(T* p, LO count) {
    Arr a;
    a.ptr = p;
    a.n = count;
    return a;
  }
};

// a device block of at least bytes (rounded up to its size class, which
// bytes receives), from the context's cache or its pool
void* dev_alloc(size_t& bytes);

template <class T>
void Arr<T>::alloc(LO count) {
  n = count;
  buf = std::make_shared<Buf>();
  size_t bytes = size_t(count > 0 ? count : 1) * sizeof(T);
  buf->p = dev_alloc(bytes);
  buf->bytes = bytes;
  Ctx& c = ctx();
  buf->stream = c.stream;
  buf->cache = c.cache;
  ptr = static_cast<T*>(buf->p);
}

// ------------------------------------------------------------ device views
// A device array view.  In builds with OHG_CHECKED every subscript is bounds
// checked: an out-of-range index is recorded (first one wins) and the access
// is redirected to a scratch slot instead of touching memory outside the
// array; the launch helper then reports the kernel's source line.
struct BoundsRecord {
  int hit;
  long long index, size;
};
#ifdef OHG_CHECKED
// one record per translation unit (no relocatable device code)
static __device__ BoundsRecord g_bounds;
static __device__ double g_bounds_scratch[4];
#endif

template <class T>
struct View {
  T* p;
  LO n;
  __host__ __device__ __forceinline__ T& operator[](LO i) const {
#ifdef OHG_CHECKED
#ifdef __CUDA_ARCH__
    if (i < 0 || i >= n) {
      if (atomicCAS(&g_bounds.hit, 0, 1) == 0) {
        g_bounds.index = i;
        g_bounds.size = n;
      }
      return *reinterpret_cast<T*>(g_bounds_scratch);
    }
#endif
#endif
    return p[i];
  }
  __host__ __device__ __forceinline__ T* ptr() const { return p; }
};
template <class T>
View<T> view(const Arr<T>& a) {
  return {a.data(), a.size()};
}
template <class T>
View<T> view(T* p, LO n) {
  return {p, n};
}
template <class T>
View<const T> cview(const Arr<T>& a) {
  return {a.data(), a.size()};
}
template <class T>
View<const T> cview(const T* p, LO n) {
  return {p, n};
}

// ------------------------------------------------------------ launches
constexpr int kBlock = 256;

template <class F>
__global__ void k_for(LO n, F f) {
  LO i = LO(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) f(i);
}

// checked builds: synchronise after a launch and report a bounds record or
// launch error together with the launching source line
#ifdef OHG_CHECKED
static inline void checked_after_launch(const char* file, int line) {
  Ctx& c = ctx();
  cudaError_t e = cudaStreamSynchronize(c.stream);
  BoundsRecord r;
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&r, g_bounds, sizeof(r));
  if (e != cudaSuccess) cuda_fail(e, "kernel launch", file, line);
  if (r.hit) {
    BoundsRecord z = {0, 0, 0};
    cudaMemcpyToSymbol(g_bounds, &z, sizeof(z));
    throw Error(2, std::string("index ") + std::to_string(r.index) + " outside [0," +
                       std::to_string(r.size) + ") in kernel launched at " + file + ":" +
                       std::to_string(line));
  }
}
#endif

// launches of at least this many items have their block size tuned
constexpr LO kTuneMinItems = 1 << 16;

// block-size variants of a k_for instance: 128, 256 (default), 512, as far
// as the kernel's register use allows
template <class F>
inline int k_for_variants() {
  static int nvar = 0;
  if (nvar == 0) {
    cudaFuncAttributes fa;
    OHG_CUDA(cudaFuncGetAttributes(&fa, k_for<F>));
    nvar = fa.maxThreadsPerBlock >= 512 ? 3 : 2;
  }
  return nvar;
}

template <class F>
inline void pfor_at(const char* file, int line, LO n, F f) {
  if (n <= 0) return;
  Ctx& c = ctx();
  int block = kBlock;
  bool timed = false;
  // A launch of fewer than kBlock items per SM takes blocks of whole warps
  // small enough for every SM to get one: small launches here are the
  // per-candidate FP64 loops (midpoint metrics, cavity qualities), and the
  // FP64 rate is a per-SM resource.
  if (n < LO(c.num_sms) * kBlock) block = std::max(32, (n / c.num_sms) & ~31);
  if (n >= kTuneMinItems && c.tuner.mode != Tuner::OFF) {
    int v = c.tuner.select(file, line, n, k_for_variants<F>(), 1, c.stream);
    timed = c.tuner.open >= 0;
    block = 128 << v;
  }
  k_for<<<(n + block - 1) / block, block, 0, c.stream>>>(n, f);
  if (timed) c.tuner.stop(c.stream);
  ++c.launches;
#ifdef OHG_CHECKED
  checked_after_launch(file, line);
#else
  (void)file;
  (void)line;
#endif
}
#define pfor(n, ...) ::ohg::pfor_at(__FILE__, __LINE__, (n), __VA_ARGS__)

// Lane groups: G consecutive lanes of a warp (G a power of two, at most 32)
// share one work item, item = global thread / G, with gl the lane in the
// group.  Every thread of the grid calls f, threads past the last item with
// item = -1, so code after the item's work may use full-warp collectives.
template <int G>
__device__ __forceinline__ unsigned group_mask() {
  unsigned lane = threadIdx.x & 31u;
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~unsigned(G - 1)));
}
template <int G>
__device__ __forceinline__ float group_min(float v, unsigned gm) {
#pragma unroll
  for (int j = G / 2; j > 0; j >>= 1) v = fminf(v, __shfl_xor_sync(gm, v, j, G));
  return v;
}
template <int G>
__device__ __forceinline__ double group_min(double v, unsigned gm) {
#pragma unroll
  for (int j = G / 2; j > 0; j >>= 1) {
    double o = __shfl_xor_sync(gm, v, j, G);
    v = (o < v) ? o : v;
  }
  return v;
}
template <int G>
__device__ __forceinline__ bool group_any(bool p, unsigned gm) {
  return (__ballot_sync(gm, p) & gm) != 0u;
}

template <int G, class F>
__global__ void k_group_for(LO n, F f) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long item = t / G;
  f(item < n ? LO(item) : LO(-1), int(t % G), group_mask<G>());
}

template <int G, class F>
inline void group_for_at(const char* file, int line, LO n, int block, F f) {
  static_assert(G >= 1 && G <= 32 && (G & (G - 1)) == 0, "G: a power of two up to 32");
  if (n <= 0) return;
  if (block % 32 != 0 || block > 1024) throw Error(8, "group_for: block not a multiple of 32");
  Ctx& c = ctx();
  long long threads = (long long)n * G;
  long long blocks = (threads + block - 1) / block;
  if (blocks > 0x7fffffffLL) throw Error(8, "group_for: too many items for one launch");
  k_group_for<G><<<unsigned(blocks), block, 0, c.stream>>>(n, f);
  ++c.launches;
#ifdef OHG_CHECKED
  checked_after_launch(file, line);
#else
  (void)file;
  (void)line;
#endif
}
#define group_for(G, n, block, ...) ::ohg::group_for_at<G>(__FILE__, __LINE__, (n), (block), __VA_ARGS__)

// Records a named kernel's launch duration (when the context times
// kernels) with its algorithmic bytes; construct before the launch, destroy
// after it.
struct KernelTimer {
  Ctx* c = nullptr;
  Ctx::KernelLaunch k;
  KernelTimer(const char* name, double bytes) {
    Ctx& x = ctx();
    if (!x.time_kernels) return;
    c = &x;
    k.name = name;
    k.bytes = bytes;
    OHG_CUDA(cudaEventCreate(&k.start));
    OHG_CUDA(cudaEventCreate(&k.stop));
    OHG_CUDA(cudaEventRecord(k.start, x.stream));
  }
  ~KernelTimer() {
    if (!c) return;
    cudaEventRecord(k.stop, c->stream);
    c->kernel_launches.push_back(k);
  }
};

// device status helper
__device__ inline void raise_status(int* st, int bits) { atomicOr(st, bits); }

// ------------------------------------------------------------ host <-> device
template <class T>
Arr<T> to_device(const std::vector<T>& h) {
  Arr<T> a(LO(h.size()));
  if (!h.empty())
    OHG_CUDA(cudaMemcpyAsync(a.data(), h.data(), h.size() * sizeof(T),
                             cudaMemcpyHostToDevice, ctx().stream));
  return a;
}
template <class T>
std::vector<T> to_host(const Arr<T>& a) {
  std::vector<T> h(size_t(a.size()));
  if (a.size())
    OHG_CUDA(cudaMemcpyAsync(h.data(), a.data(), h.size() * sizeof(T),
                             cudaMemcpyDeviceToHost, ctx().stream));
  ctx().sync();
  return h;
}
// one element read (synchronises)
template <class T>
T get_elem(const Arr<T>& a, LO i) {
  T v;
  OHG_CUDA(cudaMemcpyAsync(&v, a.data() + i, sizeof(T), cudaMemcpyDeviceToHost,
                           ctx().stream));
  ctx().sync();
  return v;
}
template <class T>
Arr<T> copy_arr(const Arr<T>& a) {
  Arr<T> b(a.size());
  if (a.size())
    OHG_CUDA(cudaMemcpyAsync(b.data(), a.data(), size_t(a.size()) * sizeof(T),
                             cudaMemcpyDeviceToDevice, ctx().stream));
  return b;
}

}  // namespace ohg
