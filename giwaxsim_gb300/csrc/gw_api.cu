// Context, error reporting, allocation and host helpers of the C ABI.
#include <atomic>
#include <map>
#include <mutex>
#include <unordered_map>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "gw_common.cuh"

namespace gw {

// True when every page of [p, p + bytes) is resident (a recycled result
// buffer): such a destination needs no faulting in before a copy.  False
// when the query fails (not a mapping the kernel reports on).
bool host_resident(const void *p, size_t bytes) {
  long pg = sysconf(_SC_PAGESIZE);
  const size_t page = pg > 0 ? (size_t)pg : 4096;
  const uintptr_t lo = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)(page - 1);
  const uintptr_t hi = reinterpret_cast<uintptr_t>(p) + bytes;
  std::vector<unsigned char> v((hi - lo + page - 1) / page);
  if (mincore(reinterpret_cast<void *>(lo), hi - lo, v.data()) != 0) return false;
  for (unsigned char c : v)
    if (!(c & 1)) return false;
  return true;
}

void prefault_host(void *p, size_t bytes) {
  if (!p || bytes < ((size_t)16 << 20) || host_resident(p, bytes)) return;
  long pg = sysconf(_SC_PAGESIZE);
  const size_t page = pg > 0 ? (size_t)pg : 4096;
  const unsigned hw = std::thread::hardware_concurrency();
  const unsigned nt = std::min(16u, std::max(1u, hw));
  const size_t chunk = ((bytes / nt) / page + 1) * page;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    const size_t lo = (size_t)t * chunk;
    if (lo >= bytes) break;
    const size_t hi = std::min(bytes, lo + chunk);
    th.emplace_back([p, lo, hi, page] {
      volatile char *b = static_cast<volatile char *>(p);
      for (size_t o = lo; o < hi; o += page) b[o] = 0;
    });
  }
  for (auto &x : th) x.join();
}

int copy_stream_ready(gw_ctx *c) {
  if (!c->copy_stream)
    GW_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  for (cudaEvent_t &e : c->copy_ev)
    if (!e) GW_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return GW_OK;
}

int copy_to_host(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  // Pipelined: worker threads fault in 32 MB chunks in order while this
  // thread copies each chunk as soon as it is ready.
  constexpr size_t kChunk = (size_t)32 << 20;
  if (bytes < 2 * kChunk || host_resident(dst, bytes)) {
    prefault_host(dst, bytes);
    GW_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    return GW_OK;
  }
  long pg = sysconf(_SC_PAGESIZE);
  const size_t page = pg > 0 ? (size_t)pg : 4096;
  const size_t nc = (bytes + kChunk - 1) / kChunk;
  std::vector<std::atomic<int>> done(nc);
  for (auto &d : done) d.store(0);
  std::atomic<size_t> next{0};
  const unsigned hw = std::thread::hardware_concurrency();
  const unsigned nt = std::min(15u, std::max(1u, hw > 1 ? hw - 1 : 1u));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, page] {
      for (size_t c; (c = next.fetch_add(1)) < nc;) {
        volatile char *b = static_cast<volatile char *>(dst);
        const size_t lo = c * kChunk, hi = std::min(bytes, lo + kChunk);
        for (size_t o = lo; o < hi; o += page) b[o] = 0;
        done[c].store(1, std::memory_order_release);
      }
    });
  cudaError_t e = cudaSuccess;
  for (size_t c = 0; c < nc; ++c) {
    while (!done[c].load(std::memory_order_acquire)) std::this_thread::yield();
    const size_t lo = c * kChunk, len = std::min(bytes - lo, kChunk);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((char *)dst + lo, (const char *)src + lo, len,
                          cudaMemcpyDeviceToHost, st);
  }
  for (auto &x : th) x.join();
  if (e != cudaSuccess) return cuda_fail(e, "copy to host", __FILE__, __LINE__);
  return GW_OK;
}

}  // namespace gw

namespace gw {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int status, const std::string &msg) {
  set_error(msg);
  return status;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "%s failed: %s (%s) at %s:%d", what,
           cudaGetErrorName(e), cudaGetErrorString(e), file, line);
  set_error(buf);
  return e == cudaErrorMemoryAllocation ? GW_ERR_OOM : GW_ERR_CUDA;
}

static std::atomic<long long> g_alloc_count{0};
// gw_set_alloc_fault: allocations numbered from here on fail (-1: off)
static std::atomic<long long> g_fault_from{-1};

void set_alloc_fault(long long after) {
  g_fault_from.store(after < 0 ? -1 : g_alloc_count.load() + after);
}

// Device blocks freed by the library are kept for reuse by an allocation of
// the same device and size (plans of one shape made again and again: the
// drop-in calls in a loop, fit candidates), up to GW_ALLOC_CACHE_MB
// (default 4096; 0 disables).  A failed cudaMalloc releases the cache and
// retries; destroying the last context of a device releases its blocks.
namespace {
std::mutex g_cache_mu;
std::multimap<std::pair<int, size_t>, void *> g_cache;   // free blocks
std::unordered_map<void *, std::pair<int, size_t>> g_live;  // our blocks
size_t g_cached = 0;

size_t cache_cap() {
  static const size_t cap = [] {
    const char *s = getenv("GW_ALLOC_CACHE_MB");
    const long long mb = s ? atoll(s) : 4096;
    return mb > 0 ? (size_t)mb << 20 : (size_t)0;
  }();
  return cap;
}

void release_cache_locked(int device) {
  int cur = 0;
  cudaGetDevice(&cur);
  for (auto it = g_cache.begin(); it != g_cache.end();) {
    if (device < 0 || it->first.first == device) {
      cudaSetDevice(it->first.first);
      cudaFree(it->second);
      g_cached -= it->first.second;
      it = g_cache.erase(it);
    } else {
      ++it;
    }
  }
  cudaSetDevice(cur);
}
}  // namespace

void release_alloc_cache(int device) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  release_cache_locked(device);
}

cudaError_t dev_malloc(void **p, size_t bytes) {
  static const long long fail_after = [] {
    const char *s = getenv("GW_FAIL_ALLOC_AFTER");
    return s ? atoll(s) : -1LL;
  }();
  const long long n = g_alloc_count.fetch_add(1);
  const long long from = g_fault_from.load();
  if ((fail_after >= 0 && n >= fail_after) || (from >= 0 && n >= from)) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  const std::pair<int, size_t> key(dev, bytes);
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = g_cache.find(key);
  if (it != g_cache.end()) {
    *p = it->second;
    g_cache.erase(it);
    g_cached -= bytes;
    g_live[*p] = key;
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation && g_cached > 0) {
    cudaGetLastError();
    release_cache_locked(-1);
    e = cudaMalloc(p, bytes);
  }
  if (e == cudaSuccess) g_live[*p] = key;
  return e;
}

void dev_free(void *p) {
  if (!p) return;
  std::pair<int, size_t> key;
  bool keep = false;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_live.find(p);
    if (it != g_live.end()) {
      key = it->second;
      g_live.erase(it);
      // reserve the block's bytes in the cache before the lock is let go
      keep = key.second <= cache_cap() - std::min(cache_cap(), g_cached);
      if (keep) g_cached += key.second;
    }
  }
  if (!keep) {
    cudaFree(p);
    return;
  }
  // work queued on any stream may still use the block: wait, as cudaFree
  // would, before it can be handed out again; outside the lock, so that
  // other threads' allocations and frees do not wait for this device
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(key.first);
  cudaDeviceSynchronize();
  cudaSetDevice(cur);
  std::lock_guard<std::mutex> lk(g_cache_mu);
  g_cache.emplace(key, p);
}

int check_device_error(gw_ctx *ctx, const char *where) {
  int h = 0;
  GW_CUDA(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                          ctx->stream));
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h == GW_DEVERR_NONE) return GW_OK;
  GW_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  const char *what = "unknown device check";
  switch (h) {
    case GW_DEVERR_BOX:
      what = "an atom fell outside the slice window sized from the structure "
             "bounds";
      break;
    case GW_DEVERR_MASK_WRAP:
      what = "the smoothing mask wraps around the grid (structure extent "
             "smaller than 2*smooth); unsupported";
      break;
    case GW_DEVERR_NO_ATOMS:
      what = "zero-size array to reduction operation minimum which has no "
             "identity (no atom inside the real-space grid)";
      break;
    case GW_DEVERR_TIMEOUT:
      return fail(GW_ERR_TIMEOUT, std::string(where) +
                                      ": a bounded wait for an asynchronous tile load ran out");
  }
  return fail(GW_ERR_BOUNDS, std::string(where) + ": " + what);
}

static cudaEvent_t take_event(gw_ctx *c) {
  if (!c->ev_free.empty()) {
    cudaEvent_t e = c->ev_free.back();
    c->ev_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

KTimer::KTimer(gw_ctx *ctx, int category) : c(ctx), cat(category) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!c->timing || cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone)
    return;
  a = take_event(c);
  if (a) cudaEventRecord(a, c->stream);
}

KTimer::~KTimer() {
  if (!a) return;
  cudaEvent_t b = take_event(c);
  if (!b) return;
  cudaEventRecord(b, c->stream);
  c->pending.push_back({a, b, cat});
}

static void collect(gw_ctx *c) {
  for (auto &p : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->kms[p.cat] += ms;
      c->kn[p.cat] += 1;
    }
    c->ev_free.push_back(p.a);
    c->ev_free.push_back(p.b);
  }
  c->pending.clear();
}

}  // namespace gw

extern "C" {

int gw_ctx_set_timing(gw_ctx *c, int32_t on) {
  if (!c) return gw::fail(GW_ERR_ARG, "gw_ctx_set_timing: null context");
  if (on) {
    GW_CUDA(cudaStreamSynchronize(c->stream));
    gw::collect(c);
    for (int i = 0; i < GW_K_COUNT; ++i) { c->kms[i] = 0; c->kn[i] = 0; }
  }
  c->timing = on != 0;
  return GW_OK;
}

int gw_ctx_kernel_times(gw_ctx *c, double *ms, int64_t *launches, int32_t n) {
  if (!c || !ms || !launches) return gw::fail(GW_ERR_ARG, "gw_ctx_kernel_times: null argument");
  GW_CUDA(cudaStreamSynchronize(c->stream));
  gw::collect(c);
  const int k = n < GW_K_COUNT ? n : GW_K_COUNT;
  for (int i = 0; i < k; ++i) { ms[i] = c->kms[i]; launches[i] = c->kn[i]; }
  return k;
}

const char *gw_kernel_category_name(int32_t i) {
  static const char *names[GW_K_COUNT] = {
      "prep", "tables", "deposit", "profile", "row_czt", "col_czt_bin",
      "finalize", "detector", "det_fix", "det_epilogue", "misc"};
  return (i >= 0 && i < GW_K_COUNT) ? names[i] : "unknown";
}

int gw_version(void) { return 1; }

const char *gw_status_string(int s) {
  switch (s) {
    case GW_OK: return "GW_OK";
    case GW_ERR_ARG: return "GW_ERR_ARG";
    case GW_ERR_OOM: return "GW_ERR_OOM";
    case GW_ERR_CUDA: return "GW_ERR_CUDA";
    case GW_ERR_TIMEOUT: return "GW_ERR_TIMEOUT";
    case GW_ERR_BOUNDS: return "GW_ERR_BOUNDS";
    case GW_ERR_STATE: return "GW_ERR_STATE";
  }
  return "GW_UNKNOWN";
}

int gw_set_alloc_fault(int64_t after) {
  gw::set_alloc_fault(after);
  return GW_OK;
}

int gw_host_pin(void *ptr, uint64_t bytes) {
  if (!ptr || bytes == 0) return gw::fail(GW_ERR_ARG, "gw_host_pin: null or empty buffer");
  const cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return gw::fail(GW_ERR_CUDA, std::string("gw_host_pin: ") + cudaGetErrorString(e));
  }
  return GW_OK;
}

int gw_host_unpin(void *ptr) {
  if (!ptr) return gw::fail(GW_ERR_ARG, "gw_host_unpin: null buffer");
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return gw::fail(GW_ERR_CUDA, std::string("gw_host_unpin: ") + cudaGetErrorString(e));
  }
  return GW_OK;
}

size_t gw_last_error(char *buf, size_t len) {
  const std::string &m = gw::g_last_error;
  if (buf && len) {
    size_t n = m.size() < len - 1 ? m.size() : len - 1;
    memcpy(buf, m.data(), n);
    buf[n] = 0;
  }
  return m.size();
}

namespace {
// Live contexts per device.  The device block cache is shared by every
// context of a device; it is released when the last of them is destroyed
// (a thread pool's per-thread contexts ending leaves it to the others).
std::mutex g_ctx_mu;
std::map<int, int> g_ctx_live;
}  // namespace

int gw_ctx_create(int device, gw_ctx **out) {
  if (!out) return gw::fail(GW_ERR_ARG, "gw_ctx_create: out is null");
  int n = 0;
  GW_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n)
    return gw::fail(GW_ERR_ARG, "gw_ctx_create: no such CUDA device");
  GW_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  GW_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    return gw::fail(GW_ERR_ARG, "gw_ctx_create: this library is built for "
                                "sm_103a (GB300); device is older");
  auto *c = new gw_ctx();
  c->device = device;
  c->sm_count = prop.multiProcessorCount;
  c->l2_bytes = (size_t)prop.l2CacheSize;
  {
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    ++g_ctx_live[device];
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&c->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    gw_ctx_destroy(c);
    return gw::cuda_fail(e, "gw_ctx_create", __FILE__, __LINE__);
  }
  *out = c;
  return GW_OK;
}

int gw_ctx_destroy(gw_ctx *c) {
  if (!c) return GW_OK;
  // contexts may be destroyed on any thread (thread exit, garbage
  // collection): leave that thread's current device as it was
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  gw::collect(c);
  for (cudaEvent_t e : c->ev_free) cudaEventDestroy(e);
  for (cudaEvent_t e : c->mark)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (cudaEvent_t e : c->copy_ev)
    if (e) cudaEventDestroy(e);
  gw::dev_free(c->d_err);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  {
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if (--g_ctx_live[c->device] <= 0) {
      g_ctx_live.erase(c->device);
      gw::release_alloc_cache(c->device);
    }
  }
  delete c;
  cudaSetDevice(prev);
  return GW_OK;
}

int gw_ctx_synchronize(gw_ctx *c) {
  if (!c) return gw::fail(GW_ERR_ARG, "gw_ctx_synchronize: null context");
  GW_CUDA(cudaStreamSynchronize(c->stream));
  return gw::check_device_error(c, "device checks");
}

int gw_ctx_stream(gw_ctx *c, void **stream) {
  if (!c || !stream) return gw::fail(GW_ERR_ARG, "gw_ctx_stream: null argument");
  *stream = (void *)c->stream;
  return GW_OK;
}

int64_t gw_ctx_launch_count(gw_ctx *c) { return c ? c->launches : -1; }

int gw_ctx_device_name(gw_ctx *c, char *buf, size_t n) {
  if (!c || !buf || n == 0) return gw::fail(GW_ERR_ARG, "gw_ctx_device_name: invalid argument");
  cudaDeviceProp prop;
  GW_CUDA(cudaGetDeviceProperties(&prop, c->device));
  snprintf(buf, n, "%s sm_%d%d x%d", prop.name, prop.major, prop.minor,
           prop.multiProcessorCount);
  return GW_OK;
}

int gw_ctx_mark(gw_ctx *c, int32_t slot) {
  if (!c || slot < 0 || slot > 1) return gw::fail(GW_ERR_ARG, "gw_ctx_mark: invalid argument");
  GW_CUDA(cudaSetDevice(c->device));
  if (!c->mark[slot]) GW_CUDA(cudaEventCreate(&c->mark[slot]));
  GW_CUDA(cudaEventRecord(c->mark[slot], c->stream));
  return GW_OK;
}

int gw_ctx_elapsed_ms(gw_ctx *c, float *ms) {
  if (!c || !ms) return gw::fail(GW_ERR_ARG, "gw_ctx_elapsed_ms: null argument");
  if (!c->mark[0] || !c->mark[1])
    return gw::fail(GW_ERR_STATE, "gw_ctx_elapsed_ms: marks 0 and 1 not recorded");
  GW_CUDA(cudaEventSynchronize(c->mark[1]));
  GW_CUDA(cudaEventElapsedTime(ms, c->mark[0], c->mark[1]));
  return GW_OK;
}

int gw_rotate_points(const double *R, const double *pts, int64_t n,
                     double *out) {
  if (!R || (!pts && n) || (!out && n) || n < 0)
    return gw::fail(GW_ERR_ARG, "gw_rotate_points: invalid argument");
  for (int64_t k = 0; k < n; ++k) {
    const double x = pts[3 * k], y = pts[3 * k + 1], z = pts[3 * k + 2];
    const double a = rot_chain(R, x, y, z);
    const double b = rot_chain(R + 3, x, y, z);
    const double c = rot_chain(R + 6, x, y, z);
    out[3 * k] = a;
    out[3 * k + 1] = b;
    out[3 * k + 2] = c;
  }
  return GW_OK;
}

int gw_collapse_base(const double *ver, const double *cos_t, int64_t n,
                     double *out) {
  if (n < 0 || (n && (!ver || !cos_t || !out)))
    return gw::fail(GW_ERR_ARG, "gw_collapse_base: invalid argument");
  // numpy's scalar x**2 calls libm pow(), which is not always x*x; the
  // volatile exponent keeps the compiler from folding pow(x, 2.0) to x*x.
  volatile double two = 2.0;
  for (int64_t i = 0; i < n; ++i) {
    const double vc = ver[i] * cos_t[i];
    out[i] = std::sqrt(std::pow(ver[i], two) - std::pow(vc, two));
  }
  return GW_OK;
}

}  // extern "C"
