// Shared device/host helpers of the GIWAXS GB300 library.
//
// Exactness rules used throughout:
//  * numpy's float `a // b` is the exact floor of the real quotient
//    (npy_divmod: fmod-based, then snapped).  floor_div_exact() reproduces
//    it with a rounded quotient estimate and two sign tests of fused
//    remainders, each of which is exact in sign.
//  * BLAS 3-term dot products are the fused chain
//    fma(p2,R2, fma(p1,R1, p0*R0)); rot_chain() states it with intrinsics.
//  * np.linspace(start, stop, num)[i] = i*step + start (two roundings), or
//    (i/div)*delta + start when step == 0, and the last element is stop.
// All FP64 arithmetic that feeds an index uses __d*_rn intrinsics so that
// nvcc cannot contract it into different fused operations.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "giwaxs_gb300.h"

#define GW_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------- exact ops
#ifdef __CUDA_ARCH__
#define GW_DMUL(a, b) __dmul_rn((a), (b))
#define GW_DADD(a, b) __dadd_rn((a), (b))
#define GW_DSUB(a, b) __dsub_rn((a), (b))
#define GW_DDIV(a, b) __ddiv_rn((a), (b))
#define GW_DFMA(a, b, c) __fma_rn((a), (b), (c))
#define GW_DSQRT(a) __dsqrt_rn(a)
#else
#include <cmath>
#define GW_DMUL(a, b) ((a) * (b))
#define GW_DADD(a, b) ((a) + (b))
#define GW_DSUB(a, b) ((a) - (b))
#define GW_DDIV(a, b) ((a) / (b))
#define GW_DFMA(a, b, c) std::fma((a), (b), (c))
#define GW_DSQRT(a) std::sqrt(a)
#endif

// Exact floor(a / b) for b > 0 and |a/b| < 2^52, as numpy's float //.
// inv_b is 1/b rounded (any estimate within a few ulps works).
GW_HD double floor_div_exact(double a, double b, double inv_b) {
  double k = floor(GW_DMUL(a, inv_b));
  if (GW_DFMA(-k, b, a) < 0.0) {
    k = GW_DSUB(k, 1.0);
  } else if (GW_DFMA(-GW_DADD(k, 1.0), b, a) >= 0.0) {
    k = GW_DADD(k, 1.0);
  }
  return k;
}

// Row i of R (row-major 3x3) applied to (x,y,z) in the BLAS fused order.
GW_HD double rot_chain(const double *Ri, double x, double y, double z) {
  return GW_DFMA(z, Ri[2], GW_DFMA(y, Ri[1], GW_DMUL(x, Ri[0])));
}

// np.linspace(start, stop, num)[i]
GW_HD double linspace_at(double start, double stop, int num, int i) {
  if (i == num - 1) return stop;
  double div = (double)(num - 1);
  double delta = GW_DSUB(stop, start);
  double step = GW_DDIV(delta, div);
  double y;
  if (step == 0.0) {
    y = GW_DMUL(GW_DDIV((double)i, div), delta);
  } else {
    y = GW_DMUL((double)i, step);
  }
  return GW_DADD(y, start);
}

// Order-preserving map double -> uint64 (for atomicMin/Max on doubles).
GW_HD unsigned long long dbl_ord(double d) {
#ifdef __CUDA_ARCH__
  long long b = __double_as_longlong(d);
#else
  long long b;
  memcpy(&b, &d, sizeof b);
#endif
  return b >= 0 ? ((unsigned long long)b | 0x8000000000000000ULL)
                : ~(unsigned long long)b;
}
GW_HD double ord_dbl(unsigned long long u) {
  long long b = (u & 0x8000000000000000ULL)
                    ? (long long)(u & 0x7fffffffffffffffULL)
                    : (long long)~u;
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// ------------------------------------------------- conversion-free helpers
// On this GPU float rounding (floorf), float <-> int and float <-> double
// conversions share the narrow float64 pipe.  Hot loops use these instead:
// plain float adds on the FMA pipe and integer bit operations.
// k = floor(t) for |t| < 2^21, by magic-number rounding: adding 1.5 * 2^23
// rounds t to the nearest integer (ties to even) and leaves that integer in
// the low mantissa bits; subtracting the magic number's bit pattern gives
// it as an int, and one comparison turns nearest into floor.  Returns false
// (k undefined) for |t| >= 2^21, infinities and NaN.
__device__ __forceinline__ bool floor_to_int(float t, int &k) {
  if (!(fabsf(t) < 2097152.0f)) return false;
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  const float r = __fadd_rn(t, kMagic);
  const int n = __float_as_int(r) - 0x4B400000;
  k = n - (__fsub_rn(r, kMagic) > t ? 1 : 0);
  return true;
}

// floor(min(max(t, 0), n - 1)) for 1 <= n < 2^21 (NaN gives 0, as fmaxf
// does): the clamped value is in range for the magic-number rounding.
__device__ __forceinline__ int floor_clamped(float t, int n) {
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  const float c = fminf(fmaxf(t, 0.f), (float)(n - 1));
  const float r = __fadd_rn(c, kMagic);
  return __float_as_int(r) - 0x4B400000 - (__fsub_rn(r, kMagic) > c ? 1 : 0);
}

// (double)x by IEEE 754 bit manipulation on 32-bit halves (exact); the
// hardware conversion only for subnormal, infinite and NaN inputs.
__device__ __forceinline__ double f2d_exact(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned sign = u & 0x80000000u;
  if (e == 0u || e == 0xffu) {
    if ((u << 1) == 0u) return __hiloint2double((int)sign, 0);
    return (double)x;
  }
  const unsigned m = u & 0x7fffffu;
  const unsigned hi = sign | ((e + 896u) << 20) | (m >> 3);
  return __hiloint2double((int)hi, (int)(m << 29));
}

// (float)x, IEEE 754 round to nearest even, by integer operations on the
// bit pattern; the hardware conversion (the float64 pipe) only where the
// result is zero from any input, subnormal, infinite or NaN (|x| below
// 2^-126 or from 2^128 on).  In range, the float's exponent and mantissa
// are bits 29..58 of the double's pattern re-biased by 896 << 23: adding
// 2^28 - 1 plus the kept lowest bit rounds to nearest even, and a mantissa
// carry into the exponent field is the correctly rounded result (up to
// infinity at the top).
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ah = hi & 0x7fffffffu;
  if (ah - 0x38100000u >= 0x47F00000u - 0x38100000u) return (float)x;
  const unsigned long long u =
      (((unsigned long long)ah << 32) | lo) + (0x0FFFFFFFull + ((lo >> 29) & 1u));
  return __uint_as_float(((unsigned)(u >> 29) - (896u << 23)) | (hi & 0x80000000u));
}

// (float)n, exact for n < 2^23 (n in the mantissa of 2^23); the hardware
// conversion above that.
__device__ __forceinline__ float small_u2f(unsigned n) {
  if (n >= 8388608u) return (float)n;
  return __fsub_rn(__uint_as_float(0x4B000000u + n), 8388608.0f);
}

// The count grid factorises, count = C2[(y, x) line] * C1[z]: a voxel's
// 1 / count (times the structure average's inv_nstruct) is the product of
// a line factor and a z factor, each correctly rounded (within about one
// float32 ulp of inv_nstruct / count); 0 where either count is 0.  The
// finalize and its adjoint use the same two factors.
__device__ __forceinline__ float line_count_factor(unsigned c2, float inv_nstruct) {
  return c2 ? inv_nstruct / small_u2f(c2) : 0.f;
}
__device__ __forceinline__ float z_count_factor(unsigned c1) {
  return c1 ? 1.f / small_u2f(c1) : 0.f;
}

// ---------------------------------------------------------------- context
#include <vector>

enum gw_kcat {
  GW_K_PREP = 0,     // per-structure z reduction and z indices
  GW_K_TABLES,       // per-phi column tables and count factors
  GW_K_DEPOSIT,      // per-slice y reduction + atom deposit
  GW_K_PROFILE,      // fill_bkg / smoothing profiles
  GW_K_ROW,          // row chirp-z transforms
  GW_K_COLBIN,       // column chirp-z transforms + |F|^2 + binning
  GW_K_FINALIZE,     // average, crop, f0
  GW_K_DETECTOR,     // detector orientation sum
  GW_K_DET_FIX,      // exact replay of the detector's undecided samples
  GW_K_DET_EPI,      // mirror / clamp / scale
  GW_K_MISC,         // conversions, debug
  GW_K_COUNT
};

struct gw_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  int sm_count = 0;
  size_t l2_bytes = 0;
  // device-side error word: first failing check writes its code.
  int *d_err = nullptr;
  // per-kernel timing
  int timing = 0;
  std::vector<cudaEvent_t> ev_free;
  struct Pending { cudaEvent_t a, b; int cat; };
  std::vector<Pending> pending;
  double kms[GW_K_COUNT] = {};
  int64_t kn[GW_K_COUNT] = {};
  cudaEvent_t mark[2] = {nullptr, nullptr};  // gw_ctx_mark / gw_ctx_elapsed_ms
  // a second stream, and its events, for result copies that overlap the
  // stream's kernels (made on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[17] = {};
};

namespace gw {

// thread-local last error message
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);

// A named NVTX range over the host-side work of a stage (its launches, or
// a graph replay), for timeline profilers; without one attached the push
// and pop cost a few nanoseconds.
struct Range {
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range &) = delete;
  Range &operator=(const Range &) = delete;
};
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

// fault injection for allocation failures: GW_FAIL_ALLOC_AFTER=<n> makes the
// (n+1)-th device allocation of the process and every later one fail with
// GW_ERR_OOM; set_alloc_fault(n) does the same counting from the call (n < 0
// turns it off).
cudaError_t dev_malloc(void **p, size_t bytes);
void set_alloc_fault(long long after);
void dev_free(void *p);
// Free the cached device blocks of one device (-1: all devices).
void release_alloc_cache(int device);

// checks the device error word of ctx (synchronizes the stream)
int check_device_error(gw_ctx *ctx, const char *where);

// Fault in the pages of a large host destination with several threads
// (one byte written per page) before a device-to-host copy into it.  For a
// fresh buffer the operating system's zeroing of every new page on first
// touch costs several times the copy itself, and it scales with threads.
void prefault_host(void *p, size_t bytes);
// Device-to-host copy of `bytes` into host memory dst on stream st (returns
// after the copy is enqueued; pageable destinations complete before), with
// the destination's page faulting pipelined ahead of the copy.
int copy_to_host(void *dst, const void *src, size_t bytes, cudaStream_t st);
// every page of [p, p + bytes) resident in host memory
bool host_resident(const void *p, size_t bytes);
// the context's copy stream and events, made on first use
int copy_stream_ready(gw_ctx *c);

}  // namespace gw

#define GW_CUDA(call)                                                    \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess)                                               \
      return gw::cuda_fail(_e, #call, __FILE__, __LINE__);               \
  } while (0)

#define GW_LAUNCHED(ctx)                                                 \
  do {                                                                   \
    (ctx)->launches++;                                                   \
    cudaError_t _e = cudaGetLastError();                                 \
    if (_e != cudaSuccess)                                               \
      return gw::cuda_fail(_e, "kernel launch", __FILE__, __LINE__);     \
  } while (0)

namespace gw {
// Brackets one launch with events when ctx->timing is on.
struct KTimer {
  gw_ctx *c;
  int cat;
  cudaEvent_t a = nullptr;
  KTimer(gw_ctx *ctx, int category);
  ~KTimer();
};
}  // namespace gw

#define GW_TRY(expr)                                                     \
  do {                                                                   \
    int _s = (expr);                                                     \
    if (_s != GW_OK) return _s;                                          \
  } while (0)

namespace gw {
// The largest dynamic shared memory a kernel has been allowed, per device
// (cudaFuncSetAttribute acts on the current device only): a launch site
// keeps one record per kernel and calls smem_limit before its launches.
// Threads may race to set the same limit, which is harmless; the record
// only grows.
constexpr int kSmemDevices = 64;
struct SmemRecord {
  std::atomic<size_t> bytes[kSmemDevices] = {};
};
template <class K>
int smem_limit(SmemRecord &r, K *kernel, size_t bytes) {
  int dev = 0;
  GW_CUDA(cudaGetDevice(&dev));
  const bool kept = dev >= 0 && dev < kSmemDevices;
  if (kept && r.bytes[dev].load(std::memory_order_acquire) >= bytes) return GW_OK;
  GW_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bytes));
  if (kept) {
    size_t cur = r.bytes[dev].load(std::memory_order_relaxed);
    while (cur < bytes && !r.bytes[dev].compare_exchange_weak(cur, bytes)) {
    }
  }
  return GW_OK;
}
}  // namespace gw

// device error codes written to ctx->d_err
enum { GW_DEVERR_NONE = 0, GW_DEVERR_BOX = 1, GW_DEVERR_MASK_WRAP = 2,
       GW_DEVERR_NO_ATOMS = 3, GW_DEVERR_TIMEOUT = 4 };

__device__ __forceinline__ void dev_error(int *err, int code) {
  atomicCAS(err, 0, code);
}

// float2 complex helpers
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a - b on both halves in one paired float32 instruction (sub.rn.f32x2:
// each half rounds exactly as the scalar subtraction).  The paired add,
// multiply and fma are CUDA's __fadd2_rn / __fmul2_rn / __ffma2_rn.
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

// Complex sums and differences as one paired float32 instruction each; the
// host build keeps the scalar form.
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return f2_sub(a, b);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) {
  return make_float2(a.x * s, a.y * s);
}
