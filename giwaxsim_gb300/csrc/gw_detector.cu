// Detector stage: sample I(q) with a rotated detector plane over many
// orientations and sum the weighted samples (tools/comparison.py:790-870,
// tools/detector.py:5-29, :194-300).
//
// One thread owns one pixel for the whole orientation loop, so the sum over
// orientations stays in registers (float64, or Kahan-compensated float32)
// and the image is written once; no atomics.  Per pixel and orientation the
// thread replays the reference's exact float64 arithmetic: the plane
// rotations in BLAS fused order (rot_chain), the shift by np.min(q), the
// floor division by np.diff(qz)[0] and np.clip, then gathers the float32
// I(q) value.  Rotation matrices and weights are computed on the host from
// the plane's corners exactly as the reference does and passed in; identity
// rotations (angle 0) are dropped by the host, which leaves every bit
// unchanged.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "gw_common.cuh"

namespace {

struct DetArgs {
  int nh, nv;
  int ny, nx, nz;
  double qmin_x, qmin_y, qmin_z, dq, inv_dq;
  const double *h, *v;
  const double *init_R;
  int n_init;
  const int *rot_start, *rot_n;
  const double *rot_R;
  const double *w;
  int n_orient;
  const float *iq;
  int kahan;
};

__device__ __forceinline__ void rotate(const double *R, double &x, double &y,
                                       double &z) {
  const double a = rot_chain(R, x, y, z);
  const double b = rot_chain(R + 3, x, y, z);
  const double c = rot_chain(R + 6, x, y, z);
  x = a; y = b; z = c;
}

__device__ __forceinline__ int clip_idx(double p, double qmin, double dq,
                                        double inv_dq, int n) {
  double k = floor_div_exact(GW_DSUB(p, qmin), dq, inv_dq);
  k = fmin(fmax(k, 0.0), (double)(n - 1));
  return (int)k;
}

__device__ __forceinline__ void base_point(const DetArgs &a, int i, int j,
                                           double &x, double &y, double &z) {
  x = 0.0; y = a.h[j]; z = a.v[i];
  for (int k = 0; k < a.n_init; ++k) rotate(a.init_R + 9 * k, x, y, z);
}

__device__ __forceinline__ int64_t gather_index(const DetArgs &a, int o,
                                                double x, double y, double z) {
  const int s = a.rot_start[o], n = a.rot_n[o];
  for (int k = 0; k < n; ++k) rotate(a.rot_R + 9 * (s + k), x, y, z);
  const int ix = clip_idx(x, a.qmin_x, a.dq, a.inv_dq, a.nx);
  const int iy = clip_idx(y, a.qmin_y, a.dq, a.inv_dq, a.ny);
  const int iz = clip_idx(z, a.qmin_z, a.dq, a.inv_dq, a.nz);
  return ((int64_t)iy * a.nx + ix) * a.nz + iz;
}

__global__ void k_detector(DetArgs a, double *acc_out) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.nh * a.nv) return;
  const int i = pix / a.nh, j = pix % a.nh;
  double x0, y0, z0;
  base_point(a, i, j, x0, y0, z0);
  if (!a.kahan) {
    double acc = 0.0;
    for (int o = 0; o < a.n_orient; ++o) {
      const int64_t idx = gather_index(a, o, x0, y0, z0);
      acc = fma((double)__ldg(a.iq + idx), a.w[o], acc);
    }
    acc_out[pix] = acc;
  } else {
    float s = 0.f, c = 0.f;
    for (int o = 0; o < a.n_orient; ++o) {
      const int64_t idx = gather_index(a, o, x0, y0, z0);
      const float yv = __ldg(a.iq + idx) * (float)a.w[o] - c;
      const float t = s + yv;
      c = (t - s) - yv;
      s = t;
    }
    acc_out[pix] = (double)s - (double)c;
  }
}

// mirror_vertical_horizontal (detector.py:246-275), then NaN/<=0 -> 1e-6 and
// the 1e-6 scale (comparison.py:859-868).
__global__ void k_det_epilogue(const double *q, int nv, int nh, int mirror,
                               double *out) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= nv * nh) return;
  const int i = pix / nh, j = pix % nh;
  const int i2 = nv - 1 - i, j2 = nh - 1 - j;
  double v = q[pix];
  if (mirror) {
    v = ((q[(size_t)i * nh + j] + q[(size_t)i * nh + j2]) + q[(size_t)i2 * nh + j]) +
        q[(size_t)i2 * nh + j2];
    const bool crow = (nv & 1) && i == nv / 2;
    const bool ccol = (nh & 1) && j == nh / 2;
    if (crow) v = (q[(size_t)i * nh + j] + q[(size_t)i * nh + j2]) * 2.0;
    if (ccol) v = (q[(size_t)i * nh + j] + q[(size_t)i2 * nh + j]) * 2.0;
    if (crow && ccol) v = q[(size_t)i * nh + j] * 4.0;
  }
  if (v != v) v = 1e-6;
  if (v <= 0.0) v = 1e-6;
  out[pix] = v * 1e-6;
}

__global__ void k_iq_to_f32(const double *in, float *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

__global__ void k_det_debug(DetArgs a, int o, int64_t *idx) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.nh * a.nv) return;
  double x, y, z;
  base_point(a, pix / a.nh, pix % a.nh, x, y, z);
  idx[pix] = gather_index(a, o, x, y, z);
}

}  // namespace

struct gw_detector_plan {
  gw_ctx *ctx = nullptr;
  gw_detector_params p{};
  int n_orient = 0, n_init = 0;
  double *d_h = nullptr, *d_v = nullptr, *d_init = nullptr, *d_rot = nullptr,
         *d_w = nullptr;
  int *d_rs = nullptr, *d_rn = nullptr;
  float *d_iq_own = nullptr;
  const float *iq = nullptr;
  double *d_acc = nullptr, *d_out = nullptr;
  bool executed = false;
};

namespace {
DetArgs det_args(gw_detector_plan *P) {
  DetArgs a{};
  a.nh = P->p.n_h; a.nv = P->p.n_v;
  a.ny = P->p.iq_shape[0]; a.nx = P->p.iq_shape[1]; a.nz = P->p.iq_shape[2];
  a.qmin_x = P->p.qmin_x; a.qmin_y = P->p.qmin_y; a.qmin_z = P->p.qmin_z;
  a.dq = P->p.dq; a.inv_dq = 1.0 / P->p.dq;
  a.h = P->d_h; a.v = P->d_v; a.init_R = P->d_init; a.n_init = P->n_init;
  a.rot_start = P->d_rs; a.rot_n = P->d_rn; a.rot_R = P->d_rot; a.w = P->d_w;
  a.n_orient = P->n_orient; a.iq = P->iq;
  a.kahan = P->p.accum == GW_ACCUM_KAHAN32;
  return a;
}

template <typename T>
int up(T **dst, const T *src, size_t n) {
  if (n == 0) { *dst = nullptr; return GW_OK; }
  GW_CUDA(gw::dev_malloc((void **)dst, n * sizeof(T)));
  GW_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return GW_OK;
}
}  // namespace

extern "C" int gw_detector_plan_create(gw_ctx *ctx, const gw_detector_params *p,
                                       const double *h_axis, const double *v_axis,
                                       const double *init_R, int32_t n_init,
                                       const int32_t *n_rot, const double *rot_R,
                                       const double *weights, int32_t n_orient,
                                       gw_detector_plan **out) {
  if (!ctx || !p || !h_axis || !v_axis || !out || !weights || !n_rot)
    return gw::fail(GW_ERR_ARG, "gw_detector_plan_create: null argument");
  if (p->n_h < 1 || p->n_v < 1 || n_orient < 1 || n_init < 0 || n_init > 3 ||
      p->iq_shape[0] < 1 || p->iq_shape[1] < 1 || p->iq_shape[2] < 1 || !(p->dq > 0))
    return gw::fail(GW_ERR_ARG, "gw_detector_plan_create: invalid sizes");
  if (n_init > 0 && !init_R)
    return gw::fail(GW_ERR_ARG, "gw_detector_plan_create: init_R missing");
  std::vector<int> rs(n_orient), rn(n_orient);
  int total = 0;
  for (int o = 0; o < n_orient; ++o) {
    if (n_rot[o] < 0 || n_rot[o] > 3)
      return gw::fail(GW_ERR_ARG, "gw_detector_plan_create: 0..3 rotations per orientation");
    rs[o] = total;
    rn[o] = n_rot[o];
    total += n_rot[o];
  }
  if (total > 0 && !rot_R)
    return gw::fail(GW_ERR_ARG, "gw_detector_plan_create: rot_R missing");
  GW_CUDA(cudaSetDevice(ctx->device));
  auto *P = new gw_detector_plan();
  P->ctx = ctx;
  P->p = *p;
  P->n_orient = n_orient;
  P->n_init = n_init;
  const size_t npx = (size_t)p->n_h * p->n_v;
  int st;
  if ((st = up(&P->d_h, h_axis, p->n_h)) || (st = up(&P->d_v, v_axis, p->n_v)) ||
      (st = up(&P->d_init, init_R, (size_t)9 * n_init)) ||
      (st = up(&P->d_rot, rot_R, (size_t)9 * total)) ||
      (st = up(&P->d_w, weights, (size_t)n_orient)) ||
      (st = up(&P->d_rs, rs.data(), rs.size())) ||
      (st = up(&P->d_rn, rn.data(), rn.size()))) {
    gw_detector_plan_destroy(P);
    return st;
  }
  cudaError_t e = gw::dev_malloc((void **)&P->d_acc, npx * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&P->d_out, npx * sizeof(double));
  if (e != cudaSuccess) {
    gw_detector_plan_destroy(P);
    return gw::cuda_fail(e, "detector buffers", __FILE__, __LINE__);
  }
  *out = P;
  return GW_OK;
}

extern "C" int gw_detector_plan_destroy(gw_detector_plan *P) {
  if (!P) return GW_OK;
  void *ptrs[] = {P->d_h, P->d_v, P->d_init, P->d_rot, P->d_w, P->d_rs,
                  P->d_rn, P->d_iq_own, P->d_acc, P->d_out};
  for (void *q : ptrs) gw::dev_free(q);
  delete P;
  return GW_OK;
}

extern "C" int gw_detector_set_iq(gw_detector_plan *P, const double *iq,
                                  int32_t on_device) {
  if (!P || !iq) return gw::fail(GW_ERR_ARG, "gw_detector_set_iq: null argument");
  const int64_t n = (int64_t)P->p.iq_shape[0] * P->p.iq_shape[1] * P->p.iq_shape[2];
  if (!P->d_iq_own)
    GW_CUDA(gw::dev_malloc((void **)&P->d_iq_own, n * sizeof(float)));
  const double *src = iq;
  double *tmp = nullptr;
  if (!on_device) {
    GW_CUDA(gw::dev_malloc((void **)&tmp, n * sizeof(double)));
    cudaError_t e = cudaMemcpyAsync(tmp, iq, n * sizeof(double),
                                    cudaMemcpyHostToDevice, P->ctx->stream);
    if (e != cudaSuccess) { gw::dev_free(tmp); return gw::cuda_fail(e, "iq upload", __FILE__, __LINE__); }
    src = tmp;
  }
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 8 * P->ctx->sm_count);
  gw::KTimer tm(P->ctx, GW_K_MISC);
  k_iq_to_f32<<<blocks, 256, 0, P->ctx->stream>>>(src, P->d_iq_own, n);
  P->ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (tmp) {
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->ctx->stream);
    gw::dev_free(tmp);
  }
  if (e != cudaSuccess) return gw::cuda_fail(e, "iq conversion", __FILE__, __LINE__);
  P->iq = P->d_iq_own;
  return GW_OK;
}

extern "C" int gw_detector_set_iq32_device(gw_detector_plan *P, const float *iq32) {
  if (!P || !iq32) return gw::fail(GW_ERR_ARG, "gw_detector_set_iq32_device: null argument");
  P->iq = iq32;
  return GW_OK;
}

extern "C" int gw_detector_execute(gw_detector_plan *P) {
  if (!P) return gw::fail(GW_ERR_ARG, "gw_detector_execute: null plan");
  if (!P->iq) return gw::fail(GW_ERR_STATE, "gw_detector_execute: I(q) not set");
  GW_CUDA(cudaSetDevice(P->ctx->device));
  const int npx = P->p.n_h * P->p.n_v;
  DetArgs a = det_args(P);
  {
    gw::KTimer tm(P->ctx, GW_K_DETECTOR);
    k_detector<<<(npx + 127) / 128, 128, 0, P->ctx->stream>>>(a, P->d_acc);
    GW_LAUNCHED(P->ctx);
  }
  gw::KTimer tm(P->ctx, GW_K_DET_EPI);
  k_det_epilogue<<<(npx + 255) / 256, 256, 0, P->ctx->stream>>>(
      P->d_acc, P->p.n_v, P->p.n_h, P->p.mirror, P->d_out);
  GW_LAUNCHED(P->ctx);
  P->executed = true;
  return GW_OK;
}

extern "C" int gw_detector_get(gw_detector_plan *P, double *out, int32_t on_device) {
  if (!P || !out) return gw::fail(GW_ERR_ARG, "gw_detector_get: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_detector_get: plan not executed");
  const size_t npx = (size_t)P->p.n_h * P->p.n_v;
  GW_CUDA(cudaMemcpyAsync(out, P->d_out, npx * sizeof(double),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          P->ctx->stream));
  return gw::check_device_error(P->ctx, "detector stage");
}

extern "C" int gw_detector_debug_indices(gw_detector_plan *P, int32_t orient,
                                         int64_t *flat_idx) {
  if (!P || !flat_idx) return gw::fail(GW_ERR_ARG, "gw_detector_debug_indices: null argument");
  if (orient < 0 || orient >= P->n_orient)
    return gw::fail(GW_ERR_ARG, "gw_detector_debug_indices: orientation out of range");
  const int npx = P->p.n_h * P->p.n_v;
  int64_t *d = nullptr;
  GW_CUDA(gw::dev_malloc((void **)&d, npx * sizeof(int64_t)));
  DetArgs a = det_args(P);
  k_det_debug<<<(npx + 255) / 256, 256, 0, P->ctx->stream>>>(a, orient, d);
  P->ctx->launches++;
  cudaError_t e = cudaMemcpyAsync(flat_idx, d, npx * sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, P->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->ctx->stream);
  gw::dev_free(d);
  if (e != cudaSuccess) return gw::cuda_fail(e, "detector debug", __FILE__, __LINE__);
  return GW_OK;
}

extern "C" int gw_detector(gw_ctx *ctx, const gw_detector_params *p,
                           const double *iq, const double *h_axis,
                           const double *v_axis, const double *init_R,
                           int32_t n_init, const int32_t *n_rot,
                           const double *rot_R, const double *weights,
                           int32_t n_orient, double *out) {
  gw_detector_plan *P = nullptr;
  GW_TRY(gw_detector_plan_create(ctx, p, h_axis, v_axis, init_R, n_init, n_rot,
                                 rot_R, weights, n_orient, &P));
  int st = gw_detector_set_iq(P, iq, 0);
  if (st == GW_OK) st = gw_detector_execute(P);
  if (st == GW_OK) st = gw_detector_get(P, out, 0);
  gw_detector_plan_destroy(P);
  return st;
}

// ======================================================================
// Allocation-free detector entry point (no counterpart in the reference).
//
// Some callers cannot allocate device memory at the moment they need a
// detector image: an acquisition or fitting loop that reserved its whole
// GPU memory budget up front (a framework's caching allocator owns it, or a
// real-time pipeline must not pay cudaMalloc/cudaFree, which can block on
// other streams' work or fail under memory pressure mid-run).
// gw_detector_noalloc takes every input and the output as caller-owned
// device pointers and keeps its only scratch -- the float64 per-pixel sum
// over orientations -- in the fixed array below, so it calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// The array is a module-level __device__ variable: every GPU that loads this
// library holds its 8 MiB until the process exits.  It is shared by all
// calls on that GPU and keeps the previous call's contents; the kernel writes
// every pixel it later reads, so nothing has to be cleared.  Calls whose work
// overlaps on the GPU (different streams, or threads issuing concurrently)
// race on it and must be serialised by the caller.
constexpr int kNoAllocMaxPixels = 1 << 20;  // 1024 x 1024 pixels
static __device__ __align__(256) double g_noalloc_sum[kNoAllocMaxPixels];

namespace {

// k_detector with the per-orientation rotation offsets accumulated on the
// fly from n_rot (the caller passes only counts), writing into `sum`.
__global__ void k_detector_noalloc(DetArgs a, const int *n_rot, double *sum) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.nh * a.nv) return;
  const int i = pix / a.nh, j = pix % a.nh;
  double x0, y0, z0;
  base_point(a, i, j, x0, y0, z0);
  double acc = 0.0;
  float s = 0.f, c = 0.f;
  int start = 0;
  for (int o = 0; o < a.n_orient; ++o) {
    const int n = n_rot[o];
    double x = x0, y = y0, z = z0;
    for (int k = 0; k < n; ++k) rotate(a.rot_R + 9 * (start + k), x, y, z);
    start += n;
    const int ix = clip_idx(x, a.qmin_x, a.dq, a.inv_dq, a.nx);
    const int iy = clip_idx(y, a.qmin_y, a.dq, a.inv_dq, a.ny);
    const int iz = clip_idx(z, a.qmin_z, a.dq, a.inv_dq, a.nz);
    const float v = __ldg(a.iq + ((int64_t)iy * a.nx + ix) * a.nz + iz);
    if (!a.kahan) {
      acc = fma((double)v, a.w[o], acc);
    } else {
      const float yv = v * (float)a.w[o] - c;
      const float t = s + yv;
      c = (t - s) - yv;
      s = t;
    }
  }
  sum[pix] = a.kahan ? (double)s - (double)c : acc;
}

// Device address of g_noalloc_sum, looked up once per device.  In host code
// the symbol names a host-side shadow, not device memory, so it must never
// be passed to a kernel directly.
std::mutex g_noalloc_mu;
double *g_noalloc_ptr[128] = {};

int noalloc_scratch(int device, double **out) {
  if (device < 0 || device >= 128)
    return gw::fail(GW_ERR_ARG, "gw_detector_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sum);
    if (e != cudaSuccess)
      return gw::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_sum)", __FILE__,
                           __LINE__);
    g_noalloc_ptr[device] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[device];
  return GW_OK;
}

}  // namespace

extern "C" int gw_detector_noalloc(const gw_detector_params *p,
                                   const float *iq32, const double *h_axis,
                                   const double *v_axis, const double *init_R,
                                   int32_t n_init, const int32_t *n_rot,
                                   const double *rot_R, const double *weights,
                                   int32_t n_orient, double *out,
                                   void *stream) {
  if (!p || !iq32 || !h_axis || !v_axis || !n_rot || !weights || !out)
    return gw::fail(GW_ERR_ARG, "gw_detector_noalloc: null argument");
  if (n_init < 0 || n_init > 3 || (n_init > 0 && !init_R))
    return gw::fail(GW_ERR_ARG, "gw_detector_noalloc: n_init must be 0..3 with init_R given");
  if (p->n_h < 1 || p->n_v < 1 || n_orient < 1 || p->iq_shape[0] < 1 ||
      p->iq_shape[1] < 1 || p->iq_shape[2] < 1 || !(p->dq > 0))
    return gw::fail(GW_ERR_ARG, "gw_detector_noalloc: invalid sizes");
  if ((int64_t)p->n_h * p->n_v > kNoAllocMaxPixels)
    return gw::fail(GW_ERR_ARG,
                    "gw_detector_noalloc: detector has " +
                        std::to_string((int64_t)p->n_h * p->n_v) +
                        " pixels; the allocation-free entry point is limited "
                        "to 1048576 (1024 x 1024). Use gw_detector_plan_create "
                        "for larger images.");
  int device = 0;
  GW_CUDA(cudaGetDevice(&device));
  double *sum = nullptr;
  GW_TRY(noalloc_scratch(device, &sum));
  DetArgs a{};
  a.nh = p->n_h; a.nv = p->n_v;
  a.ny = p->iq_shape[0]; a.nx = p->iq_shape[1]; a.nz = p->iq_shape[2];
  a.qmin_x = p->qmin_x; a.qmin_y = p->qmin_y; a.qmin_z = p->qmin_z;
  a.dq = p->dq; a.inv_dq = 1.0 / p->dq;
  a.h = h_axis; a.v = v_axis; a.init_R = init_R; a.n_init = n_init;
  a.rot_start = nullptr; a.rot_n = nullptr; a.rot_R = rot_R; a.w = weights;
  a.n_orient = n_orient; a.iq = iq32;
  a.kahan = p->accum == GW_ACCUM_KAHAN32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int npx = p->n_h * p->n_v;
  k_detector_noalloc<<<(npx + 127) / 128, 128, 0, st>>>(a, n_rot, sum);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gw::cuda_fail(e, "k_detector_noalloc launch", __FILE__, __LINE__);
  k_det_epilogue<<<(npx + 255) / 256, 256, 0, st>>>(sum, p->n_v, p->n_h,
                                                    p->mirror, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return gw::cuda_fail(e, "k_det_epilogue launch", __FILE__, __LINE__);
  return GW_OK;
}
