// Experimental comparison on the device: tools/comparison.py:161-191
// (trim_sim_data), :406-445 (rebin_qmap_and_mask), :873-882
// (optimize_scale_offset) and the residual of fit_slabsize.py:43-44.
//
// The experimental map is rebinned once onto the trimmed simulation grid by
// a sparse interpolation matrix (three barycentric weights per target pixel
// from the Delaunay triangulation griddata uses; a target outside the
// triangulation gets NaN, griddata's fill value).  The mask is rebinned with
// the same weights and thresholded (> 0 -> 1); masked pixels take no part in
// the fit and have residual 0 (fit_slabsize.py:142, :43-44).  Each
// evaluation then reduces, over the
// trimmed window of a simulated image and the unmasked pixels, the float64
// moments n, sum x, sum t, sum xx, sum xt, sum tt; the host solves the 2x2
// least-squares system for scale and offset.
#include <algorithm>
#include <climits>
#include <cmath>

#include "gw_common.cuh"

// shift_peak (comparison.py:566-592) as two fixed sparse maps: the polar
// warp P (linear_polar, order 1: four weighted input pixels per polar
// pixel), the padded column map of add_pad with the zero mask
// (polar_image_pad[polar_image == 0] = 0), and the inverse warp Q
// (polar_linear, four weighted polar pixels per image pixel).  The weights
// are scipy's own (extracted on the host); the sums run in scipy's order.
struct gw_warp {
  gw_ctx *ctx = nullptr;
  int rows = 0, cols = 0, n_t = 0, n_r = 0;
  int *d_pidx = nullptr, *d_qidx = nullptr, *d_src = nullptr;
  double *d_pw = nullptr, *d_qw = nullptr;
  double *d_polar = nullptr;  // n_t x n_r
  double *d_in = nullptr, *d_out = nullptr;  // staging for host images
};

struct gw_compare {
  gw_ctx *ctx = nullptr;
  int n_v = 0, n_h = 0, v0 = 0, h0 = 0, rows = 0, cols = 0;
  double *d_target = nullptr;   // rows x cols
  unsigned char *d_mask = nullptr;
  double *d_sim = nullptr;      // staging of a host image (n_v x n_h)
  double *d_mom = nullptr;      // 6 moments
  double *d_res = nullptr;      // residual staging (rows x cols)
  gw_warp *warp = nullptr;      // borrowed; applied to the trimmed image
  double *d_warped = nullptr;   // rows x cols
};

namespace {

// polar[j] = sum_k w[4j+k] in[idx[4j+k]], in a rows x cols window with row
// stride `stride`
__global__ void k_to_polar(const double *in, int cols, int64_t stride,
                           const int *idx, const double *w, int64_t n,
                           double *polar) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int a = idx[4 * j + k];
      if (a >= 0) {
        const int r = a / cols, c = a - r * cols;
        acc = GW_DADD(acc, GW_DMUL(in[r * stride + c], w[4 * j + k]));
      }
    }
    polar[j] = acc;
  }
}

// out[i] = sum_k w[4i+k] z[idx[4i+k]], z the padded polar image with the
// zero mask: z[t][c] = polar[t][c] == 0 ? 0 : polar[t][src[c]]
__global__ void k_from_polar(const double *polar, int n_r, const int *src,
                             const int *idx, const double *w, int64_t n,
                             double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int a = idx[4 * i + k];
      if (a >= 0) {
        const int t = a / n_r, c = a - t * n_r;
        const double y = polar[a];
        const double z = y == 0.0 ? 0.0 : polar[(int64_t)t * n_r + src[c]];
        acc = GW_DADD(acc, GW_DMUL(z, w[4 * i + k]));
      }
    }
    out[i] = acc;
  }
}

__global__ void k_rebin(const int *idx, const double *w, int64_t n,
                        const double *val, const double *mval,
                        double *target, unsigned char *mask) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int a = idx[3 * i];
    double t, m;
    if (a < 0) {
      t = m = __longlong_as_double(0x7ff8000000000000LL);  // NaN
    } else {
      const int b = idx[3 * i + 1], c = idx[3 * i + 2];
      // griddata's order, unfused: ((w0 v0) + w1 v1) + w2 v2
      t = GW_DADD(GW_DADD(GW_DMUL(w[3 * i], val[a]), GW_DMUL(w[3 * i + 1], val[b])),
                  GW_DMUL(w[3 * i + 2], val[c]));
      m = GW_DADD(GW_DADD(GW_DMUL(w[3 * i], mval[a]), GW_DMUL(w[3 * i + 1], mval[b])),
                  GW_DMUL(w[3 * i + 2], mval[c]));
    }
    mask[i] = m > 0.0 ? 1 : 0;  // NaN > 0 is false
    target[i] = t;              // masked pixels are excluded downstream
  }
}

// moments over the unmasked pixels of the trimmed window
__global__ void k_moments(const double *sim, int n_h, int v0, int h0, int rows,
                          int cols, const double *target,
                          const unsigned char *mask, double *mom) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (mask[i]) continue;
    const int r = (int)(i / cols), c = (int)(i - (int64_t)r * cols);
    const double x = sim[(int64_t)(v0 + r) * n_h + h0 + c], t = target[i];
    s[0] += 1.0;
    s[1] += x;
    s[2] += t;
    s[3] += x * x;
    s[4] += x * t;
    s[5] += t * t;
  }
  for (int k = 0; k < 6; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(mom + k, v);
  }
}

// (target - (scale x + offset)) where unmasked, 0 where masked
__global__ void k_residual(const double *sim, int n_h, int v0, int h0,
                           int rows, int cols, const double *target,
                           const unsigned char *mask, double scale,
                           double offset, double *res) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i - (int64_t)r * cols);
    const double x = sim[(int64_t)(v0 + r) * n_h + h0 + c];
    res[i] = mask[i] ? 0.0 : target[i] - (scale * x + offset);
  }
}

int blocks_for(gw_ctx *ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * ctx->sm_count));
}

}  // namespace

// Enqueue the warp of a rows x cols device image (row stride `stride`) into
// `out` (rows x cols, contiguous).
static int warp_enqueue(gw_warp *W, const double *in, int64_t stride, double *out) {
  gw_ctx *ctx = W->ctx;
  const int64_t np = (int64_t)W->n_t * W->n_r, ni = (int64_t)W->rows * W->cols;
  k_to_polar<<<blocks_for(ctx, np), 256, 0, ctx->stream>>>(in, W->cols, stride, W->d_pidx,
                                                           W->d_pw, np, W->d_polar);
  ctx->launches++;
  GW_CUDA(cudaGetLastError());
  k_from_polar<<<blocks_for(ctx, ni), 256, 0, ctx->stream>>>(W->d_polar, W->n_r, W->d_src,
                                                             W->d_qidx, W->d_qw, ni, out);
  ctx->launches++;
  GW_CUDA(cudaGetLastError());
  return GW_OK;
}

extern "C" int gw_warp_destroy(gw_warp *W) {
  if (!W) return GW_OK;
  void *p[] = {W->d_pidx, W->d_qidx, W->d_src, W->d_pw, W->d_qw, W->d_polar,
               W->d_in, W->d_out};
  for (void *q : p) gw::dev_free(q);
  delete W;
  return GW_OK;
}

extern "C" int gw_warp_create(gw_ctx *ctx, int32_t rows, int32_t cols, int32_t n_t,
                              int32_t n_r, const int32_t *p_idx, const double *p_w,
                              const int32_t *col_src, const int32_t *q_idx,
                              const double *q_w, gw_warp **out) {
  if (!ctx || !p_idx || !p_w || !col_src || !q_idx || !q_w || !out)
    return gw::fail(GW_ERR_ARG, "gw_warp_create: null argument");
  if (rows < 1 || cols < 1 || n_t < 1 || n_r < 1 ||
      (int64_t)rows * cols >= INT32_MAX || (int64_t)n_t * n_r >= INT32_MAX)
    return gw::fail(GW_ERR_ARG, "gw_warp_create: bad shape");
  const int64_t np = (int64_t)n_t * n_r, ni = (int64_t)rows * cols;
  for (int64_t i = 0; i < 4 * np; ++i)
    if (p_idx[i] >= ni || p_idx[i] < -1)
      return gw::fail(GW_ERR_ARG, "gw_warp_create: polar-map index out of range");
  for (int64_t i = 0; i < 4 * ni; ++i)
    if (q_idx[i] >= np || q_idx[i] < -1)
      return gw::fail(GW_ERR_ARG, "gw_warp_create: image-map index out of range");
  for (int c = 0; c < n_r; ++c)
    if (col_src[c] < 0 || col_src[c] >= n_r)
      return gw::fail(GW_ERR_ARG, "gw_warp_create: column map out of range");
  GW_CUDA(cudaSetDevice(ctx->device));
  auto *W = new gw_warp();
  W->ctx = ctx;
  W->rows = rows; W->cols = cols; W->n_t = n_t; W->n_r = n_r;
  cudaStream_t st = ctx->stream;
  cudaError_t e = gw::dev_malloc((void **)&W->d_pidx, 4 * np * sizeof(int));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&W->d_pw, 4 * np * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&W->d_qidx, 4 * ni * sizeof(int));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&W->d_qw, 4 * ni * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&W->d_src, n_r * sizeof(int));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&W->d_polar, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(W->d_pidx, p_idx, 4 * np * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(W->d_pw, p_w, 4 * np * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(W->d_qidx, q_idx, 4 * ni * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(W->d_qw, q_w, 4 * ni * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(W->d_src, col_src, n_r * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    gw_warp_destroy(W);
    return gw::cuda_fail(e, "gw_warp_create", __FILE__, __LINE__);
  }
  *out = W;
  return GW_OK;
}

extern "C" int gw_warp_apply(gw_warp *W, const double *in, int32_t in_on_device,
                             double *out, int32_t out_on_device) {
  if (!W || !in || !out) return gw::fail(GW_ERR_ARG, "gw_warp_apply: null argument");
  gw_ctx *ctx = W->ctx;
  cudaStream_t st = ctx->stream;
  GW_CUDA(cudaSetDevice(ctx->device));
  const size_t n = (size_t)W->rows * W->cols;
  const double *src = in;
  if (!in_on_device) {
    if (!W->d_in) GW_CUDA(gw::dev_malloc((void **)&W->d_in, n * sizeof(double)));
    GW_CUDA(cudaMemcpyAsync(W->d_in, in, n * sizeof(double), cudaMemcpyHostToDevice, st));
    src = W->d_in;
  }
  double *dst = out;
  if (!out_on_device) {
    if (!W->d_out) GW_CUDA(gw::dev_malloc((void **)&W->d_out, n * sizeof(double)));
    dst = W->d_out;
  }
  GW_TRY(warp_enqueue(W, src, W->cols, dst));
  if (!out_on_device)
    GW_CUDA(cudaMemcpyAsync(out, dst, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaStreamSynchronize(st));
  return GW_OK;
}

extern "C" int gw_compare_set_warp(gw_compare *C, gw_warp *W) {
  if (!C) return gw::fail(GW_ERR_ARG, "gw_compare_set_warp: null comparison");
  if (W && (W->rows != C->rows || W->cols != C->cols || W->ctx != C->ctx))
    return gw::fail(GW_ERR_ARG, "gw_compare_set_warp: warp shape or context differs");
  if (W && !C->d_warped)
    GW_CUDA(gw::dev_malloc((void **)&C->d_warped, (size_t)C->rows * C->cols * sizeof(double)));
  C->warp = W;
  return GW_OK;
}

extern "C" int gw_compare_destroy(gw_compare *C) {
  if (!C) return GW_OK;
  void *p[] = {C->d_target, C->d_mask, C->d_sim, C->d_mom, C->d_res, C->d_warped};
  for (void *q : p) gw::dev_free(q);
  delete C;
  return GW_OK;
}

extern "C" int gw_compare_create(gw_ctx *ctx, int32_t n_v, int32_t n_h,
                                 int32_t v0, int32_t h0, int32_t rows,
                                 int32_t cols, const int32_t *idx,
                                 const double *w, const double *exp_values,
                                 const double *exp_mask, int64_t n_src,
                                 gw_compare **out) {
  if (!ctx || !idx || !w || !exp_values || !exp_mask || !out || n_src < 1)
    return gw::fail(GW_ERR_ARG, "gw_compare_create: null argument");
  if (rows < 1 || cols < 1 || v0 < 0 || h0 < 0 || v0 + rows > n_v || h0 + cols > n_h)
    return gw::fail(GW_ERR_ARG, "gw_compare_create: trimmed window outside the image");
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = 0; i < 3 * n; ++i)
    if (idx[i] >= n_src || (idx[i] < 0 && idx[3 * (i / 3)] >= 0))
      return gw::fail(GW_ERR_ARG, "gw_compare_create: interpolation index out of range");
  GW_CUDA(cudaSetDevice(ctx->device));
  auto *C = new gw_compare();
  C->ctx = ctx;
  C->n_v = n_v; C->n_h = n_h; C->v0 = v0; C->h0 = h0; C->rows = rows; C->cols = cols;
  int *d_idx = nullptr;
  double *d_w = nullptr, *d_val = nullptr, *d_mval = nullptr;
  cudaStream_t st = ctx->stream;
  cudaError_t e = gw::dev_malloc((void **)&C->d_target, n * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&C->d_mask, n);
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&C->d_mom, 6 * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_idx, 3 * n * sizeof(int));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_w, 3 * n * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_val, n_src * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_mval, n_src * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx, idx, 3 * n * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, w, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_val, exp_values, n_src * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_mval, exp_mask, n_src * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_rebin<<<blocks_for(ctx, n), 256, 0, st>>>(d_idx, d_w, n, d_val, d_mval,
                                                C->d_target, C->d_mask);
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  gw::dev_free(d_idx);
  gw::dev_free(d_w);
  gw::dev_free(d_val);
  gw::dev_free(d_mval);
  if (e != cudaSuccess) {
    gw_compare_destroy(C);
    return gw::cuda_fail(e, "gw_compare_create", __FILE__, __LINE__);
  }
  *out = C;
  return GW_OK;
}

extern "C" int gw_compare_target(gw_compare *C, double *target, uint8_t *mask) {
  if (!C || !target || !mask) return gw::fail(GW_ERR_ARG, "gw_compare_target: null argument");
  const size_t n = (size_t)C->rows * C->cols;
  GW_CUDA(cudaMemcpyAsync(target, C->d_target, n * sizeof(double), cudaMemcpyDeviceToHost, C->ctx->stream));
  GW_CUDA(cudaMemcpyAsync(mask, C->d_mask, n, cudaMemcpyDeviceToHost, C->ctx->stream));
  GW_CUDA(cudaStreamSynchronize(C->ctx->stream));
  return GW_OK;
}

extern "C" int gw_compare_eval(gw_compare *C, const double *sim,
                               int32_t sim_on_device, double *out,
                               double *residual) {
  if (!C || !sim || !out) return gw::fail(GW_ERR_ARG, "gw_compare_eval: null argument");
  gw_ctx *ctx = C->ctx;
  cudaStream_t st = ctx->stream;
  GW_CUDA(cudaSetDevice(ctx->device));
  const double *s = sim;
  if (!sim_on_device) {
    const size_t np = (size_t)C->n_v * C->n_h;
    if (!C->d_sim) GW_CUDA(gw::dev_malloc((void **)&C->d_sim, np * sizeof(double)));
    GW_CUDA(cudaMemcpyAsync(C->d_sim, sim, np * sizeof(double), cudaMemcpyHostToDevice, st));
    s = C->d_sim;
  }
  const int64_t n = (int64_t)C->rows * C->cols;
  // the simulated values: the trimmed window, or its shift_peak warp
  int n_h = C->n_h, v0 = C->v0, h0 = C->h0;
  if (C->warp) {
    GW_TRY(warp_enqueue(C->warp, s + (int64_t)C->v0 * C->n_h + C->h0, C->n_h, C->d_warped));
    s = C->d_warped;
    n_h = C->cols; v0 = 0; h0 = 0;
  }
  GW_CUDA(cudaMemsetAsync(C->d_mom, 0, 6 * sizeof(double), st));
  k_moments<<<blocks_for(ctx, n), 256, 0, st>>>(s, n_h, v0, h0, C->rows,
                                                C->cols, C->d_target, C->d_mask,
                                                C->d_mom);
  ctx->launches++;
  GW_CUDA(cudaGetLastError());
  double m[6];
  GW_CUDA(cudaMemcpyAsync(m, C->d_mom, sizeof m, cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaStreamSynchronize(st));
  // normal equations of min |scale x + offset - t|^2
  const double N = m[0], sx = m[1], stt = m[2], sxx = m[3], sxt = m[4], stt2 = m[5];
  const double det = N * sxx - sx * sx;
  const double scale = (N * sxt - sx * stt) / det;
  const double offset = (stt - scale * sx) / N;
  const double misfit = scale * scale * sxx + 2 * scale * offset * sx + N * offset * offset -
                        2 * scale * sxt - 2 * offset * stt + stt2;
  out[0] = scale;
  out[1] = offset;
  out[2] = misfit;
  out[3] = N;
  if (residual) {
    if (!C->d_res) GW_CUDA(gw::dev_malloc((void **)&C->d_res, n * sizeof(double)));
    k_residual<<<blocks_for(ctx, n), 256, 0, st>>>(s, n_h, v0, h0, C->rows,
                                                   C->cols, C->d_target, C->d_mask,
                                                   scale, offset, C->d_res);
    ctx->launches++;
    GW_CUDA(cudaGetLastError());
    GW_CUDA(cudaMemcpyAsync(residual, C->d_res, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    GW_CUDA(cudaStreamSynchronize(st));
    double ss = 0.0;  // the misfit from the residuals themselves
    for (int64_t i = 0; i < n; ++i) ss += residual[i] * residual[i];
    out[2] = ss;
  }
  return GW_OK;
}
