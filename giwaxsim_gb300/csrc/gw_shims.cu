// Device implementations of the reference's per-slice and helper entry
// points, for callers that use them one at a time (the batched plans in
// gw_voxel.cu / gw_detector.cu are the fast path).  Each call uploads its
// host inputs, runs on the context stream, downloads its result and
// synchronises.
//
//   gw_gather            tools/detector.py:194-232 intersect_detector, and
//                        (with rotations and a weight) :278-300
//                        generate_detector_ints
//   gw_bin_slice         tools/voxelgrids.py:464-506 process_file2
//   gw_mirror            tools/detector.py:246-275 mirror_vertical_horizontal
//   gw_f0_scale          tools/voxelgrids.py:828-857 add_f0_q_3d
//   gw_collapse_lengths  tools/voxelgrids.py:238-309 rectangular_collapse_lengths
#include <algorithm>
#include <cmath>
#include <vector>

#include "gw_common.cuh"
#include "gw_slice.cuh"

namespace {

struct F0Coef {
  double c[9];
  double z;
  double s;  // 16*np.pi**2 as numpy evaluates it (libm pow)
};

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { gw::dev_free(p); }
};

int up_bytes(gw_ctx *c, DevBuf &b, const void *src, size_t bytes) {
  GW_CUDA(gw::dev_malloc(&b.p, bytes ? bytes : 1));
  if (bytes)
    GW_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream));
  return GW_OK;
}

__global__ void k_gather(const double *iq, int ny, int nx, int nz, double qx0,
                         double qy0, double qz0, double dq, double inv_dq,
                         const double *x, const double *y, const double *z,
                         int64_t n, const double *R, int nR, double w,
                         int use_w, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double a = x[i], b = y[i], c = z[i];
    for (int k = 0; k < nR; ++k) {
      const double *M = R + 9 * k;
      const double a2 = rot_chain(M, a, b, c);
      const double b2 = rot_chain(M + 3, a, b, c);
      const double c2 = rot_chain(M + 6, a, b, c);
      a = a2; b = b2; c = c2;
    }
    double kx = floor_div_exact(GW_DSUB(a, qx0), dq, inv_dq);
    double ky = floor_div_exact(GW_DSUB(b, qy0), dq, inv_dq);
    double kz = floor_div_exact(GW_DSUB(c, qz0), dq, inv_dq);
    kx = fmin(fmax(kx, 0.0), (double)(nx - 1));
    ky = fmin(fmax(ky, 0.0), (double)(ny - 1));
    kz = fmin(fmax(kz, 0.0), (double)(nz - 1));
    const double v = iq[((int64_t)ky * nx + (int64_t)kx) * nz + (int64_t)kz];
    out[i] = use_w ? GW_DMUL(v, w) : v;
  }
}

__global__ void k_bin_slice(const double *iq2d, int nv, int nh, const double *hx,
                            const double *hy, const double *vz, int qn,
                            double qmin, double qmax, double dq, double inv_dq,
                            double *sum, double *cnt) {
  const int64_t total = (int64_t)nv * nh;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / nh), c = (int)(i % nh);
    const double qx = hx[c], qy = hy[c], qz = vz[r];
    if (!(qx <= qmax && qx >= qmin && qy <= qmax && qy >= qmin)) continue;
    if (!(qz <= qmax && qz >= qmin)) continue;
    const int ix = (int)floor_div_exact(GW_DSUB(qx, qmin), dq, inv_dq);
    const int iy = (int)floor_div_exact(GW_DSUB(qy, qmin), dq, inv_dq);
    const int iz = (int)floor_div_exact(GW_DSUB(qz, qmin), dq, inv_dq);
    if (ix < 0 || iy < 0 || iz < 0 || ix >= qn || iy >= qn || iz >= qn) continue;
    const size_t v = ((size_t)iy * qn + ix) * qn + iz;
    atomicAdd(sum + v, iq2d[i]);
    atomicAdd(cnt + v, 1.0);
  }
}

__global__ void k_mirror(const double *q, int nr, int nc, double *out) {
  const int64_t total = (int64_t)nr * nc;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p / nc), j = (int)(p % nc);
    const int i2 = nr - 1 - i, j2 = nc - 1 - j;
    double v = ((q[(size_t)i * nc + j] + q[(size_t)i * nc + j2]) + q[(size_t)i2 * nc + j]) +
               q[(size_t)i2 * nc + j2];
    const bool crow = (nr & 1) && i == nr / 2;
    const bool ccol = (nc & 1) && j == nc / 2;
    if (crow) v = (q[(size_t)i * nc + j] + q[(size_t)i * nc + j2]) * 2.0;
    if (ccol) v = (q[(size_t)i * nc + j] + q[(size_t)i2 * nc + j]) * 2.0;
    if (crow && ccol) v = q[(size_t)i * nc + j] * 4.0;
    out[p] = v;
  }
}

// iq * ((a1 e^(-b1 s) + a2 e^(-b2 s) + a3 e^(-b3 s) + a4 e^(-b4 s) + c)/Z)^2,
// s = (qx^2+qy^2+qz^2)/(16 pi^2), in float64.
__global__ void k_f0(const double *iq, int ny, int nx, int nz, const double *qx,
                     const double *qy, const double *qz, F0Coef k, double *out) {
  const int64_t total = (int64_t)ny * nx * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(p % nz);
    const int ix = (int)((p / nz) % nx);
    const int iy = (int)(p / ((int64_t)nz * nx));
    const double q2 = GW_DADD(GW_DADD(GW_DMUL(qx[ix], qx[ix]), GW_DMUL(qy[iy], qy[iy])),
                              GW_DMUL(qz[iz], qz[iz]));
    const double s = k.s;
    const double f = (k.c[0] * exp(-k.c[1] * q2 / s) + k.c[2] * exp(-k.c[3] * q2 / s) +
                      k.c[4] * exp(-k.c[5] * q2 / s) + k.c[6] * exp(-k.c[7] * q2 / s) +
                      k.c[8]) / k.z;
    out[p] = iq[p] * (f * f);
  }
}

__global__ void k_collapse(const double *x, int64_t n, double hor, double ver,
                           gw_phi ph, double base, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = collapse_length(ph, hor, ver, base, x[i]);
}

int grid_for(gw_ctx *c, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * c->sm_count));
}

}  // namespace

extern "C" int gw_gather(gw_ctx *ctx, const double *iq, const int32_t *shape,
                         const double *qmin, double dq, const double *x,
                         const double *y, const double *z, int64_t n,
                         const double *R, int32_t n_R, double weight,
                         int32_t use_weight, double *out) {
  if (!ctx || !iq || !shape || !qmin || !x || !y || !z || !out || n < 0 ||
      n_R < 0 || (n_R && !R) || !(dq > 0))
    return gw::fail(GW_ERR_ARG, "gw_gather: invalid argument");
  if (shape[0] < 1 || shape[1] < 1 || shape[2] < 1)
    return gw::fail(GW_ERR_ARG, "gw_gather: empty I(q) grid");
  GW_CUDA(cudaSetDevice(ctx->device));
  const size_t niq = (size_t)shape[0] * shape[1] * shape[2];
  DevBuf diq, dx, dy, dz, dR, dout;
  GW_TRY(up_bytes(ctx, diq, iq, niq * 8));
  GW_TRY(up_bytes(ctx, dx, x, n * 8));
  GW_TRY(up_bytes(ctx, dy, y, n * 8));
  GW_TRY(up_bytes(ctx, dz, z, n * 8));
  GW_TRY(up_bytes(ctx, dR, R, (size_t)n_R * 72));
  GW_CUDA(gw::dev_malloc(&dout.p, n ? n * 8 : 8));
  if (n) {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_gather<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(
        (const double *)diq.p, shape[0], shape[1], shape[2], qmin[0], qmin[1],
        qmin[2], dq, 1.0 / dq, (const double *)dx.p, (const double *)dy.p,
        (const double *)dz.p, n, (const double *)dR.p, n_R, weight, use_weight,
        (double *)dout.p);
    GW_LAUNCHED(ctx);
    GW_CUDA(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  return GW_OK;
}

extern "C" int gw_bin_slice(gw_ctx *ctx, const double *iq2d, int32_t nv,
                            int32_t nh, const double *hx, const double *hy,
                            const double *vz, int32_t q_num, double q_min,
                            double q_max, double dq, double *sum,
                            double *count) {
  if (!ctx || !iq2d || !hx || !hy || !vz || !sum || !count || nv < 1 ||
      nh < 1 || q_num < 1 || !(dq > 0))
    return gw::fail(GW_ERR_ARG, "gw_bin_slice: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  const size_t nq = (size_t)q_num * q_num * q_num;
  DevBuf d2, dhx, dhy, dvz, ds, dc;
  GW_TRY(up_bytes(ctx, d2, iq2d, (size_t)nv * nh * 8));
  GW_TRY(up_bytes(ctx, dhx, hx, (size_t)nh * 8));
  GW_TRY(up_bytes(ctx, dhy, hy, (size_t)nh * 8));
  GW_TRY(up_bytes(ctx, dvz, vz, (size_t)nv * 8));
  GW_CUDA(gw::dev_malloc(&ds.p, nq * 8));
  GW_CUDA(gw::dev_malloc(&dc.p, nq * 8));
  GW_CUDA(cudaMemsetAsync(ds.p, 0, nq * 8, ctx->stream));
  GW_CUDA(cudaMemsetAsync(dc.p, 0, nq * 8, ctx->stream));
  {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_bin_slice<<<grid_for(ctx, (int64_t)nv * nh), 256, 0, ctx->stream>>>(
        (const double *)d2.p, nv, nh, (const double *)dhx.p,
        (const double *)dhy.p, (const double *)dvz.p, q_num, q_min, q_max, dq,
        1.0 / dq, (double *)ds.p, (double *)dc.p);
    GW_LAUNCHED(ctx);
  }
  std::vector<double> hs(nq), hc(nq);
  GW_CUDA(cudaMemcpyAsync(hs.data(), ds.p, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaMemcpyAsync(hc.data(), dc.p, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < nq; ++i) {
    if (hc[i] != 0.0) {
      sum[i] += hs[i];
      count[i] += hc[i];
    }
  }
  return GW_OK;
}

extern "C" int gw_mirror(gw_ctx *ctx, const double *in, int32_t nr, int32_t nc,
                         double *out) {
  if (!ctx || !in || !out || nr < 1 || nc < 1)
    return gw::fail(GW_ERR_ARG, "gw_mirror: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  const size_t n = (size_t)nr * nc;
  DevBuf di, dout;
  GW_TRY(up_bytes(ctx, di, in, n * 8));
  GW_CUDA(gw::dev_malloc(&dout.p, n * 8));
  {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_mirror<<<grid_for(ctx, n), 256, 0, ctx->stream>>>((const double *)di.p, nr,
                                                        nc, (double *)dout.p);
    GW_LAUNCHED(ctx);
  }
  GW_CUDA(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  return GW_OK;
}

extern "C" int gw_f0_scale(gw_ctx *ctx, const double *iq, const int32_t *shape,
                           const double *qx, const double *qy, const double *qz,
                           const double *coef, double z, double *out) {
  if (!ctx || !iq || !shape || !qx || !qy || !qz || !coef || !out || !(z > 0) ||
      shape[0] < 1 || shape[1] < 1 || shape[2] < 1)
    return gw::fail(GW_ERR_ARG, "gw_f0_scale: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  const size_t n = (size_t)shape[0] * shape[1] * shape[2];
  DevBuf di, dx, dy, dz, dout;
  GW_TRY(up_bytes(ctx, di, iq, n * 8));
  GW_TRY(up_bytes(ctx, dx, qx, (size_t)shape[1] * 8));
  GW_TRY(up_bytes(ctx, dy, qy, (size_t)shape[0] * 8));
  GW_TRY(up_bytes(ctx, dz, qz, (size_t)shape[2] * 8));
  GW_CUDA(gw::dev_malloc(&dout.p, n * 8));
  F0Coef k;
  for (int i = 0; i < 9; ++i) k.c[i] = coef[i];
  k.z = z;
  volatile double two = 2.0;
  k.s = 16 * std::pow(M_PI, two);
  {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_f0<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(
        (const double *)di.p, shape[0], shape[1], shape[2], (const double *)dx.p,
        (const double *)dy.p, (const double *)dz.p, k, (double *)dout.p);
    GW_LAUNCHED(ctx);
  }
  GW_CUDA(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  return GW_OK;
}

__global__ void k_debug_convert(const double *in, int64_t n, float *f32,
                                double *f64, int *fl, int *fl_ok) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    f32[i] = d2f_rn(in[i]);
    const float x = (float)in[i];
    f64[i] = f2d_exact(x);
    int k = 0;
    fl_ok[i] = floor_to_int(x, k) ? 1 : 0;
    fl[i] = k;
  }
}

extern "C" int gw_debug_convert(gw_ctx *ctx, const double *in, int64_t n,
                                float *f32, double *f64, int32_t *fl,
                                int32_t *fl_ok) {
  if (!ctx || !in || !f32 || !f64 || !fl || !fl_ok || n < 1)
    return gw::fail(GW_ERR_ARG, "gw_debug_convert: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  DevBuf di, d32, d64, dfl, dok;
  GW_TRY(up_bytes(ctx, di, in, n * 8));
  GW_CUDA(gw::dev_malloc(&d32.p, n * 4));
  GW_CUDA(gw::dev_malloc(&d64.p, n * 8));
  GW_CUDA(gw::dev_malloc(&dfl.p, n * 4));
  GW_CUDA(gw::dev_malloc(&dok.p, n * 4));
  {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_debug_convert<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(
        (const double *)di.p, n, (float *)d32.p, (double *)d64.p, (int *)dfl.p,
        (int *)dok.p);
    GW_LAUNCHED(ctx);
  }
  GW_CUDA(cudaMemcpyAsync(f32, d32.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaMemcpyAsync(f64, d64.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaMemcpyAsync(fl, dfl.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaMemcpyAsync(fl_ok, dok.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  return GW_OK;
}

extern "C" int gw_collapse_lengths(gw_ctx *ctx, const double *x_vals, int64_t n,
                                   double hor, double ver, const gw_phi *ph,
                                   double *out) {
  if (!ctx || !x_vals || !ph || !out || n < 0)
    return gw::fail(GW_ERR_ARG, "gw_collapse_lengths: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  double v = ph->cl_swap ? hor : ver, base = 0.0;
  GW_TRY(gw_collapse_base(&v, &ph->cos_t, 1, &base));
  DevBuf dx, dout;
  GW_TRY(up_bytes(ctx, dx, x_vals, n * 8));
  GW_CUDA(gw::dev_malloc(&dout.p, n ? n * 8 : 8));
  if (n) {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_collapse<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(
        (const double *)dx.p, n, hor, ver, *ph, base, (double *)dout.p);
    GW_LAUNCHED(ctx);
    GW_CUDA(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  GW_CUDA(cudaStreamSynchronize(ctx->stream));
  return GW_OK;
}
