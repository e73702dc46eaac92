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
#include <cstdlib>
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

// ---------------------------------------------------------------- fast path
// Per orientation, the composed rotation M = R_n...R_1 maps the base plane
// point p0 to index space: t = (M p0 - qmin) / dq = A p0 + b.  Evaluated in
// float32, t differs from the exact float64 replay by at most d (a bound the
// host derives from |A|, |p0| and |b|: 10 u S + 1e-5 with u = 2^-24 and S the
// sum of the magnitudes of the terms).  When floor(t-d) and floor(t+d) agree
// after clipping on all three axes the gathered voxel is the exact one;
// otherwise the (pixel, orientation) pair goes to a worklist that
// k_detector_fix replays with the exact float64 chain.
struct OrientFast {
  float A[9];
  float b[3];
  float d[3];
  float w;
  int fix[3];  // >= 0: the axis' coordinate is exactly +-0 for every pixel
  int pad;     //       and its (clipped) index is this constant
};
constexpr int kOrientFloats = sizeof(OrientFast) / 4;

constexpr int kDetThreads = 256, kDetPix = 2, kDetChunk = 128, kDetFlush = 16;
static_assert(kDetChunk % kDetFlush == 0, "orientation chunks hold whole flush groups");
static_assert(kDetFlush * 2 <= 32, "a flush group's uncertain samples fit one 32-bit mask");

__device__ __forceinline__ bool fast_axis(float t, float d, int n, int &k) {
  // k = clamp(floor(t + d), 0, n-1) (clamping first is the same: NaN and
  // -inf give 0, +inf n-1), by magic-number rounding; clamp(floor(t - d))
  // equals it exactly when max(t - d, 0) >= k
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  const float c = fminf(fmaxf(t + d, 0.f), (float)(n - 1));
  const float r = __fadd_rn(c, kMagic);
  const float fr = __fsub_rn(r, kMagic);
  const bool down = fr > c;
  k = __float_as_int(r) - 0x4B400000 - (down ? 1 : 0);
  return fmaxf(t - d, 0.f) >= (down ? fr - 1.f : fr);
}

__device__ __forceinline__ bool fast_index(const OrientFast &T, const DetArgs &a,
                                           float x, float y, float z,
                                           int64_t &idx) {
  const float tx = fmaf(T.A[0], x, fmaf(T.A[1], y, fmaf(T.A[2], z, T.b[0])));
  const float ty = fmaf(T.A[3], x, fmaf(T.A[4], y, fmaf(T.A[5], z, T.b[1])));
  const float tz = fmaf(T.A[6], x, fmaf(T.A[7], y, fmaf(T.A[8], z, T.b[2])));
  int ix, iy, iz;
  bool ok = fast_axis(tx, T.d[0], a.nx, ix) & fast_axis(ty, T.d[1], a.ny, iy) &
            fast_axis(tz, T.d[2], a.nz, iz);
  if (T.fix[0] >= 0 || T.fix[1] >= 0 || T.fix[2] >= 0) {
    ok = (T.fix[0] >= 0 || fast_axis(tx, T.d[0], a.nx, ix)) &
         (T.fix[1] >= 0 || fast_axis(ty, T.d[1], a.ny, iy)) &
         (T.fix[2] >= 0 || fast_axis(tz, T.d[2], a.nz, iz));
    if (T.fix[0] >= 0) ix = T.fix[0];
    if (T.fix[1] >= 0) iy = T.fix[1];
    if (T.fix[2] >= 0) iz = T.fix[2];
  }
  idx = ((int64_t)iy * a.nx + ix) * a.nz + iz;
  return ok;
}

__global__ void __launch_bounds__(kDetThreads)
k_detector_fast(DetArgs a, const OrientFast *ot, double *acc_out, int2 *wl,
                int *wl_count, int wl_cap) {
  __shared__ OrientFast s_ot[kDetChunk];
  const int npx = a.nh * a.nv;
  const int lane = threadIdx.x & 31;
  int pix[kDetPix];
  bool valid[kDetPix];
  float xf[kDetPix], yf[kDetPix], zf[kDetPix];
  double x0[kDetPix], y0[kDetPix], z0[kDetPix];
  double acc[kDetPix];
  float part[kDetPix], kc[kDetPix];
#pragma unroll
  for (int k = 0; k < kDetPix; ++k) {
    pix[k] = blockIdx.x * (kDetThreads * kDetPix) + k * kDetThreads + threadIdx.x;
    valid[k] = pix[k] < npx;
    x0[k] = y0[k] = z0[k] = 0.0;
    if (valid[k]) base_point(a, pix[k] / a.nh, pix[k] % a.nh, x0[k], y0[k], z0[k]);
    xf[k] = (float)x0[k]; yf[k] = (float)y0[k]; zf[k] = (float)z0[k];
    acc[k] = 0.0; part[k] = 0.f; kc[k] = 0.f;
  }
  for (int c0 = 0; c0 < a.n_orient; c0 += kDetChunk) {
    const int nc = min(kDetChunk, a.n_orient - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc * kOrientFloats; t += kDetThreads)
      reinterpret_cast<float *>(s_ot)[t] = reinterpret_cast<const float *>(ot + c0)[t];
    __syncthreads();
    for (int oo = 0; oo < nc; ++oo) {
      const OrientFast &T = s_ot[oo];
      const int o = c0 + oo;
#pragma unroll
      for (int k = 0; k < kDetPix; ++k) {
        int64_t idx;
        const bool ok = fast_index(T, a, xf[k], yf[k], zf[k], idx);
        const bool need = valid[k] && !ok;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        bool inline_exact = false;
        if (m) {
          int base = 0;
          const int leader = __ffs(m) - 1;
          if (lane == leader) base = atomicAdd(wl_count, __popc(m));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (need) {
            const int slot = base + __popc(m & ((1u << lane) - 1u));
            if (slot < wl_cap) wl[slot] = make_int2(pix[k], o);
            else inline_exact = true;
          }
        }
        float v = 0.f;
        if (valid[k] && ok) v = __ldg(a.iq + idx);
        if (inline_exact) v = __ldg(a.iq + gather_index(a, o, x0[k], y0[k], z0[k]));
        if (valid[k] && (ok || inline_exact)) {
          if (!a.kahan) {
            part[k] = fmaf(v, T.w, part[k]);
          } else {
            const float yv = v * T.w - kc[k];
            const float t = part[k] + yv;
            kc[k] = (t - part[k]) - yv;
            part[k] = t;
          }
        }
      }
      // float32 partial sums of kDetFlush orientations, float64 across them
      if (!a.kahan && ((o + 1) % kDetFlush == 0)) {
#pragma unroll
        for (int k = 0; k < kDetPix; ++k) { acc[k] += f2d_exact(part[k]); part[k] = 0.f; }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kDetPix; ++k) {
    if (!valid[k]) continue;
    acc_out[pix[k]] = a.kahan ? f2d_exact(part[k]) - f2d_exact(kc[k])
                              : acc[k] + f2d_exact(part[k]);
  }
}

// ------------------------------------------------------------ plane mode
// When every orientation keeps the same axis at a fixed index (the plane
// rotated about its own normal, the reference's psi rotations), all samples
// lie in one plane of I(q).  The plane is copied to a compact nu x nv array
// (u, v the two free axes in memory order) and each block gathers from it:
// from shared memory when the plane fits, else from global memory through
// L1.  Blocks own 16 x 32 pixel tiles, so that per orientation a block's
// samples cover a compact patch of the plane.  Indices, worklist decisions
// and the per-pixel accumulation order are those of k_detector_fast; only
// the order in which k_detector_fix atomically adds the replayed samples
// differs (it is scheduling order in both).
struct PlaneArgs {
  int fa, fi;   // fixed axis (0 x, 1 y, 2 z) and its index
  int ua, va;   // free axes, slower and faster in memory
  int nu, nv;
  const float *P;
};
// The two free rows of an orientation's affine map, packed for three
// 16-byte shared loads: (A_u, b_u), (A_v, b_v), (d_u, d_v, w, -).
// One orientation of the plane gather.  Each member pairs the u axis's
// value with the v axis's (x, y and z coefficients, constant, certainty
// bound), so that both axes' indices are made with paired float32
// instructions; w is the orientation's weight.  Three 16-byte words.
struct __align__(16) PlaneOrient {
  float2 x, y, z, c, d;
  float w, pad;
};
static_assert(sizeof(PlaneOrient) == 48, "three 16-byte words per orientation");
constexpr int kPlTW = 32, kPlTH = 32, kPlThreads = 512;
// A compile-time bool as a value (selects a lambda's instantiation).
template <bool B>
struct BoolC {
  static constexpr bool value = B;
};
constexpr size_t kPlaneSmemMax = 200 * 1024;

__global__ void k_plane_extract(DetArgs a, PlaneArgs pa, float *P) {
  const int64_t n = (int64_t)pa.nu * pa.nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int idx[3];
    idx[pa.fa] = pa.fi;
    idx[pa.ua] = (int)(t / pa.nv);
    idx[pa.va] = (int)(t % pa.nv);
    P[t] = a.iq[((int64_t)idx[1] * a.nx + idx[0]) * a.nz + idx[2]];
  }
}

// Both axes of fast_index on those rows, u in the first half of each pair
// and v in the second: t = (y c_y + (z c_z + c)) (same operation order), and
// for each axis fast_axis with the floor taken by one addition rounded
// toward minus infinity: r = 1.5 * 2^23 + floor(t + d) exactly for clamped
// values in [0, 2^22), so the index and the certainty test are those of
// fast_axis, in fewer operations.  The paired instructions round each half
// as the scalar ones.  n1 = (nu - 1, nv - 1) as floats.  ZX: the pixels' x
// is +-0 for every pixel, so the x products (exact zeros added to the rest
// of the chain) are left out: fmaf(a, +-0, c) == c for c != 0, and a signed
// zero does not change a floor.
template <bool ZX>
__device__ __forceinline__ bool plane_index(const PlaneOrient &T, float2 n1,
                                            float2 xx, float2 yy, float2 zz,
                                            int &iu, int &iv) {
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  const float2 mg = make_float2(kMagic, kMagic);
  float2 t = __ffma2_rn(T.y, yy, __ffma2_rn(T.z, zz, T.c));
  if (!ZX) t = __ffma2_rn(T.x, xx, t);
  const float2 hi = __fadd2_rn(t, T.d), lo = f2_sub(t, T.d);
  const float2 c = make_float2(fminf(fmaxf(hi.x, 0.f), n1.x), fminf(fmaxf(hi.y, 0.f), n1.y));
  const float2 r = __fadd2_rd(c, mg);
  iu = __float_as_int(r.x) - 0x4B400000;
  iv = __float_as_int(r.y) - 0x4B400000;
  const float2 fl = f2_sub(r, mg);
  return (fmaxf(lo.x, 0.f) >= fl.x) & (fmaxf(lo.y, 0.f) >= fl.y);
}

template <bool SMEM, bool ZX>
__global__ void __launch_bounds__(kPlThreads)
k_detector_plane(DetArgs a, const PlaneOrient *ot, PlaneArgs pa,
                 double *acc_out, int2 *wl, int *wl_count, int wl_cap) {
  extern __shared__ float s_plane[];
  __shared__ PlaneOrient s_ot[kDetChunk];
  constexpr int KP = kPlTH * kPlTW / kPlThreads;  // pixels per thread
  const float2 n1 = make_float2((float)(pa.nu - 1), (float)(pa.nv - 1));
  const int tiles_x = (a.nh + kPlTW - 1) / kPlTW;
  const int j = (blockIdx.x % tiles_x) * kPlTW + (threadIdx.x % kPlTW);
  const int ib = (blockIdx.x / tiles_x) * kPlTH + threadIdx.x / kPlTW;
  const float *src = pa.P;
  if (SMEM) {
    const int n = pa.nu * pa.nv;
    for (int t = threadIdx.x; t < n; t += kPlThreads) s_plane[t] = pa.P[t];
    src = s_plane;
  }
  int pix[KP];
  bool valid[KP];
  float xf[KP], yf[KP], zf[KP];
  double acc[KP];
  float part[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k) {
    const int i = ib + k * (kPlThreads / kPlTW);
    valid[k] = i < a.nv && j < a.nh;
    pix[k] = valid[k] ? i * a.nh + j : 0;
    double x0 = 0.0, y0 = 0.0, z0 = 0.0;
    if (valid[k]) base_point(a, i, j, x0, y0, z0);
    xf[k] = (float)x0; yf[k] = (float)y0; zf[k] = (float)z0;
    acc[k] = 0.0;
    part[k] = 0.f;
  }
  // tiles wholly inside the detector (all but the last tile row and
  // column) run the loop without the per-pixel validity tests
  auto orient_loop = [&](auto all_valid) {
    constexpr bool AV = decltype(all_valid)::value;
    for (int c0 = 0; c0 < a.n_orient; c0 += kDetChunk) {
      const int nc = min(kDetChunk, a.n_orient - c0);
      __syncthreads();
      for (int t = threadIdx.x; t < nc * 3; t += kPlThreads)
        reinterpret_cast<float4 *>(s_ot)[t] = reinterpret_cast<const float4 *>(ot + c0)[t];
      __syncthreads();
      // groups of kDetFlush orientations (chunks start at multiples of it),
      // two per loop trip, flushed to float64 after each full group
      for (int g0 = 0; g0 < nc; g0 += kDetFlush) {
        const int ge = min(g0 + kDetFlush, nc);
        // bit (oo - g0) KP + k: a sample whose index is not certain in
        // float32, replayed in float64 after the group
        unsigned need_bits = 0;
  #pragma unroll 2
        for (int oo = g0; oo < ge; ++oo) {
          // three 16-byte loads; each holds two (u, v) pairs
          const float4 *q = reinterpret_cast<const float4 *>(s_ot + oo);
          const float4 q0 = q[0], q1 = q[1], q2 = q[2];
          PlaneOrient T;
          T.x = make_float2(q0.x, q0.y);
          T.y = make_float2(q0.z, q0.w);
          T.z = make_float2(q1.x, q1.y);
          T.c = make_float2(q1.z, q1.w);
          T.d = make_float2(q2.x, q2.y);
          T.w = q2.z;
  #pragma unroll
          for (int k = 0; k < KP; ++k) {
            int iu, iv;
            const bool ok = plane_index<ZX>(T, n1, make_float2(xf[k], xf[k]),
                                            make_float2(yf[k], yf[k]),
                                            make_float2(zf[k], zf[k]), iu, iv);
            if ((AV || valid[k]) && ok)
              part[k] = fmaf(SMEM ? src[iu * pa.nv + iv] : __ldg(src + iu * pa.nv + iv), T.w,
                             part[k]);
            need_bits |= (unsigned)((AV || valid[k]) && !ok) << ((oo - g0) * KP + k);
          }
        }
        // the group's uncertain samples go to the worklist (replayed exactly
        // by k_detector_fix), or, once it is full, are replayed here into the
        // float64 accumulator
        if (__any_sync(0xffffffffu, need_bits != 0)) {
          while (need_bits) {
            const int b = __ffs(need_bits) - 1;
            need_bits &= need_bits - 1;
            const int k = b % KP, o = c0 + g0 + b / KP;
            int px = pix[0];
  #pragma unroll
            for (int q = 1; q < KP; ++q)
              if (k == q) px = pix[q];
            const int slot = atomicAdd(wl_count, 1);
            if (slot < wl_cap) {
              wl[slot] = make_int2(px, o);
            } else {
              double x, y, z;
              base_point(a, px / a.nh, px % a.nh, x, y, z);
              const double sv = (double)__ldg(a.iq + gather_index(a, o, x, y, z)) * a.w[o];
  #pragma unroll
              for (int q = 0; q < KP; ++q)
                if (k == q) acc[q] += sv;
            }
          }
        }
        if (ge - g0 == kDetFlush) {
  #pragma unroll
          for (int k = 0; k < KP; ++k) { acc[k] += f2d_exact(part[k]); part[k] = 0.f; }
        }
      }
    }
  };
  const int tile_i = (blockIdx.x / tiles_x) * kPlTH, tile_j = (blockIdx.x % tiles_x) * kPlTW;
  if (tile_i + kPlTH <= a.nv && tile_j + kPlTW <= a.nh) orient_loop(BoolC<true>{});
  else orient_loop(BoolC<false>{});
#pragma unroll
  for (int k = 0; k < KP; ++k)
    if (valid[k]) acc_out[pix[k]] = acc[k] + f2d_exact(part[k]);
}

// Exact float64 replay of the worklist's (pixel, orientation) pairs.
__global__ void k_detector_fix(DetArgs a, const int2 *wl, const int *wl_count,
                               int wl_cap, double *acc) {
  const int n = min(*wl_count, wl_cap);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x) {
    const int2 it = wl[e];
    double x, y, z;
    base_point(a, it.x / a.nh, it.x % a.nh, x, y, z);
    const float v = __ldg(a.iq + gather_index(a, it.y, x, y, z));
    atomicAdd(acc + it.x, (double)v * a.w[it.y]);
  }
}

// ------------------------------------------------------------------ adjoint
// Transpose of the epilogue: the image is out = 1e-6 * max'(mirror(acc))
// with max' the NaN/<=0 -> 1e-6 clamp (zero derivative where it acts) and
// mirror the sum over the four flips (a symmetric map: each output pixel
// sums its orbit under the flips, with multiplicity).  Hence
// dL/dacc[p] = 1e-6 * [v_p > 0] * sum over the flips q of p of dL/dout[q],
// v = mirror(acc) being constant on the orbit.
__global__ void k_det_epi_adj(const double *acc, const double *gout, int nv,
                              int nh, int mirror, double *gpix) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= nv * nh) return;
  const int i = pix / nh, j = pix % nh;
  const int i2 = nv - 1 - i, j2 = nh - 1 - j;
  const size_t q0 = (size_t)i * nh + j, q1 = (size_t)i * nh + j2,
               q2 = (size_t)i2 * nh + j, q3 = (size_t)i2 * nh + j2;
  double v, g;
  if (mirror) {
    v = ((acc[q0] + acc[q1]) + acc[q2]) + acc[q3];
    g = gout[q0] + gout[q1] + gout[q2] + gout[q3];
  } else {
    v = acc[q0];
    g = gout[q0];
  }
  gpix[pix] = (v == v && v > 0.0) ? 1e-6 * g : 0.0;
}

// Transpose of the orientation sum: every (pixel, orientation) sample adds
// w_o dL/dacc[pixel] to dL/dI at the voxel it gathered.  Indices come from
// the same float32 estimate with exact float64 replay as the forward (the
// ambiguous samples are replayed inline), so they are the forward's.
__global__ void __launch_bounds__(kDetThreads)
k_detector_adj(DetArgs a, const OrientFast *ot, const double *gpix,
               double *g_iq) {
  __shared__ OrientFast s_ot[kDetChunk];
  const int npx = a.nh * a.nv;
  const int pix = blockIdx.x * kDetThreads + threadIdx.x;
  const bool valid = pix < npx;
  double x0 = 0.0, y0 = 0.0, z0 = 0.0, g = 0.0;
  if (valid) {
    base_point(a, pix / a.nh, pix % a.nh, x0, y0, z0);
    g = gpix[pix];
  }
  const bool live = valid && g != 0.0;
  const float xf = (float)x0, yf = (float)y0, zf = (float)z0;
  for (int c0 = 0; c0 < a.n_orient; c0 += kDetChunk) {
    const int nc = min(kDetChunk, a.n_orient - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc * kOrientFloats; t += kDetThreads)
      reinterpret_cast<float *>(s_ot)[t] = reinterpret_cast<const float *>(ot + c0)[t];
    __syncthreads();
    if (!live) continue;
    for (int oo = 0; oo < nc; ++oo) {
      const int o = c0 + oo;
      int64_t idx;
      if (!fast_index(s_ot[oo], a, xf, yf, zf, idx))
        idx = gather_index(a, o, x0, y0, z0);
      atomicAdd(g_iq + idx, g * a.w[o]);
    }
  }
}

// Exact-path adjoint (plans built with exact indices).
__global__ void k_detector_adj_exact(DetArgs a, const double *gpix,
                                     double *g_iq) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.nh * a.nv) return;
  const double g = gpix[pix];
  if (g == 0.0) return;
  double x0, y0, z0;
  base_point(a, pix / a.nh, pix % a.nh, x0, y0, z0);
  for (int o = 0; o < a.n_orient; ++o)
    atomicAdd(g_iq + gather_index(a, o, x0, y0, z0), g * a.w[o]);
}

__global__ void k_det_debug_fast(DetArgs a, const OrientFast *ot, int o,
                                 int64_t *idx) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.nh * a.nv) return;
  double x, y, z;
  base_point(a, pix / a.nh, pix % a.nh, x, y, z);
  int64_t k;
  if (!fast_index(ot[o], a, (float)x, (float)y, (float)z, k))
    k = gather_index(a, o, x, y, z);
  idx[pix] = k;
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
  OrientFast *d_ot = nullptr;   // fast-path orientation table
  int2 *d_wl = nullptr;         // exact-replay worklist
  int *d_wl_count = nullptr;
  int wl_cap = 0;
  double *d_gout = nullptr, *d_gpix = nullptr, *d_giq = nullptr;  // adjoint
  PlaneArgs plane{-1, -1, 0, 0, 0, 0, nullptr};  // plane mode when fa >= 0
  float *d_plane = nullptr;
  PlaneOrient *d_po = nullptr;
  bool zero_x = false;  // every pixel's x is +-0 after the init rotations
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
  if (!p->exact) {
    // corners of the base plane after the initial rotations bound |p0|
    double pmax[3] = {0, 0, 0};
    const double hs[2] = {h_axis[0], h_axis[p->n_h - 1]};
    const double vs[2] = {v_axis[0], v_axis[p->n_v - 1]};
    for (double hh : hs)
      for (double vv : vs) {
        double c[3] = {0.0, hh, vv};
        for (int k = 0; k < n_init; ++k) {
          const double *R = init_R + 9 * k;
          const double a0 = rot_chain(R, c[0], c[1], c[2]);
          const double a1 = rot_chain(R + 3, c[0], c[1], c[2]);
          const double a2 = rot_chain(R + 6, c[0], c[1], c[2]);
          c[0] = a0; c[1] = a1; c[2] = a2;
        }
        for (int k = 0; k < 3; ++k) pmax[k] = std::max(pmax[k], std::fabs(c[k]) * (1 + 1e-12));
      }
    const double inv_dq = 1.0 / p->dq;
    const double qmin[3] = {p->qmin_x, p->qmin_y, p->qmin_z};
    const int dims[3] = {p->iq_shape[1], p->iq_shape[0], p->iq_shape[2]};  // x, y, z
    // Axes whose coordinate is exactly +-0 for every pixel: the plane starts
    // at x = 0 (detector.py:27); a rotation keeps output c at +-0 when each
    // of its row-c entries is 0 or multiplies a coordinate that is +-0
    // (fma of exact zeros).  Such an axis gathers index floor((0-qmin)/dq),
    // a constant; deciding it in float32 would be ambiguous whenever q=0
    // lies on a voxel boundary.
    auto propagate = [](const double *R, const bool in[3], bool out[3]) {
      for (int c = 0; c < 3; ++c) {
        bool z = true;
        for (int k = 0; k < 3; ++k) z = z && (R[3 * c + k] == 0.0 || in[k]);
        out[c] = z;
      }
    };
    bool zero0[3] = {true, false, false};
    for (int k = 0; k < n_init; ++k) {
      bool nz[3];
      propagate(init_R + 9 * k, zero0, nz);
      std::copy(nz, nz + 3, zero0);
    }
    P->zero_x = zero0[0];
    std::vector<OrientFast> ot(n_orient);
    for (int o = 0; o < n_orient; ++o) {
      bool zero[3] = {zero0[0], zero0[1], zero0[2]};
      for (int r = 0; r < rn[o]; ++r) {
        bool nz[3];
        propagate(rot_R + 9 * (rs[o] + r), zero, nz);
        std::copy(nz, nz + 3, zero);
      }
      for (int c = 0; c < 3; ++c) {
        ot[o].fix[c] = -1;
        if (zero[c]) {
          double k = floor_div_exact(0.0 - qmin[c], p->dq, inv_dq);
          k = std::min(std::max(k, 0.0), (double)(dims[c] - 1));
          ot[o].fix[c] = (int)k;
        }
      }
      ot[o].pad = 0;
      double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
      for (int r = 0; r < rn[o]; ++r) {
        const double *R = rot_R + 9 * (rs[o] + r);
        double T[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            T[3 * i + j] = R[3 * i] * M[j] + R[3 * i + 1] * M[3 + j] + R[3 * i + 2] * M[6 + j];
        std::copy(T, T + 9, M);
      }
      for (int c = 0; c < 3; ++c) {
        double S = std::fabs(qmin[c] * inv_dq);
        for (int k = 0; k < 3; ++k) {
          ot[o].A[3 * c + k] = (float)(M[3 * c + k] * inv_dq);
          S += std::fabs(M[3 * c + k] * inv_dq) * pmax[k];
        }
        ot[o].b[c] = (float)(-qmin[c] * inv_dq);
        ot[o].d[c] = (float)(10.0 * std::ldexp(1.0, -24) * S + 1e-5);
      }
      ot[o].w = (float)weights[o];
    }
    const int64_t pairs = (int64_t)npx * n_orient;
    P->wl_cap = (int)std::max<int64_t>(1 << 16, std::min<int64_t>(pairs / 8, 1 << 26));
    // GW_DET_WORKLIST_CAP shrinks the worklist (tests use it to exercise the
    // in-kernel exact path taken when the list is full)
    if (const char *cap = getenv("GW_DET_WORKLIST_CAP")) P->wl_cap = std::max(1, atoi(cap));
    if ((st = up(&P->d_ot, ot.data(), ot.size()))) {
      gw_detector_plan_destroy(P);
      return st;
    }
    e = gw::dev_malloc((void **)&P->d_wl, (size_t)P->wl_cap * sizeof(int2));
    if (e == cudaSuccess) e = gw::dev_malloc((void **)&P->d_wl_count, sizeof(int));
    if (e != cudaSuccess) {
      gw_detector_plan_destroy(P);
      return gw::cuda_fail(e, "detector worklist", __FILE__, __LINE__);
    }
    // plane mode: one axis at the same fixed index in every orientation
    if (p->accum != GW_ACCUM_KAHAN32 && !p->no_plane) {
      for (int c = 0; c < 3 && P->plane.fa < 0; ++c) {
        bool same = true;
        for (int o = 0; o < n_orient && same; ++o)
          same = ot[o].fix[c] >= 0 && ot[o].fix[c] == ot[0].fix[c];
        if (!same) continue;
        // free axes in memory order (y, x, z)
        const int order[3] = {1, 0, 2};
        int fr[2], k = 0;
        for (int q : order)
          if (q != c) fr[k++] = q;
        PlaneArgs pa{c, ot[0].fix[c], fr[0], fr[1], dims[fr[0]], dims[fr[1]], nullptr};
        e = gw::dev_malloc((void **)&P->d_plane, (size_t)pa.nu * pa.nv * sizeof(float));
        if (e != cudaSuccess) {
          gw_detector_plan_destroy(P);
          return gw::cuda_fail(e, "detector plane", __FILE__, __LINE__);
        }
        pa.P = P->d_plane;
        P->plane = pa;
        std::vector<PlaneOrient> po(n_orient);
        for (int o = 0; o < n_orient; ++o) {
          const OrientFast &T = ot[o];
          po[o].x = make_float2(T.A[3 * pa.ua], T.A[3 * pa.va]);
          po[o].y = make_float2(T.A[3 * pa.ua + 1], T.A[3 * pa.va + 1]);
          po[o].z = make_float2(T.A[3 * pa.ua + 2], T.A[3 * pa.va + 2]);
          po[o].c = make_float2(T.b[pa.ua], T.b[pa.va]);
          po[o].d = make_float2(T.d[pa.ua], T.d[pa.va]);
          po[o].w = T.w;
          po[o].pad = 0.f;
        }
        if ((st = up(&P->d_po, po.data(), po.size()))) {
          gw_detector_plan_destroy(P);
          return st;
        }
      }
    }
  }
  *out = P;
  return GW_OK;
}

extern "C" int gw_detector_plan_destroy(gw_detector_plan *P) {
  if (!P) return GW_OK;
  void *ptrs[] = {P->d_h, P->d_v, P->d_init, P->d_rot, P->d_w, P->d_rs,
                  P->d_rn, P->d_iq_own, P->d_acc, P->d_out, P->d_ot, P->d_wl,
                  P->d_wl_count, P->d_gout, P->d_gpix, P->d_giq, P->d_plane,
                  P->d_po};
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
  gw::Range r("giwaxsim: detector image");
  const int npx = P->p.n_h * P->p.n_v;
  DetArgs a = det_args(P);
  if (P->p.exact) {
    gw::KTimer tm(P->ctx, GW_K_DETECTOR);
    k_detector<<<(npx + 127) / 128, 128, 0, P->ctx->stream>>>(a, P->d_acc);
    GW_LAUNCHED(P->ctx);
  } else {
    GW_CUDA(cudaMemsetAsync(P->d_wl_count, 0, sizeof(int), P->ctx->stream));
    if (P->plane.fa >= 0) {
      const PlaneArgs &pa = P->plane;
      {
        gw::KTimer tm(P->ctx, GW_K_MISC);
        const int64_t n = (int64_t)pa.nu * pa.nv;
        k_plane_extract<<<(int)std::min<int64_t>((n + 255) / 256, 4 * P->ctx->sm_count),
                          256, 0, P->ctx->stream>>>(a, pa, P->d_plane);
        GW_LAUNCHED(P->ctx);
      }
      const size_t smem = (size_t)pa.nu * pa.nv * sizeof(float);
      const int tiles = ((P->p.n_h + kPlTW - 1) / kPlTW) * ((P->p.n_v + kPlTH - 1) / kPlTH);
      gw::KTimer tm(P->ctx, GW_K_DETECTOR);
      if (smem <= kPlaneSmemMax) {
        static gw::SmemRecord attr_zx, attr_gen;
        GW_TRY(gw::smem_limit(attr_zx, k_detector_plane<true, true>, kPlaneSmemMax));
        GW_TRY(gw::smem_limit(attr_gen, k_detector_plane<true, false>, kPlaneSmemMax));
        if (P->zero_x)
          k_detector_plane<true, true><<<tiles, kPlThreads, smem, P->ctx->stream>>>(
              a, P->d_po, pa, P->d_acc, P->d_wl, P->d_wl_count, P->wl_cap);
        else
          k_detector_plane<true, false><<<tiles, kPlThreads, smem, P->ctx->stream>>>(
              a, P->d_po, pa, P->d_acc, P->d_wl, P->d_wl_count, P->wl_cap);
      } else if (P->zero_x) {
        k_detector_plane<false, true><<<tiles, kPlThreads, 0, P->ctx->stream>>>(
            a, P->d_po, pa, P->d_acc, P->d_wl, P->d_wl_count, P->wl_cap);
      } else {
        k_detector_plane<false, false><<<tiles, kPlThreads, 0, P->ctx->stream>>>(
            a, P->d_po, pa, P->d_acc, P->d_wl, P->d_wl_count, P->wl_cap);
      }
      GW_LAUNCHED(P->ctx);
    } else {
      gw::KTimer tm(P->ctx, GW_K_DETECTOR);
      const int per = kDetThreads * kDetPix;
      k_detector_fast<<<(npx + per - 1) / per, kDetThreads, 0, P->ctx->stream>>>(
          a, P->d_ot, P->d_acc, P->d_wl, P->d_wl_count, P->wl_cap);
      GW_LAUNCHED(P->ctx);
    }
    gw::KTimer tm(P->ctx, GW_K_DET_FIX);
    k_detector_fix<<<2 * P->ctx->sm_count, 256, 0, P->ctx->stream>>>(
        a, P->d_wl, P->d_wl_count, P->wl_cap, P->d_acc);
    GW_LAUNCHED(P->ctx);
  }
  gw::KTimer tm(P->ctx, GW_K_DET_EPI);
  k_det_epilogue<<<(npx + 255) / 256, 256, 0, P->ctx->stream>>>(
      P->d_acc, P->p.n_v, P->p.n_h, P->p.mirror, P->d_out);
  GW_LAUNCHED(P->ctx);
  P->executed = true;
  return GW_OK;
}

extern "C" int gw_detector_device_out(gw_detector_plan *P, const double **out) {
  if (!P || !out) return gw::fail(GW_ERR_ARG, "gw_detector_device_out: null argument");
  *out = P->d_out;
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

extern "C" int gw_detector_backward(gw_detector_plan *P, const double *g_out,
                                    int32_t out_on_device, double *g_iq,
                                    int32_t iq_on_device) {
  if (!P || !g_out || !g_iq)
    return gw::fail(GW_ERR_ARG, "gw_detector_backward: null argument");
  if (!P->executed)
    return gw::fail(GW_ERR_STATE, "gw_detector_backward: plan not executed");
  GW_CUDA(cudaSetDevice(P->ctx->device));
  const int npx = P->p.n_h * P->p.n_v;
  const size_t niq = (size_t)P->p.iq_shape[0] * P->p.iq_shape[1] * P->p.iq_shape[2];
  cudaStream_t st = P->ctx->stream;
  if (!P->d_gpix) {
    GW_CUDA(gw::dev_malloc((void **)&P->d_gpix, npx * sizeof(double)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_gout, npx * sizeof(double)));
  }
  const double *gout = g_out;
  if (!out_on_device) {
    GW_CUDA(cudaMemcpyAsync(P->d_gout, g_out, npx * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    gout = P->d_gout;
  }
  double *giq = g_iq;
  if (!iq_on_device) {
    if (!P->d_giq) GW_CUDA(gw::dev_malloc((void **)&P->d_giq, niq * sizeof(double)));
    giq = P->d_giq;
  }
  GW_CUDA(cudaMemsetAsync(giq, 0, niq * sizeof(double), st));
  {
    gw::KTimer tm(P->ctx, GW_K_DET_EPI);
    k_det_epi_adj<<<(npx + 255) / 256, 256, 0, st>>>(P->d_acc, gout, P->p.n_v,
                                                     P->p.n_h, P->p.mirror, P->d_gpix);
    GW_LAUNCHED(P->ctx);
  }
  DetArgs a = det_args(P);
  {
    gw::KTimer tm(P->ctx, GW_K_DETECTOR);
    if (P->p.exact)
      k_detector_adj_exact<<<(npx + 127) / 128, 128, 0, st>>>(a, P->d_gpix, giq);
    else
      k_detector_adj<<<(npx + kDetThreads - 1) / kDetThreads, kDetThreads, 0, st>>>(
          a, P->d_ot, P->d_gpix, giq);
    GW_LAUNCHED(P->ctx);
  }
  if (!iq_on_device)
    GW_CUDA(cudaMemcpyAsync(g_iq, giq, niq * sizeof(double), cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaStreamSynchronize(st));
  return gw::check_device_error(P->ctx, "detector backward");
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
  if (P->p.exact)
    k_det_debug<<<(npx + 255) / 256, 256, 0, P->ctx->stream>>>(a, orient, d);
  else
    k_det_debug_fast<<<(npx + 255) / 256, 256, 0, P->ctx->stream>>>(a, P->d_ot, orient, d);
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
    // counts come from caller memory the host cannot check: clamp them to
    // the documented 0..3, so that `start` only moves forward by at most 3
    const int n = min(max(n_rot[o], 0), 3);
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
