// Adjoint of the batched voxel stage: given dL/dI(q) on the cropped cube,
// the gradient of L with respect to the deposited scattering factor of
// every atom, the smoothing sigma, the background constant of every
// structure and (bilinear deposit) the atom coordinates.
//
// Forward model per slice (tools/voxelgrids.py:318-416 with fill_bkg off,
// batched formulation of gw_voxel.cu):
//   D[z,y] = (dep[z,y] - c) * m_z[z] m_y[y]        (smoothing on; D = dep off)
//   F[k]   = sum_{z,y} D[z,y] W^{kz z + ky y} + c g^2 [k = 0]
//   sum[v] += |F[k]|^2 for the pixels k binned into voxel v
//   I[v]   = sum[v] * s[v]   (1/count, f0 factor, 1/structures)
// Adjoint, slice by slice (the slices are recomputed from the atoms, never
// stored: the batch size is the checkpoint interval):
//   G_sum = G_I * s                                   k_fin_adj
//   G_F   = 2 F G_sum[bin(k)]                         k_col_bwd (gather)
//   G_D   = sum_k G_F[k] W^{-(kz z + ky y)}           k_col_bwd + k_row_bwd
//           (inverse transform restricted to the window: the conjugate of a
//            chirp-z transform from the kept band to the window)
//   dL/d f_a  = sum_slices w_a G_D m    (gather at the atom's cells)
//   dL/d sigma, dL/dc, dL/d xyz         per-row and per-atom reductions
// All gradients with respect to complex quantities are dL/dRe + i dL/dIm.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "gw_voxel_impl.cuh"

using namespace gwv;

namespace {

// per-slice float64 scalars
enum {
  SC_DC_RE = 0, SC_DC_IM,    // g^2 G_F[0,0]
  SC_SM_RE, SC_SM_IM,        // sum G_D m
  SC_SDM_RE, SC_SDM_IM,      // sum G_D dm/dsigma
  SC_SIG_AT,                 // sum over atoms Re(conj(G_D) f_s) w dm/dsigma
  SC_SU,                     // sum over atoms dL/dy' (shift to the minimum)
  SC_SV,                     // sum over atoms dL/dz
  SC_N
};

}  // namespace

struct gw_grad_state {
  float2 *d_Ay = nullptr, *d_Hy = nullptr, *d_By = nullptr;  // band -> y window
  float2 *d_Az = nullptr, *d_Hz = nullptr, *d_Bz = nullptr;  // band -> z window
  float *d_dgw = nullptr;          // d(gaussian weights)/d sigma
  float *d_dmy = nullptr, *d_dmz = nullptr;
  float *d_gsum = nullptr;         // W^3 dL/dsum
  double *d_giq = nullptr;         // Qc^3 staging of a host dL/dI
  float2 *d_G1 = nullptr;          // [slot][Nc][Lz] column-stage adjoint
  double2 *d_gacc = nullptr;       // per sorted atom dL/d f
  double *d_gxyz = nullptr;        // per sorted atom dL/d xyz (bilinear)
  double2 *d_out_f = nullptr;      // input order
  double *d_out_xyz = nullptr;
  double *d_sc = nullptr;          // [n_slices][SC_N]
  int *d_amy = nullptr, *d_amz = nullptr;  // argmin of y' per slice, z per structure
  int64_t n_atoms = -1;
};

namespace gwv {
void grad_state_destroy(gw_grad_state *g) {
  if (!g) return;
  void *ptrs[] = {g->d_Ay, g->d_Hy, g->d_By, g->d_Az, g->d_Hz, g->d_Bz,
                  g->d_dgw, g->d_dmy, g->d_dmz, g->d_gsum, g->d_giq, g->d_G1,
                  g->d_gacc, g->d_gxyz, g->d_out_f, g->d_out_xyz, g->d_sc,
                  g->d_amy, g->d_amz};
  for (void *q : ptrs) gw::dev_free(q);
  delete g;
}
}  // namespace gwv

namespace {

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// Re(conj(a) b)
__device__ __forceinline__ float redot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }

// dL/dsum on the batched window (= the crop) from dL/dI, with the scale the
// forward's k_finalize applies (count, f0 factor, structure average).
__global__ void k_fin_adj(const double *g_iq, const unsigned int *C2,
                          const int *C1, int W, int off, int Qc,
                          float inv_nstruct, const float *f0tab, int use_f0,
                          float f0_c, float f0_invz, float *gsum) {
  const int line = blockIdx.x;
  const int iy = line / Qc, ix = line - iy * Qc;
  const int wy = iy + off, wx = ix + off;
  const unsigned c2 = C2[(size_t)wy * W + wx];
  const size_t wbase = ((size_t)wy * W + wx) * W + off;
  const size_t obase = (size_t)line * Qc;
  float fxy[4];
  if (use_f0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float *t = f0tab + i * 3 * Qc;
      fxy[i] = t[ix] * t[Qc + iy];
    }
  }
  const float r2 = line_count_factor(c2, inv_nstruct);
  for (int iz = threadIdx.x; iz < Qc; iz += blockDim.x) {
    float scale = r2 * z_count_factor((unsigned)C1[iz + off]);
    if (use_f0) {
      float acc = f0_c;
#pragma unroll
      for (int i = 0; i < 4; ++i) acc += fxy[i] * f0tab[(i * 3 + 2) * Qc + iz];
      const float fq = acc * f0_invz;
      scale *= fq * fq;
    }
    gsum[wbase + iz] = (float)(g_iq[obase + iz] * (double)scale);
  }
}

// sigma derivative of the smoothing profiles of slices [slice0, slice0+n)
__global__ void k_dprofile(SliceArgs a, int slice0, const float *dgw,
                           float *dmy, float *dmz) {
  const int sl = slice0 + blockIdx.x;
  const int4 e = a.ext[sl];
  if (e.y < 0) return;
  int ys, ye, zs, ze;
  plateau(a, e, ys, ye, zs, ze);
  for (int yy = threadIdx.x; yy < a.Ly; yy += blockDim.x) {
    int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
    dmy[(size_t)blockIdx.x * a.Ly + yy] = smooth_at(yi, ys, ye, a.g, a.radius, dgw);
  }
  for (int zz = threadIdx.x; zz < a.Lz; zz += blockDim.x) {
    int zi = a.z_lo + zz; if (zi < 0) zi += a.g; if (zi >= a.g) zi -= a.g;
    dmz[(size_t)blockIdx.x * a.Lz + zz] = smooth_at(zi, zs, ze, a.g, a.radius, dgw);
  }
}

// Input index of the atom at the minimum rotated y of each slice (ties: the
// smallest index) -- the atom the shift to the minimum follows.
__global__ void k_argmin_y(SliceArgs a, int slice0, const int *perm, int *amy) {
  const int sl = slice0 + blockIdx.y;
  const int t = sl / a.n_phi, p = sl % a.n_phi;
  const gw_structure s = a.st[t];
  const unsigned long long mn = a.ymin_ord[sl];
  const double c = a.ph[p].cos_phi, sn = a.ph[p].sin_phi;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = s.atom_begin + i;
    if (dbl_ord(rot_y(a.xyz_s + 3 * pos, c, sn)) == mn) atomicMin(amy + sl, perm[pos]);
  }
}

__global__ void k_argmin_z(const double *xyz_s, const gw_structure *st,
                           const unsigned long long *zmin_ord, const int *perm,
                           int *amz) {
  const gw_structure s = st[blockIdx.y];
  const unsigned long long mn = zmin_ord[blockIdx.y];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = s.atom_begin + i;
    if (dbl_ord(xyz_s[3 * pos + 2]) == mn) atomicMin(amz + blockIdx.y, perm[pos]);
  }
}

// ------------------------------------------------------------ column stage
struct ColLoadF1 {
  const float2 *src, *A;
  int L, nc, m0;
  __device__ float2 operator()(int f, int n) const {
    if (n >= L || m0 + f >= nc) return make_float2(0.f, 0.f);
    return cmul(src[(size_t)n * nc + m0 + f], __ldg(A + n));
  }
};

// conj(B' v) -> G1 stored column-major per slice: [col][z]
struct ColStoreAdj {
  const float2 *B;
  float2 *G1;  // slice base
  int Lz, nc, m0;
  __device__ void operator()(int f, int j, float2 v) const {
    const int m = m0 + f;
    if (j < Lz && m < nc) G1[(size_t)m * Lz + j] = conjf2(cmul(v, __ldg(B + j)));
  }
};

struct GradCol {
  const float *gsum;
  const float2 *Aa, *Ha, *Ba;  // adjoint z tables (band -> window)
  float2 *G1;
  double *sc;
  float dc2;
};

// NB columns of one slice: recompute F along z from F1 (forward chirp-z),
// form G_F = 2 F dL/dsum[bin] on the binned pixels, and transform G_F back
// to the z window (adjoint chirp-z), leaving G1[col][z].
template <int M>
__global__ void __launch_bounds__(FftShape<M>::NT, FftShape<M>::MINB)
k_col_bwd(SliceArgs a, CztArgs cz, BinArgs bn, GradCol gc, int slice0, int nc,
          const float2 *F1) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  constexpr int TWL = FftPlan<M>::tw_len();
  constexpr int LDM = FftPlan<M>::LDM;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *buf = smem + TWL;
  const int slot = blockIdx.y, sl = slice0 + slot;
  const int p = sl % a.n_phi;
  const int m0 = blockIdx.x * NB;
  const int *cofs = bn.colofs + (size_t)p * nc;
  for (int t = threadIdx.x; t < TWL; t += NT) tw[t] = cz.tw[t];
  __syncthreads();
  int first, rows;
  slice_rows(a, slice0, sl, first, rows);
  ColLoadF1 ld{F1 + (size_t)first * nc, cz.A, rows, nc, m0};
  fft_run<M, NB, NT, false, 1, false, 0, true>(buf, tw, nullptr, ld, NoStore());
  fft_run<M, NB, NT, true, 0, true, 0, false>(buf, tw, cz.H, NoLoad(), NoStore());
  const float2 cbg = slice_const(a, sl).cbg;
  for (int t = threadIdx.x; t < NB * M; t += NT) {
    const int f = t / M, mr = t - f * M;
    const int m = m0 + f;
    float2 out = make_float2(0.f, 0.f);
    if (mr < cz.N && m < nc) {
      const int co = cofs[m], ro = bn.rowofs[mr];
      if (co >= 0 && ro >= 0) {
        float2 X = cmul(buf[f * LDM + fft_pad(mr)], __ldg(cz.B + mr));
        const bool dc = bn.k0 + m == 0 && bn.kz0 + mr == 0;
        if (dc) {
          X.x += cbg.x * bn.dc_scale;
          X.y += cbg.y * bn.dc_scale;
        }
        const float gi = 2.f * gc.gsum[co + ro];
        const float2 GF = make_float2(gi * X.x, gi * X.y);
        if (dc) {
          atomicAdd(gc.sc + (size_t)sl * SC_N + SC_DC_RE, (double)GF.x * gc.dc2);
          atomicAdd(gc.sc + (size_t)sl * SC_N + SC_DC_IM, (double)GF.y * gc.dc2);
        }
        out = cmul(conjf2(GF), __ldg(gc.Aa + mr));
      }
    }
    buf[f * LDM + fft_pad(mr)] = out;
  }
  __syncthreads();
  fft_run<M, NB, NT, false, 0, false, 0, false>(buf, tw, nullptr, NoLoad(), NoStore());
  ColStoreAdj st{gc.Ba, gc.G1 + (size_t)slot * a.Lz * nc, a.Lz, nc, m0};
  fft_run<M, NB, NT, true, 0, true, 1, false>(buf, tw, gc.Ha, NoLoad(), st);
}

// ------------------------------------------------------------ row stage
struct GradRow {
  const float2 *Aa, *Ha, *Ba, *tw;  // adjoint y tables (band -> window)
  const float2 *G1;
  const float *dmy, *dmz;
  double2 *gacc;
  double *gxyz;
  double *sc;
  int nc;
};

template <int M>
struct RowLoadAdj {
  const float2 *G1, *Aa;  // by value: no reads through the parameters
  int nc, Lz;
  const int *r_slot, *r_zz;
  int row0, n_rows;
  __device__ float2 operator()(int f, int n) const {
    const int row = row0 + f;
    if (row >= n_rows || n >= nc) return make_float2(0.f, 0.f);
    const int slot = r_slot[f], zz = r_zz[f];
    const float2 g = G1[((size_t)slot * nc + n) * Lz + zz];
    return cmul(conjf2(g), __ldg(Aa + n));
  }
};

// NB window rows: transform G1 back to the y window (G_D), then the atoms of
// the rows gather G_D at their cells; per-row sums go to the slice scalars.
template <int M, bool BIL>
__global__ void __launch_bounds__(FftShape<M>::NT, FftShape<M>::MINB)
k_row_bwd(SliceArgs a, GradRow gr, int slice0, int n_sl, int n_rows) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  constexpr int TWL = FftPlan<M>::tw_len();
  constexpr int LDM = FftPlan<M>::LDM;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *buf = smem + TWL;
  __shared__ int r_lo[NB], r_mid[NB], r_cnt[NB + 1], r_slot[NB], r_zz[NB];
  __shared__ float racc[NB][7];
  for (int t = threadIdx.x; t < TWL; t += NT) tw[t] = gr.tw[t];
  const int row0 = blockIdx.x * NB;
  for (int t = threadIdx.x; t < NB * 7; t += NT) racc[t / 7][t % 7] = 0.f;
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int f = 0; f < NB; ++f) {
      const int row = row0 + f;
      int lo = 0, mid = 0, hi = 0, slot = 0, zz = 0;
      if (row < n_rows) {
        row_slot(a, slice0, n_sl, row, slot, zz);
        const int sl = slice0 + slot, t = sl / a.n_phi;
        row_atoms(a, t, zz, lo, mid, hi);
      }
      r_lo[f] = lo;
      r_mid[f] = mid;
      r_cnt[f] = acc;
      r_slot[f] = slot;
      r_zz[f] = zz;
      acc += hi - lo;
    }
    r_cnt[NB] = acc;
  }
  __syncthreads();
  RowLoadAdj<M> ld{gr.G1, gr.Aa, gr.nc, a.Lz, r_slot, r_zz, row0, n_rows};
  fft_run<M, NB, NT, false, 1, false, 0, true>(buf, tw, nullptr, ld, NoStore());
  fft_run<M, NB, NT, true, 0, true, 0, false>(buf, tw, gr.Ha, NoLoad(), NoStore());
  // G_D on the window, and the per-row sums of G_D m and G_D dm/dsigma
  for (int t = threadIdx.x; t < NB * a.Ly; t += NT) {
    const int f = t / a.Ly, yy = t - f * a.Ly;
    const int row = row0 + f;
    if (row >= n_rows) continue;
    float2 *q = buf + f * LDM + fft_pad(yy);
    const float2 v = conjf2(cmul(*q, __ldg(gr.Ba + yy)));
    *q = v;
    if (a.smooth_on) {
      const int slot = r_slot[f], zz = r_zz[f];
      const float mz = a.mz[(size_t)slot * a.Lz + zz], my = a.my[(size_t)slot * a.Ly + yy];
      const float dm = gr.dmz[(size_t)slot * a.Lz + zz] * my +
                       mz * gr.dmy[(size_t)slot * a.Ly + yy];
      const float m = mz * my;
      atomicAdd(&racc[f][0], v.x * m);
      atomicAdd(&racc[f][1], v.y * m);
      atomicAdd(&racc[f][2], v.x * dm);
      atomicAdd(&racc[f][3], v.y * dm);
    }
  }
  __syncthreads();
  const int total = r_cnt[NB];
  for (int i = threadIdx.x; i < total; i += NT) {
    int f = 0;
    while (f + 1 < NB && i >= r_cnt[f + 1]) ++f;
    const int at = r_lo[f] + (i - r_cnt[f]);
    const int slot = r_slot[f], zz = r_zz[f];
    const int sl = slice0 + slot;
    const float mz = a.smooth_on ? a.mz[(size_t)slot * a.Lz + zz] : 1.f;
    const float dmz = a.smooth_on ? gr.dmz[(size_t)slot * a.Lz + zz] : 0.f;
    const float4 q = a.xyf_s[at];
    const float2 fs = make_float2(q.z, q.w);
    if constexpr (!BIL) {
      int yy;
      if (!deposit_column(a, at, sl, yy) || yy >= a.Ly) continue;
      const float2 G = buf[f * LDM + fft_pad(yy)];
      float m = 1.f;
      if (a.smooth_on) {
        const float my = a.my[(size_t)slot * a.Ly + yy];
        m = mz * my;
        const float dm = dmz * my + mz * gr.dmy[(size_t)slot * a.Ly + yy];
        atomicAdd(&racc[f][4], redot(G, fs) * dm);
      }
      atomicAdd(&gr.gacc[at].x, (double)(G.x * m));
      atomicAdd(&gr.gacc[at].y, (double)(G.y * m));
    } else {
      int i0;
      float fu;
      if (!bilinear_column(a, at, sl, i0, fu)) continue;
      const bool own = at >= r_mid[f];  // this row holds the atom's lower z corner
      const float fz = a.fz_s[at];
      const float wz = own ? 1.f - fz : fz;
      float2 acc = make_float2(0.f, 0.f), du = acc, dv = acc;
      float sig = 0.f;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int ic = i0 + c;
        if (ic >= a.g) continue;
        const int yy = window_col(a, ic);
        if (yy >= a.Ly) continue;
        const float2 G = buf[f * LDM + fft_pad(yy)];
        float m = 1.f;
        if (a.smooth_on) {
          const float my = a.my[(size_t)slot * a.Ly + yy];
          m = mz * my;
          const float dm = dmz * my + mz * gr.dmy[(size_t)slot * a.Ly + yy];
          sig += (c ? fu : 1.f - fu) * dm * redot(G, fs);
        }
        const float wy = c ? fu : 1.f - fu, dwy = c ? 1.f : -1.f;
        const float2 Gm = make_float2(G.x * m, G.y * m);
        acc.x += wy * Gm.x; acc.y += wy * Gm.y;
        du.x += dwy * Gm.x; du.y += dwy * Gm.y;
        dv.x += wy * Gm.x; dv.y += wy * Gm.y;
      }
      if (a.smooth_on) atomicAdd(&racc[f][4], wz * sig);
      atomicAdd(&gr.gacc[at].x, (double)(wz * acc.x));
      atomicAdd(&gr.gacc[at].y, (double)(wz * acc.y));
      const gw_phi &ph = a.ph[sl % a.n_phi];
      const double gyp = (double)(wz * redot(du, fs)) * a.inv_r;   // dL/dy'
      const double gz = (double)((own ? -1.f : 1.f) * redot(dv, fs)) * a.inv_r;
      atomicAdd(gr.gxyz + 3 * (size_t)at, gyp * ph.sin_phi);
      atomicAdd(gr.gxyz + 3 * (size_t)at + 1, gyp * ph.cos_phi);
      atomicAdd(gr.gxyz + 3 * (size_t)at + 2, gz);
      atomicAdd(&racc[f][5], (float)gyp);
      atomicAdd(&racc[f][6], (float)gz);
    }
  }
  __syncthreads();
  if (threadIdx.x < NB) {
    const int f = threadIdx.x, row = row0 + f;
    if (row < n_rows) {
      const int sl = slice0 + r_slot[f];
      double *s = gr.sc + (size_t)sl * SC_N;
      if (a.smooth_on) {
        atomicAdd(s + SC_SM_RE, (double)racc[f][0]);
        atomicAdd(s + SC_SM_IM, (double)racc[f][1]);
        atomicAdd(s + SC_SDM_RE, (double)racc[f][2]);
        atomicAdd(s + SC_SDM_IM, (double)racc[f][3]);
        atomicAdd(s + SC_SIG_AT, (double)racc[f][4]);
      }
      if (BIL) {
        atomicAdd(s + SC_SU, (double)racc[f][5]);
        atomicAdd(s + SC_SV, (double)racc[f][6]);
      }
    }
  }
}

// sorted order -> input order
__global__ void k_unperm(int64_t n, const int *perm, const double2 *gacc,
                         const double *gxyz, double2 *out_f, double *out_xyz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int a = perm[i];
    out_f[a] = gacc[i];
    if (gxyz) {
      out_xyz[3 * (size_t)a] = gxyz[3 * i];
      out_xyz[3 * (size_t)a + 1] = gxyz[3 * i + 1];
      out_xyz[3 * (size_t)a + 2] = gxyz[3 * i + 2];
    }
  }
}

// ------------------------------------------------------------ launchers
template <int M>
size_t fft_smem() {
  return (size_t)(FftShape<M>::NB * FftPlan<M>::LDM + FftPlan<M>::tw_len()) * sizeof(float2);
}

template <int M>
int launch_col_bwd(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                   const BinArgs &bn, const GradCol &gc, int s0, int n) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = fft_smem<M>();
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_col_bwd<M>, smem));
  dim3 grid((P->Nc + NB - 1) / NB, n);
  gw::KTimer tm(P->ctx, GW_K_COLBIN);
  k_col_bwd<M><<<grid, NT, smem, P->ctx->stream>>>(a, cz, bn, gc, s0, P->Nc, P->d_F1);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M, bool BIL>
int launch_row_bwd_t(gw_voxel_plan *P, const SliceArgs &a, const GradRow &gr,
                     int s0, int n_sl) {
  const int n_rows = batch_rows(P, s0, n_sl);
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = fft_smem<M>();
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_row_bwd<M, BIL>, smem));
  gw::KTimer tm(P->ctx, GW_K_ROW);
  k_row_bwd<M, BIL><<<(n_rows + NB - 1) / NB, NT, smem, P->ctx->stream>>>(a, gr, s0, n_sl,
                                                                          n_rows);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M>
int launch_row_bwd(gw_voxel_plan *P, const SliceArgs &a, const GradRow &gr,
                   int s0, int n_sl) {
  return a.bil ? launch_row_bwd_t<M, true>(P, a, gr, s0, n_sl)
               : launch_row_bwd_t<M, false>(P, a, gr, s0, n_sl);
}

int col_bwd_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                     const BinArgs &bn, const GradCol &gc, int s0, int n) {
  GW_DISPATCH_M(P->Mz, launch_col_bwd, P, a, cz, bn, gc, s0, n)
}
int row_bwd_dispatch(gw_voxel_plan *P, const SliceArgs &a, const GradRow &gr,
                     int s0, int n_sl) {
  GW_DISPATCH_M(P->My, launch_row_bwd, P, a, gr, s0, n_sl)
}

int grad_state_init(gw_voxel_plan *P) {
  gw_grad_state *G = P->grad;
  if (!G) {
    G = new gw_grad_state();
    P->grad = G;
    size_t B = 0;
    // adjoint chirp-z: input positions are the kept frequencies, outputs
    // the real-space window; the convolution length is the forward one.
    CztTables ty = make_czt(P->g, P->k0, P->Nc, P->y_lo, P->Ly, P->My);
    CztTables tz = make_czt(P->g, P->kz0, P->Nr, P->z_lo, P->Lz, P->Mz);
    std::vector<float> dgw;
    const double sigma = P->p.smooth;
    if (sigma > 0) {
      std::vector<double> w(2 * P->radius + 1);
      double sum = 0, m2 = 0;
      for (int j = -P->radius; j <= P->radius; ++j) {
        w[j + P->radius] = std::exp(-0.5 / (sigma * sigma) * (double)j * j);
        sum += w[j + P->radius];
      }
      for (int j = -P->radius; j <= P->radius; ++j) {
        w[j + P->radius] /= sum;
        m2 += w[j + P->radius] * (double)j * j;
      }
      // d/dsigma of the normalised weights: w_j (j^2 - <k^2>) / sigma^3
      for (int j = -P->radius; j <= P->radius; ++j)
        dgw.push_back((float)(w[j + P->radius] * ((double)j * j - m2) /
                              (sigma * sigma * sigma)));
    }
    const size_t W3 = (size_t)P->W * P->W * P->W;
    const size_t Qc3 = (size_t)P->Qc * P->Qc * P->Qc;
    int st = GW_OK;
    if ((st = upload(&G->d_Ay, ty.A, &B)) || (st = upload(&G->d_Hy, ty.H, &B)) ||
        (st = upload(&G->d_By, ty.B, &B)) || (st = upload(&G->d_Az, tz.A, &B)) ||
        (st = upload(&G->d_Hz, tz.H, &B)) || (st = upload(&G->d_Bz, tz.B, &B)) ||
        (st = upload(&G->d_dgw, dgw, &B)) ||
        (st = alloc(&G->d_dmy, (size_t)P->S * P->Ly, &B)) ||
        (st = alloc(&G->d_dmz, (size_t)P->S * P->Lz, &B)) ||
        (st = alloc(&G->d_gsum, W3, &B)) || (st = alloc(&G->d_giq, Qc3, &B)) ||
        (st = alloc(&G->d_G1, (size_t)P->S * P->Lz * P->Nc, &B)) ||
        (st = alloc(&G->d_sc, (size_t)P->n_slices * SC_N, &B)) ||
        (st = alloc(&G->d_amy, P->n_slices, &B)) ||
        (st = alloc(&G->d_amz, P->n_struct, &B)))
      return st;
  }
  if (G->n_atoms != P->n_atoms) {
    void *old[] = {G->d_gacc, G->d_gxyz, G->d_out_f, G->d_out_xyz};
    for (void *q : old) gw::dev_free(q);
    G->d_gacc = nullptr; G->d_gxyz = nullptr; G->d_out_f = nullptr; G->d_out_xyz = nullptr;
    G->n_atoms = -1;
    size_t B = 0;
    const size_t n = (size_t)P->n_atoms;
    int st = GW_OK;
    if ((st = alloc(&G->d_gacc, n, &B)) || (st = alloc(&G->d_out_f, n, &B)) ||
        (P->bil && ((st = alloc(&G->d_gxyz, 3 * n, &B)) ||
                    (st = alloc(&G->d_out_xyz, 3 * n, &B)))))
      return st;
    G->n_atoms = P->n_atoms;
  }
  return GW_OK;
}

}  // namespace

extern "C" int gw_voxel_grad_buffer(gw_voxel_plan *P, double **g_iq_dev) {
  if (!P || !g_iq_dev) return gw::fail(GW_ERR_ARG, "gw_voxel_grad_buffer: null argument");
  if (P->n_atoms < 0) return gw::fail(GW_ERR_STATE, "gw_voxel_grad_buffer: atoms not set");
  GW_CUDA(cudaSetDevice(P->ctx->device));
  GW_TRY(grad_state_init(P));
  *g_iq_dev = P->grad->d_giq;
  return GW_OK;
}

extern "C" int gw_voxel_backward(gw_voxel_plan *P, const double *g_iq,
                                 int32_t iq_on_device, double *g_f,
                                 double *g_xyz, double *g_sigma, double *g_c) {
  if (P && P->real)
    return gw::fail(GW_ERR_STATE, "gw_voxel_backward: the plan was made with "
                                  "real_grids; the adjoint needs real_grids 0");
  if (!P || !g_iq || !g_f)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: null argument");
  if (P->plain)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: needs the batched mode");
  if (P->p.fill_bkg)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: fill_bkg is not differentiated");
  if (P->n_out > 1)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: separate structures are not differentiated");
  if (P->n_shells > 0)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: multi-q shells are not differentiated");
  if (g_xyz && !P->bil)
    return gw::fail(GW_ERR_ARG, "gw_voxel_backward: coordinate gradients need the bilinear deposit");
  if (P->n_atoms < 0)
    return gw::fail(GW_ERR_STATE, "gw_voxel_backward: atoms not set");
  GW_CUDA(cudaSetDevice(P->ctx->device));
  GW_TRY(grad_state_init(P));
  gw_grad_state *G = P->grad;
  gw_ctx *ctx = P->ctx;
  cudaStream_t st = ctx->stream;
  const size_t Qc3 = (size_t)P->Qc * P->Qc * P->Qc;
  const double *giq = g_iq;
  if (!iq_on_device) {
    GW_CUDA(cudaMemcpyAsync(G->d_giq, g_iq, Qc3 * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    giq = G->d_giq;
  }
  GW_TRY(enqueue_prep(P));
  {
    const float f0c = (float)P->p.f0_coef[8];
    const float f0iz = P->p.f0_z > 0 ? (float)(1.0 / P->p.f0_z) : 1.f;
    const int thr = P->Qc >= 256 ? 256 : ((P->Qc + 31) / 32) * 32;
    gw::KTimer tm(ctx, GW_K_FINALIZE);
    k_fin_adj<<<P->Qc * P->Qc, thr, 0, st>>>(
        giq, P->d_C2, P->d_C1, P->W, P->lo - P->wlo, P->Qc,
        P->p.average ? 1.0f / (float)P->n_struct : 1.0f, P->d_f0,
        P->p.f0_z > 0, f0c, f0iz, G->d_gsum);
    GW_LAUNCHED(ctx);
  }
  const size_t n = (size_t)P->n_atoms;
  GW_CUDA(cudaMemsetAsync(G->d_gacc, 0, n * sizeof(double2), st));
  if (P->bil) GW_CUDA(cudaMemsetAsync(G->d_gxyz, 0, 3 * n * sizeof(double), st));
  GW_CUDA(cudaMemsetAsync(G->d_sc, 0, (size_t)P->n_slices * SC_N * sizeof(double), st));
  GW_CUDA(cudaMemsetAsync(G->d_amy, 0x7f, P->n_slices * sizeof(int), st));
  GW_CUDA(cudaMemsetAsync(G->d_amz, 0x7f, P->n_struct * sizeof(int), st));
  int64_t max_atoms = 0;
  for (auto &s : P->structs) max_atoms = std::max(max_atoms, s.atom_count);
  const int nblk_at = (int)std::min<int64_t>(
      std::max<int64_t>(1, (max_atoms + 255) / 256), 4 * ctx->sm_count);
  if (P->bil) {
    gw::KTimer tm(ctx, GW_K_MISC);
    k_argmin_z<<<dim3(nblk_at, P->n_struct), 256, 0, st>>>(
        P->d_xyz_s, P->d_structs, P->d_zmin, P->d_perm, G->d_amz);
    GW_LAUNCHED(ctx);
  }
  SliceArgs a = slice_args(P);
  CztArgs cy{P->My, P->Ly, P->Nc, P->d_Ay, P->d_Hy, P->d_By, P->d_twy};
  CztArgs cz{P->Mz, P->Lz, P->Nr, P->d_Az, P->d_Hz, P->d_Bz, P->d_twz};
  BinArgs bn{P->d_colofs, P->d_rowofs, P->d_sum, P->d_sumk, 0, P->k0, P->kz0,
             (float)((double)P->g * (double)P->g), 0};
  GradCol gc{G->d_gsum, G->d_Az, G->d_Hz, G->d_Bz, G->d_G1, G->d_sc,
             (float)((double)P->g * (double)P->g)};
  GradRow gr{G->d_Ay, G->d_Hy, G->d_By, P->d_twy, G->d_G1, G->d_dmy, G->d_dmz,
             G->d_gacc, G->d_gxyz, G->d_sc, P->Nc};
  for (int s0 = 0; s0 < P->n_slices; s0 += P->S) {
    const int nb = std::min(P->S, P->n_slices - s0);
    GW_TRY(enqueue_slice_setup(P, a, s0, nb));
    if (a.smooth_on) {
      gw::KTimer tm(ctx, GW_K_PROFILE);
      k_dprofile<<<nb, 256, 0, st>>>(a, s0, G->d_dgw, G->d_dmy, G->d_dmz);
      GW_LAUNCHED(ctx);
    }
    if (P->bil) {
      gw::KTimer tm(ctx, GW_K_MISC);
      k_argmin_y<<<dim3(nblk_at, nb), 256, 0, st>>>(a, s0, P->d_perm, G->d_amy);
      GW_LAUNCHED(ctx);
    }
    GW_TRY(row_dispatch(P, a, cy, s0, nb));
    GW_TRY(col_bwd_dispatch(P, a, cz, bn, gc, s0, nb));
    GW_TRY(row_bwd_dispatch(P, a, gr, s0, nb));
  }
  {
    gw::KTimer tm(ctx, GW_K_MISC);
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 8 * (size_t)ctx->sm_count);
    k_unperm<<<blocks, 256, 0, st>>>((int64_t)n, P->d_perm, G->d_gacc, G->d_gxyz,
                                     G->d_out_f, G->d_out_xyz);
    GW_LAUNCHED(ctx);
  }
  std::vector<double> sc((size_t)P->n_slices * SC_N);
  std::vector<int> amy(P->n_slices), amz(P->n_struct);
  GW_CUDA(cudaMemcpyAsync(g_f, G->d_out_f, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
  if (g_xyz)
    GW_CUDA(cudaMemcpyAsync(g_xyz, G->d_out_xyz, 3 * n * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaMemcpyAsync(sc.data(), G->d_sc, sc.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaMemcpyAsync(amy.data(), G->d_amy, amy.size() * sizeof(int),
                          cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaMemcpyAsync(amz.data(), G->d_amz, amz.size() * sizeof(int),
                          cudaMemcpyDeviceToHost, st));
  GW_CUDA(cudaStreamSynchronize(st));
  GW_TRY(gw::check_device_error(ctx, "voxel backward"));

  // host reductions of the per-slice scalars
  const bool smooth = P->p.smooth != 0.0;
  double gs = 0.0;
  for (int t = 0; t < P->n_struct; ++t) {
    const gw_structure &s = P->structs[t];
    const double cre = s.avg_f_re * s.max_voxels, cim = s.avg_f_im * s.max_voxels;
    double gcre = 0.0, gcim = 0.0, sv = 0.0;
    for (int q = 0; q < P->n_phi; ++q) {
      const int sl = t * P->n_phi + q;
      const double *v = sc.data() + (size_t)sl * SC_N;
      if (smooth) {
        // D = (dep - c) m and the q = 0 term c g^2
        gcre += v[SC_DC_RE] - v[SC_SM_RE];
        gcim += v[SC_DC_IM] - v[SC_SM_IM];
        gs += v[SC_SIG_AT] - (v[SC_SDM_RE] * cre + v[SC_SDM_IM] * cim);
      }
      if (g_xyz) {
        // the shift to the minimum moves every atom with the argmin atom
        const int am = amy[sl];
        if (am >= 0 && am < (int)n) {
          g_xyz[3 * (size_t)am] -= v[SC_SU] * P->phis[q].sin_phi;
          g_xyz[3 * (size_t)am + 1] -= v[SC_SU] * P->phis[q].cos_phi;
        }
        sv += v[SC_SV];
      }
    }
    if (g_xyz) {
      const int am = amz[t];
      if (am >= 0 && am < (int)n) g_xyz[3 * (size_t)am + 2] -= sv;
    }
    if (g_c) { g_c[2 * t] = gcre; g_c[2 * t + 1] = gcim; }
  }
  if (g_sigma) *g_sigma = gs;
  return GW_OK;
}
