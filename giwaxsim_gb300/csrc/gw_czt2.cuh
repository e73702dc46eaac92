// Fused chirp-z kernels of the batched voxel stage: the row transform
// (along y, with the deposit) and the column transform with the binning
// (along z), each a circular convolution of length M = R1 * R2 done with two
// shared-memory exchanges instead of the Stockham plan's five.
//
// Reference: tools/voxelgrids.py:382-392 (fftn, fftshift, |.|^2) and
// :464-506 (process_file2 binning); the band-limited chirp-z evaluation
// X[k0+m] = B[m] * sum_n (D[n] A[n]) h[m-n] is the same as in gw_voxel.cu.
//
// The convolution y = IDFT_M(DFT_M(x) * H) (H = DFT_M(h) / M) is split with
// n = n1 R2 + n2 (n1 < R1, n2 < R2) and k = k1 + R1 k2 (k1 < R1, k2 < R2):
//   pass 1  (thread n2)  Y[k1][n2] = sum_n1 x[n1 R2 + n2] W_R1^{n1 k1}
//           only n1 < KIN are read: the window is shorter than M
//   middle  (thread k1)  V[k2] = sum_n2 Y[k1][n2] W_M^{n2 k1} W_R2^{n2 k2};
//                        V[k2] *= H[k1 + R1 k2];
//                        U[n2] = conj(W_M^{n2 k1}) sum_k2 V[k2] W_R2^{-n2 k2}
//   pass 3  (thread n2)  y[n1 R2 + n2] = sum_k1 U[k1][n2] W_R1^{-n1 k1}
// The forward DFT's second stage, the spectrum product and the inverse DFT's
// first stage run in one thread's registers, so the transform pair costs two
// exchanges through shared memory (after pass 1 and after the middle).
//
// Shared layout of a sequence: Y[k1][n2] at k1 * (R2 + 1) + n2.  Pass 1 and
// pass 3 threads of a warp read or write consecutive n2; middle threads of a
// warp read consecutive k1 rows of odd pitch R2 + 1; both are free of bank
// conflicts (sequence strides below keep it so across sequences).
//
// Block shapes: NB sequences per block and a register cap of MINB resident
// blocks per SM (__launch_bounds__); the plan's block_variant picks one of
// kFusedVariants (an autotuner times them).  gw_czt2_row.cu and
// gw_czt2_col.cu instantiate the row and column kernels.
#pragma once

#include "gw_dft.cuh"
#include "gw_tma.cuh"
#include "gw_voxel_impl.cuh"

namespace gwv {
namespace czt2 {

struct FusedVariant { int nb, minb; };
// 0: 4 sequences, no cap below the shape's need; 1, 2: 4 sequences capped
// for 3 or 4 blocks per SM; 3: 8 sequences per block
constexpr FusedVariant kFusedVariants[] = {{4, 1}, {4, 3}, {4, 4}, {8, 1}};
constexpr int kFusedVariantCount = 4;

// Fused shape of length M: M = R1 * R2 with R1 >= R2 (the middle pass, the
// heaviest, has R1 threads per sequence and uses the whole block).
template <int M> struct Fused;
template <> struct Fused<1024> { static constexpr int R1 = 32, R2 = 32; };
template <> struct Fused<1280> { static constexpr int R1 = 40, R2 = 32; };

template <int M>
struct FusedLayout {
  static constexpr int R1 = Fused<M>::R1, R2 = Fused<M>::R2;
  static constexpr int PITCH = R2 + 1;
  static constexpr int SEQ = R1 * PITCH;  // one sequence's exchange array
};

// ------------------------------------------------------------ middle pass
// One thread, one k1 of one sequence (seq = the sequence's exchange array):
// twiddle, DFT R2, spectrum product, inverse DFT R2, conjugate twiddle, in
// place.  tw2[n2 * R1 + k1] = W_M^{n2 k1}.
template <int M>
__device__ __forceinline__ void fused_middle(float2 *seq, int k1,
                                             const float2 *__restrict__ tw2,
                                             const float2 *__restrict__ H) {
  constexpr int R1 = Fused<M>::R1, R2 = Fused<M>::R2, PITCH = R2 + 1;
  float2 v[R2];
  float2 *p = seq + k1 * PITCH;
  gwd::sfor<R2>([&](auto n2) { v[n2] = p[n2]; });
  gwd::sfor<R2 - 1>([&](auto i) {
    constexpr int n2 = i + 1;
    v[n2] = cmul(v[n2], __ldg(tw2 + n2 * R1 + k1));
  });
  // in place: V[k2] is left in slot out_at<R2, 0>(k2), and the inverse
  // reads that order and leaves U[n2] in slot out_at<R2, 1>(n2)
  gwd::dft_ip<R2, false, R2, 0>(v);
  gwd::sfor<R2>([&](auto k2) {
    constexpr int s = gwd::out_at<R2, 0>(k2);
    v[s] = cmul(v[s], __ldg(H + k1 + R1 * k2));
  });
  gwd::dft_ip<R2, true, R2, 1>(v);
  gwd::sfor<R2>([&](auto n2) {
    constexpr int s = gwd::out_at<R2, 1>(n2);
    float2 u = v[s];
    if constexpr (n2 > 0) {
      const float2 w = __ldg(tw2 + n2 * R1 + k1);
      u = cmul(u, make_float2(w.x, -w.y));
    }
    p[n2] = u;
  });
}

// ------------------------------------------------------------ row kernel
// NB window rows per block: deposit into shared memory (deposit_rows),
// pass 1 reading the deposit with the fill/smoothing value and the chirp A,
// the middle, pass 3 writing F1 = B * y for the band.  HALF: the window (L)
// and the band (N) both fit in M / 2, so pass 1 reads only n1 < R1 / 2 and
// pass 3 produces only n1 < R1 / 2.
template <int M, int NB, int MINB, bool HALF, bool BIL>
__global__ void __launch_bounds__(NB * Fused<M>::R1, MINB)
k_row_fused(SliceArgs a, CztArgs cz, const float2 *__restrict__ tw2, int slice0,
            int n_sl, int n_rows, int nc_out, float2 *F1) {
  constexpr int R1 = Fused<M>::R1, R2 = Fused<M>::R2;
  constexpr int PITCH = FusedLayout<M>::PITCH, SEQ = FusedLayout<M>::SEQ;
  constexpr int NT = NB * R1;
  constexpr int NIN = HALF ? R1 / 2 : R1;
  extern __shared__ float2 smem[];
  __shared__ RowShared<NB> rs;
  const int row0 = blockIdx.x * NB;
  deposit_rows<NB, NT, BIL>(a, cz.L, slice0, n_sl, n_rows, row0, smem, SEQ, rs);

  // pass 1: all inputs into registers, then (the deposit shares the memory)
  // a barrier, then the outputs
  const int t = threadIdx.x;
  const bool p13 = t < NB * R2;
  const int f = t / R2, n2 = t - (t / R2) * R2;
  float2 x[R1];
  if (p13) {
    const int row = row0 + f;
    const bool live = row < n_rows;
    const RowConst &rk = rs.k[f];
    const float2 *dep = smem + f * SEQ;
    gwd::sfor<NIN>([&](auto n1) {
      const int n = n1 * R2 + n2;
      float2 v = make_float2(0.f, 0.f);
      if (live && n < cz.L) v = cmul(d_value_row(a, rk, n, dep[n]), __ldg(cz.A + n));
      x[n1] = v;
    });
  }
  __syncthreads();
  if (p13) {
    gwd::dft_ip<R1, false, NIN, 0>(x);
    float2 *q = smem + f * SEQ + n2;
    gwd::sfor<R1>([&](auto k1) { q[k1 * PITCH] = x[gwd::out_at<R1, 0>(k1)]; });
  }
  __syncthreads();
  // middle: every thread one k1 of one row
  {
    const int fm = t / R1, k1 = t - (t / R1) * R1;
    fused_middle<M>(smem + fm * SEQ, k1, tw2, cz.H);
  }
  __syncthreads();
  // pass 3
  if (p13) {
    const int row = row0 + f;
    const float2 *q = smem + f * SEQ + n2;
    gwd::sfor<R1>([&](auto k1) { x[k1] = q[k1 * PITCH]; });
    gwd::dft_ip<R1, true, R1, 0>(x);
    if (row < n_rows) {
      float2 *out = F1 + (size_t)row * nc_out;
      gwd::sfor<NIN>([&](auto n1) {
        const int m = n1 * R2 + n2;
        if (m < nc_out) out[m] = cmul(x[gwd::out_at<R1, 0>(n1)], __ldg(cz.B + m));
      });
    }
  }
}

// ------------------------------------------------------------ column kernel
// NB columns of one slice per block, transformed along z; pass 3 squares
// B * y (plus the background's DC term) and bins it into the float64 sum
// grid (or the Kahan float32 pairs).  With TMA the slice's F1 rows of the
// block's columns arrive as boxes of a 2-D tensor map into the (aliased)
// exchange memory; pass 1 then reads the tile (column f fastest across
// threads, so the tile's rows are read whole).
template <int M, int NB>
struct ColLayout {
  static constexpr int R1 = Fused<M>::R1, R2 = Fused<M>::R2;
  static constexpr int PITCH = R2 + 1;
  // sequence stride: pass 1 writes with the column fastest across lanes;
  // a stride of 16 / NB mod 16 (in 8-byte words) spreads the NB columns
  // over distinct banks
  static constexpr int SEQ = R1 * PITCH + (16 / NB - (R1 * PITCH) % 16 + 16) % 16;
  static constexpr int BR = tma_box_rows(M);
  // the tile: up to M rows of NB values, 128-byte aligned inside the area
  static constexpr int AREA = (NB * SEQ > NB * M ? NB * SEQ : NB * M) + 16;
};

template <int M, int NB, int MINB, bool HALF, bool TMA>
__global__ void __launch_bounds__(NB * Fused<M>::R1, MINB)
k_col_fused(SliceArgs a, CztArgs cz, BinArgs bn, const float2 *__restrict__ tw2,
            int slice0, int nc, const float2 *F1,
            const __grid_constant__ CUtensorMap f1map) {
  using Lay = ColLayout<M, NB>;
  constexpr int R1 = Lay::R1, R2 = Lay::R2, PITCH = Lay::PITCH, SEQ = Lay::SEQ;
  constexpr int NIN = HALF ? R1 / 2 : R1;
  static_assert(R2 <= R1, "pass threads");
  extern __shared__ __align__(128) float2 smem[];
  __shared__ uint64_t tile_bar;
  const int slot = blockIdx.y, sl = slice0 + slot;
  const int p = sl % a.n_phi;
  const int m0 = blockIdx.x * NB;
  const int *cofs = bn.colofs + (size_t)p * nc;
  // column groups none of whose pixels lands in the binned window
  bool any = false;
  for (int f = 0; f < NB; ++f)
    if (m0 + f < nc && cofs[m0 + f] >= 0) any = true;
  if (!any) return;
  int first, rows;
  slice_rows(a, slice0, sl, first, rows);
  float2 *tile = smem + ((128u - (smem_u32(smem) & 127u)) & 127u) / sizeof(float2);
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      const int nload = (rows + Lay::BR - 1) / Lay::BR;
      mbar_init(&tile_bar, 1);
      mbar_arrive_expect_tx(&tile_bar, (unsigned)(nload * Lay::BR * NB * sizeof(float2)));
      for (int i = 0; i < nload; ++i)
        tma_load_2d(tile + (size_t)i * Lay::BR * NB, &f1map, m0, first + i * Lay::BR, &tile_bar);
    }
    __syncthreads();
    // one decision for the whole block: every thread goes on, or none
    if (!__syncthreads_and(mbar_wait_bounded(&tile_bar, 0, bn.wait_polls))) {
      if (threadIdx.x == 0) dev_error(a.err, GW_DEVERR_TIMEOUT);
      // the loads still in flight must land before the block's shared
      // memory is released; nothing is binned from this block
      mbar_wait_bounded(&tile_bar, 0, kTileWaitPolls);
      return;
    }
  }
  const int t = threadIdx.x;
  const bool p13 = t < NB * R2;
  float2 x[R1];
  {
    // pass 1 loads: column f fastest
    const int f = t % NB, n2 = t / NB;
    if (p13) {
      const bool live = m0 + f < nc;
      gwd::sfor<NIN>([&](auto n1) {
        const int n = n1 * R2 + n2;
        float2 v = make_float2(0.f, 0.f);
        if (live && n < rows) {
          const float2 d = TMA ? tile[n * NB + f] : F1[(size_t)(first + n) * nc + m0 + f];
          v = cmul(d, __ldg(cz.A + n));
        }
        x[n1] = v;
      });
    }
    if (TMA) __syncthreads();  // the tile shares the exchange memory
    if (p13) {
      gwd::dft_ip<R1, false, NIN, 0>(x);
      float2 *q = smem + f * SEQ + n2;
      gwd::sfor<R1>([&](auto k1) { q[k1 * PITCH] = x[gwd::out_at<R1, 0>(k1)]; });
    }
  }
  __syncthreads();
  {
    const int fm = t / R1, k1 = t - (t / R1) * R1;
    fused_middle<M>(smem + fm * SEQ, k1, tw2, cz.H);
  }
  __syncthreads();
  if (p13) {
    // pass 3: row n2 fastest, so that the atomics of a warp go to
    // consecutive qz voxels
    const int f = t / R2, n2 = t - (t / R2) * R2;
    const int m = m0 + f;
    const float2 *q = smem + f * SEQ + n2;
    gwd::sfor<R1>([&](auto k1) { x[k1] = q[k1 * PITCH]; });
    gwd::dft_ip<R1, true, R1, 0>(x);
    const int co = m < nc ? cofs[m] : -1;
    if (co >= 0) {
      const float2 cbg = slice_const(a, sl).cbg;
      const int64_t soff = bn.sstride * (int64_t)(sl / a.n_phi);
      gwd::sfor<NIN>([&](auto n1) {
        const int mr = n1 * R2 + n2;
        if (mr < cz.N) {
          const int ro = bn.rowofs[mr];
          if (ro >= 0 && (!bn.shell || shell_member(bn.shell[co + ro], bn.shell_k))) {
            float2 X = cmul(x[gwd::out_at<R1, 0>(n1)], __ldg(cz.B + mr));
            if (bn.k0 + m == 0 && bn.kz0 + mr == 0) {
              X.x += cbg.x * bn.dc_scale;
              X.y += cbg.y * bn.dc_scale;
            }
            const float I = X.x * X.x + X.y * X.y;
            if (bn.kahan) kahan_add(bn.sumk + soff + co + ro, I);
            else atomicAdd(bn.sum + soff + co + ro, f2d_exact(I));
          }
        }
      });
    }
  }
}

template <int M>
bool half_fits(int L, int N) { return L <= M / 2 && N <= M / 2; }

}  // namespace czt2
}  // namespace gwv
