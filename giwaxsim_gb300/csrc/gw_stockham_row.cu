// Stockham chirp-z row kernels of the voxel stage (any supported length):
// the row transform along y with the deposit, and its launch.  The fused
// kernels (gw_czt2.cuh) replace it for the lengths with a fused shape when
// the plan asks for those.
//
// Reference: tools/voxelgrids.py:319-341 (deposit), :382-392 (fftn).
#include <cstring>

#include "gw_tma.cuh"
#include "gw_voxel_impl.cuh"

using namespace gwv;

namespace {

// --------------------------------------------------------------- CZT stages
// Row stage: NB rows (slice, z) per block, transformed along y; Nc outputs
// kept.  The block first deposits the atoms of its rows (contiguous in the
// z-sorted arrays) into shared-memory row buffers with shared atomics
// (voxelgrids.py:328-341: shift, floor division, valid mask, np.add.at).
// The forward FFT's first pass reads those rows with the fill/smoothing
// transform and the chirp A; the inverse FFT's first pass multiplies by the
// filter spectrum H, and its last pass writes F1 = B * result to global
// memory.  The row buffers share storage with the FFT buffer: the first pass
// reads all its inputs before it writes.
template <int M>
// Functors hold what they read by value (registers), never a pointer to
// the kernel's parameters.
struct RowLoad {
  RowValueArgs va;
  const float2 *A;        // forward chirp
  int L;                  // window length
  const float2 *rows;     // row f at rows + f * LDM
  const RowConst *rc;     // per block row (shared memory)
  int row0, n_rows;
  __device__ float2 operator()(int f, int n) const {
    const int row = row0 + f;
    if (row >= n_rows || n >= L) return make_float2(0.f, 0.f);
    const float2 dep = rows[f * FftPlan<M>::LDM + n];
    return cmul(d_value_row(va, rc[f], n, dep), __ldg(A + n));
  }
};

struct RowStore {
  const float2 *B;
  float2 *F1;
  int row0, n_rows, nc;
  __device__ void operator()(int f, int m, float2 v) const {
    const int row = row0 + f;
    if (row < n_rows && m < nc) F1[(size_t)row * nc + m] = cmul(v, __ldg(B + m));
  }
};

// HALF: the window (L) and the band (N) both fit in M / 2, so the forward
// transform's first pass and the inverse transform's last pass are pruned.
template <int M, bool BIL, bool HALF>
__global__ void __launch_bounds__(FftShape<M>::NT,
                                  HALF ? minb_pruned_rows<M>() : FftShape<M>::MINB)
k_row_czt(SliceArgs a, CztArgs cz, int slice0, int n_sl, int n_rows,
          int nc_out, float2 *F1) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  constexpr int TWL = FftPlan<M>::tw_len();
  constexpr int LDM = FftPlan<M>::LDM;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *buf = smem + TWL;
  __shared__ RowShared<NB> rs;
  for (int t = threadIdx.x; t < TWL; t += NT) tw[t] = cz.tw[t];
  const int row0 = blockIdx.x * NB;
  deposit_rows<NB, NT, BIL>(a, cz.L, slice0, n_sl, n_rows, row0, buf, LDM, rs);
  RowLoad<M> ld{row_value_args(a), cz.A, cz.L, buf, rs.k, row0, n_rows};
  fft_run<M, NB, NT, false, 1, false, 0, false, HALF, false>(buf, tw, nullptr, ld,
                                                            NoStore());
  RowStore stv{cz.B, F1, row0, n_rows, nc_out};
  fft_run<M, NB, NT, true, 0, true, 1, false, false, HALF>(buf, tw, cz.H, NoLoad(), stv);
}

// Real grids: when every atom's f is a real multiple of one complex value,
// a slice's grid is u R with R real and u the unit phase of the
// structure's average voxel f (fill and smoothing values are multiples of
// it too).  The DFT of a real row is Hermitian, Y[-k] = conj(Y[k]), so two
// window rows A and B share one transform: x = R_A + i R_B gives
// Z = Y_A + i Y_B, and Y_A[k] = (Z[k] + conj(Z[-k])) / 2,
// Y_B[k] = (Z[k] - conj(Z[-k])) / (2 i).  The block deposits its 2 NB rows
// as float arrays into the halves of its NB transform buffers (row r at
// float offset r LDM: row 2f in the first half of buffer f, row 2f+1 in the
// second; the window fits: L <= LDM), transforms the NB packed
// rows, leaves the inverse transform in shared memory, and writes F1 for
// the columns ky >= 0 only (the column stage needs no others):
// F1[row][j] = u_row Y_row[m_zero + j], j < nf.
template <int M>
struct RowLoadPair {
  RowValueArgs va;
  const float2 *A;        // forward chirp
  int L;                  // window length
  const float *rows;      // block row r: floats rows[r * LDM + n]
  const RowConst *rc;     // per block row (shared memory)
  int row0, n_rows;       // row0: the block's first window row
  __device__ float2 operator()(int f, int n) const {
    if (n >= L) return make_float2(0.f, 0.f);
    constexpr int LD = FftPlan<M>::LDM;
    float re = 0.f, im = 0.f;
    const int ra = 2 * f, rb = 2 * f + 1;
    // the deposit holds the real row's atom sum r (deposit_rows<.., REAL>):
    // the grid value there is d_value_row of r u, projected back on u
    if (row0 + ra < n_rows) re = d_value_row_real(va, rc[ra], n, rows[ra * LD + n]);
    if (row0 + rb < n_rows) im = d_value_row_real(va, rc[rb], n, rows[rb * LD + n]);
    return cmul(make_float2(re, im), __ldg(A + n));
  }
};

template <int M, bool HALF>
__global__ void __launch_bounds__(FftShape<M>::NT,
                                  HALF ? minb_pruned_rows<M>() : FftShape<M>::MINB)
k_row_czt_real(SliceArgs a, CztArgs cz, int slice0, int n_sl, int n_rows,
               int m_zero, int nf, float2 *F1) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  constexpr int TWL = FftPlan<M>::tw_len();
  constexpr int LDM = FftPlan<M>::LDM;
  static_assert(LDM % 2 == 0, "two rows per transform buffer");
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *buf = smem + TWL;
  __shared__ RowShared<2 * NB> rs;
  for (int t = threadIdx.x; t < TWL; t += NT) tw[t] = cz.tw[t];
  const int row0 = blockIdx.x * 2 * NB;
  deposit_rows<2 * NB, NT, false, true>(a, cz.L, slice0, n_sl, n_rows, row0, buf,
                                        LDM, rs);
  RowLoadPair<M> ld{row_value_args(a), cz.A, cz.L, reinterpret_cast<const float *>(buf),
                    rs.k, row0, n_rows};
  fft_run<M, NB, NT, false, 1, false, 0, false, HALF, false>(buf, tw, nullptr, ld,
                                                            NoStore());
  // the inverse transform stays in shared memory (natural order; with HALF
  // only the outputs below M/2, which hold the band); the block is
  // synchronised afterwards
  fft_run<M, NB, NT, true, 0, true, 0, false, false, HALF>(buf, tw, cz.H, NoLoad(),
                                                          NoStore());
  for (int f = 0; f < NB; ++f) {
    for (int j = threadIdx.x; j < nf; j += NT) {
      const int m = m_zero + j, mm = m_zero - j;  // k and -k
      float2 X = make_float2(0.f, 0.f), Xm = make_float2(0.f, 0.f);
      if (m < cz.N) X = cmul(buf[f * LDM + fft_pad(m)], __ldg(cz.B + m));
      if (mm >= 0) Xm = cmul(buf[f * LDM + fft_pad(mm)], __ldg(cz.B + mm));
      // Y_A = (X + conj(Xm)) / 2, Y_B = -i (X - conj(Xm)) / 2
      const float2 ya = make_float2(0.5f * (X.x + Xm.x), 0.5f * (X.y - Xm.y));
      const float2 yb = make_float2(0.5f * (X.y + Xm.y), -0.5f * (X.x - Xm.x));
      const int ra = row0 + 2 * f, rb = ra + 1;
      if (ra < n_rows) F1[(size_t)ra * nf + j] = cmul(rs.k[2 * f].u, ya);
      if (rb < n_rows) F1[(size_t)rb * nf + j] = cmul(rs.k[2 * f + 1].u, yb);
    }
  }
}

}  // namespace

namespace gwv {

template <int M, bool BIL, bool HALF>
int launch_row_t(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 int slice0, int n_sl) {
  const int n_rows = batch_rows(P, slice0, n_sl);
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = (size_t)(NB * FftPlan<M>::LDM + FftPlan<M>::tw_len()) * sizeof(float2);
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_row_czt<M, BIL, HALF>, smem));
  const int blocks = (n_rows + NB - 1) / NB;
  gw::KTimer tm(P->ctx, GW_K_ROW);
  k_row_czt<M, BIL, HALF><<<blocks, NT, smem, P->ctx->stream>>>(a, cz, slice0, n_sl,
                                                                n_rows, P->Nf, P->d_F1);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M, bool HALF>
int launch_row_real(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                    int slice0, int n_sl) {
  const int n_rows = batch_rows(P, slice0, n_sl);
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = (size_t)(NB * FftPlan<M>::LDM + FftPlan<M>::tw_len()) * sizeof(float2);
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_row_czt_real<M, HALF>, smem));
  const int blocks = (n_rows + 2 * NB - 1) / (2 * NB);
  gw::KTimer tm(P->ctx, GW_K_ROW);
  k_row_czt_real<M, HALF><<<blocks, NT, smem, P->ctx->stream>>>(
      a, cz, slice0, n_sl, n_rows, P->m_zero, P->Nf, P->d_F1);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M>
int launch_row(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
               int slice0, int n_sl) {
  if constexpr (M <= 2048 && FftShape<M>::NB <= 16) {
    if (P->real)
      return pruned<M>(cz) ? launch_row_real<M, true>(P, a, cz, slice0, n_sl)
                           : launch_row_real<M, false>(P, a, cz, slice0, n_sl);
    if (pruned<M>(cz))
      return a.bil ? launch_row_t<M, true, true>(P, a, cz, slice0, n_sl)
                   : launch_row_t<M, false, true>(P, a, cz, slice0, n_sl);
  }
  if (P->real) return gw::fail(GW_ERR_ARG, "real-grid rows need a length up to 2048");
  return a.bil ? launch_row_t<M, true, false>(P, a, cz, slice0, n_sl)
               : launch_row_t<M, false, false>(P, a, cz, slice0, n_sl);
}

int row_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 int s0, int n) {
  if (P->fused_y) return fused_row_dispatch(P, a, cz, s0, n);
  GW_DISPATCH_M(P->My, launch_row, P, a, cz, s0, n)
}
}  // namespace gwv
