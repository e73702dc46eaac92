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
struct RowLoad {
  const SliceArgs *a;
  const CztArgs *cz;
  const float2 *rows;     // row f at rows + f * LDM
  const RowConst *rc;     // per block row (shared memory)
  int row0, n_rows;
  __device__ float2 operator()(int f, int n) const {
    const int row = row0 + f;
    if (row >= n_rows || n >= cz->L) return make_float2(0.f, 0.f);
    const float2 dep = rows[f * FftPlan<M>::LDM + n];
    return cmul(d_value_row(*a, rc[f], n, dep), __ldg(cz->A + n));
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
__global__ void __launch_bounds__(FftShape<M>::NT, FftShape<M>::MINB)
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
  RowLoad<M> ld{&a, &cz, buf, rs.k, row0, n_rows};
  fft_run<M, NB, NT, false, 1, false, 0, false, HALF, false>(buf, tw, nullptr, ld,
                                                            NoStore());
  RowStore stv{cz.B, F1, row0, n_rows, nc_out};
  fft_run<M, NB, NT, true, 0, true, 1, false, false, HALF>(buf, tw, cz.H, NoLoad(), stv);
}

// Column stage: NB columns of one slice, transformed along z.  The forward
// FFT's first pass reads F1 columns (sequence index fastest across threads,
// so a warp reads whole 32-byte sectors), and the inverse FFT's last pass
// squares B * result and bins it into the float64 sum grid.
}  // namespace

namespace gwv {

template <int M, bool BIL, bool HALF>
int launch_row_t(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 int slice0, int n_sl) {
  const int n_rows = batch_rows(P, slice0, n_sl);
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = (size_t)(NB * FftPlan<M>::LDM + FftPlan<M>::tw_len()) * sizeof(float2);
  static bool attr = false;
  if (!attr) {
    GW_CUDA(cudaFuncSetAttribute(k_row_czt<M, BIL, HALF>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    attr = true;
  }
  const int blocks = (n_rows + NB - 1) / NB;
  gw::KTimer tm(P->ctx, GW_K_ROW);
  k_row_czt<M, BIL, HALF><<<blocks, NT, smem, P->ctx->stream>>>(a, cz, slice0, n_sl,
                                                                n_rows, P->Nc, P->d_F1);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M>
int launch_row(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
               int slice0, int n_sl) {
  if constexpr (M <= 2048) {
    if (pruned<M>(cz))
      return a.bil ? launch_row_t<M, true, true>(P, a, cz, slice0, n_sl)
                   : launch_row_t<M, false, true>(P, a, cz, slice0, n_sl);
  }
  return a.bil ? launch_row_t<M, true, false>(P, a, cz, slice0, n_sl)
               : launch_row_t<M, false, false>(P, a, cz, slice0, n_sl);
}

int row_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 int s0, int n) {
  if (P->fused_y) return fused_row_dispatch(P, a, cz, s0, n);
  GW_DISPATCH_M(P->My, launch_row, P, a, cz, s0, n)
}
}  // namespace gwv
