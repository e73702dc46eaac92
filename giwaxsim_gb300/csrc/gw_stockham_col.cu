// Stockham chirp-z column kernels of the voxel stage (any supported
// length): the column transform along z with |F|^2 and the binning, its
// launch, and the F1 tensor map the column kernels' TMA tile loads use.
//
// Reference: tools/voxelgrids.py:382-392 (fftn, fftshift, |.|^2), :464-506
// (process_file2 binning).
#include <cstring>

#include "gw_tma.cuh"
#include "gw_voxel_impl.cuh"

using namespace gwv;

namespace {

// F1 columns j0 + f (nf per row) of the slice's rows.
struct ColLoad {
  const float2 *src, *A;
  int L, nf, j0;
  __device__ float2 operator()(int f, int n) const {
    if (n >= L || j0 + f >= nf) return make_float2(0.f, 0.f);
    return cmul(src[(size_t)n * nf + j0 + f], __ldg(A + n));
  }
};

// The same columns from a shared-memory tile (row n, column f at
// tile[n * NB + f]) that a TMA load brought in.
template <int NB>
struct ColTileLoad {
  const float2 *tile, *A;
  int L, nf, j0;
  __device__ float2 operator()(int f, int n) const {
    if (n >= L || j0 + f >= nf) return make_float2(0.f, 0.f);
    return cmul(tile[n * NB + f], __ldg(A + n));
  }
};

// The box's inner extent (NB complex values) must be a multiple of 16 bytes.
template <int M>
__host__ __device__ constexpr bool col_tma_ok() {
  return (FftShape<M>::NB * (int)sizeof(float2)) % 16 == 0;
}

// |B y|^2 (plus the background's DC term at q = 0) of output row mr of F1
// column j0 + f (table column m = moff + j0 + f) binned into the float64
// sums; with mirrored binning (real grids) also at (2 m_zero - m,
// 2 r_zero - mr) for m > m_zero.
struct ColBin {
  BinArgs bn;       // by value: no reads through a pointer to the parameters
  const int *cofs;
  const float2 *B;
  float2 cbg;
  int nr, nc, j0, moff;
  int64_t soff;  // sum-grid offset of the slice's structure (separate mode)
  float *gcol;   // gather binning: the slice's pixels of F1 column j0, then
                 // j0 + 1, .. (Nr each); null: atomic adds
  __device__ void add(int co, int ro, float I) const {
    if (co < 0 || ro < 0) return;
    if (bn.shell && !shell_member(bn.shell[co + ro], bn.shell_k)) return;
    if (bn.kahan) kahan_add(bn.sumk + soff + co + ro, I);
    else atomicAdd(bn.sum + soff + co + ro, f2d_exact(I));
  }
  __device__ void operator()(int f, int mr, float2 v) const {
    const int m = moff + j0 + f;
    if (mr >= nr || m >= nc) return;
    const int co = cofs[m], ro = bn.rowofs[mr];
    // the band's extra even-width column (m = 2 m_zero + 1) has no mirror
    const bool mir = bn.mirror && m > bn.m_zero && m <= 2 * bn.m_zero;
    const int cm = mir ? cofs[2 * bn.m_zero - m] : -1;
    const int rm = mir ? bn.rowofs[2 * bn.r_zero - mr] : -1;
    if ((co < 0 || ro < 0) && (cm < 0 || rm < 0)) return;
    float2 X = cmul(v, __ldg(B + mr));
    if (bn.k0 + m == 0 && bn.kz0 + mr == 0) {
      X.x += cbg.x * bn.dc_scale;
      X.y += cbg.y * bn.dc_scale;
    }
    const float I = X.x * X.x + X.y * X.y;
    if (gcol) {  // every pixel a voxel line will gather (its own or mirrored)
      gcol[(size_t)f * nr + mr] = I;
      return;
    }
    add(co, ro, I);
    if (mir) add(cm, rm, I);
  }
};

// TMA: the slice's F1 rows of the block's NB columns come in as boxes of a
// 2-D tensor map of F1 (one thread issues them, an mbarrier counts their
// bytes) into the FFT buffer, which the first pass reads completely before
// it writes; otherwise each thread loads its elements.
template <int M, bool TMA, bool HALF>
__global__ void __launch_bounds__(FftShape<M>::NT, FftShape<M>::MINB)
k_col_czt_bin(SliceArgs a, CztArgs cz, BinArgs bn, int slice0, int nc, int nf,
              const float2 *F1, const __grid_constant__ CUtensorMap f1map) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  constexpr int TWL = FftPlan<M>::tw_len();
  extern __shared__ __align__(128) float2 smem[];
  __shared__ uint64_t tile_bar;
  float2 *tw = smem;
  float2 *buf = smem + TWL;
  const int slot = blockIdx.y, sl = slice0 + slot;
  const int p = sl % a.n_phi;
  // F1 columns j0 .. j0 + NB - 1 (table columns moff + j)
  const int j0 = blockIdx.x * NB, moff = bn.mirror ? bn.m_zero : 0;
  const int *cofs = bn.colofs + (size_t)p * nc;
  // skip column groups none of whose pixels (nor their mirrors) lands in
  // the binned window
  bool any = false;
  for (int f = 0; f < NB; ++f) {
    const int m = moff + j0 + f;
    if (j0 + f < nf && m < nc &&
        (cofs[m] >= 0 || (bn.mirror && m > bn.m_zero && m <= 2 * bn.m_zero &&
                          cofs[2 * bn.m_zero - m] >= 0)))
      any = true;
  }
  if (!any) return;
  int first, rows;
  slice_rows(a, slice0, sl, first, rows);
  // 128-byte aligned tile inside the FFT buffer: the boxes cover at most M
  // rows of NB values, the buffer holds NB (M + M/16 + 4), and the
  // alignment skips at most 15 values
  constexpr int BR = tma_box_rows(M);
  static_assert(M % BR == 0 && NB * (FftPlan<M>::LDM - M) >= 16, "tile fits");
  float2 *tile = buf + ((128u - (smem_u32(buf) & 127u)) & 127u) / sizeof(float2);
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      const int nload = (rows + BR - 1) / BR;
      mbar_init(&tile_bar, 1);
      mbar_arrive_expect_tx(&tile_bar, (unsigned)(nload * BR * NB * sizeof(float2)));
      for (int i = 0; i < nload; ++i)
        tma_load_2d(tile + (size_t)i * BR * NB, &f1map, j0, first + i * BR, &tile_bar);
    }
  }
  for (int t = threadIdx.x; t < TWL; t += NT) tw[t] = cz.tw[t];
  __syncthreads();
  if constexpr (TMA) {
    // one decision for the whole block: every thread goes on, or none
    if (!__syncthreads_and(mbar_wait_bounded(&tile_bar, 0, bn.wait_polls))) {
      if (threadIdx.x == 0) dev_error(a.err, GW_DEVERR_TIMEOUT);
      // the loads still in flight must land before the block's shared
      // memory is released; nothing is binned from this block
      mbar_wait_bounded(&tile_bar, 0, kTileWaitPolls);
      return;
    }
    ColTileLoad<NB> ld{tile, cz.A, rows, nf, j0};
    fft_run<M, NB, NT, false, 1, false, 0, true, HALF, false>(buf, tw, nullptr, ld,
                                                             NoStore());
  } else {
    ColLoad ld{F1 + (size_t)first * nf, cz.A, rows, nf, j0};
    fft_run<M, NB, NT, false, 1, false, 0, true, HALF, false>(buf, tw, nullptr, ld,
                                                             NoStore());
  }
  ColBin st{bn, cofs, cz.B, slice_const(a, sl).cbg, cz.N, nc, j0, moff,
            bn.sstride * (int64_t)(sl / a.n_phi),
            bn.G ? bn.G + ((size_t)sl * nf + j0) * cz.N : nullptr};
  fft_run<M, NB, NT, true, 0, true, 1, false, false, HALF>(buf, tw, cz.H, NoLoad(), st);
}

}  // namespace

namespace gwv {

template <int M, bool HALF>
int launch_col_t(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 const BinArgs &bn, int slice0, int n_sl) {
  constexpr int NB = FftShape<M>::NB, NT = FftShape<M>::NT;
  const size_t smem = (size_t)(NB * FftPlan<M>::LDM + FftPlan<M>::tw_len()) * sizeof(float2);
  static gw::SmemRecord attr, attr_tma;
  GW_TRY(gw::smem_limit(attr, k_col_czt_bin<M, false, HALF>, smem));
  if constexpr (col_tma_ok<M>())
    GW_TRY(gw::smem_limit(attr_tma, k_col_czt_bin<M, true, HALF>, smem));
  dim3 grid((P->Nf + NB - 1) / NB, n_sl);
  gw::KTimer tm(P->ctx, GW_K_COLBIN);
  if constexpr (col_tma_ok<M>()) {
    if (P->f1_tma) {
      k_col_czt_bin<M, true, HALF><<<grid, NT, smem, P->ctx->stream>>>(
          a, cz, bn, slice0, P->Nc, P->Nf, P->d_F1, P->f1map);
      GW_LAUNCHED(P->ctx);
      return GW_OK;
    }
  }
  k_col_czt_bin<M, false, HALF><<<grid, NT, smem, P->ctx->stream>>>(
      a, cz, bn, slice0, P->Nc, P->Nf, P->d_F1, P->f1map);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

template <int M>
int launch_col(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
               const BinArgs &bn, int slice0, int n_sl) {
  if constexpr (M <= 2048) {
    if (pruned<M>(cz)) return launch_col_t<M, true>(P, a, cz, bn, slice0, n_sl);
  }
  return launch_col_t<M, false>(P, a, cz, bn, slice0, n_sl);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                   void *, const cuuint64_t *, const cuuint64_t *,
                                   const cuuint32_t *, const cuuint32_t *,
                                   CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// Tensor map of F1 (S*Lz rows of Nc complex values) with NB x BR boxes;
// leaves f1_tma false where the rules of tiled loads are not met (odd
// band: row pitch not a multiple of 16 bytes; NB * 8 bytes not a multiple
// of 16) or the encoder is unavailable.  Rows and columns past the map
// read as zeros.
template <int M>
int col_map_create(gw_voxel_plan *P) {
  P->f1_tma = false;
  // the box is as wide as the column kernel's block of columns: a box of
  // another width would deliver other than the bytes the kernel waits for
  const int NB = P->fused_z ? fused_col_block(P) : FftShape<M>::NB;
  P->f1_box_cols = NB;
  if ((NB * (int)sizeof(float2)) % 16 == 0) {
    constexpr int BR = tma_box_rows(M);
    const size_t pitch = (size_t)P->Nf * sizeof(float2);
    EncodeTiledFn enc = encode_tiled();
    if (P->plain || !enc || pitch % 16 != 0 ||
        reinterpret_cast<uintptr_t>(P->d_F1) % 16 != 0)
      return GW_OK;
    const cuuint64_t dims[2] = {(cuuint64_t)P->Nf, (cuuint64_t)P->S * P->Lz};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch};
    const cuuint32_t box[2] = {(cuuint32_t)NB, (cuuint32_t)BR};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&P->f1map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, P->d_F1,
                           dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    P->f1_tma = r == CUDA_SUCCESS;
  }
  return GW_OK;
}

int col_map_dispatch(gw_voxel_plan *P) { GW_DISPATCH_M(P->Mz, col_map_create, P) }

int col_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 const BinArgs &bn, int s0, int n) {
  if (P->fused_z) return fused_col_dispatch(P, a, cz, bn, s0, n);
  GW_DISPATCH_M(P->Mz, launch_col, P, a, cz, bn, s0, n)
}

}  // namespace gwv
