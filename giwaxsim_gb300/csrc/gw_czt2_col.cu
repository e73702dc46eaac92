// Launches of the fused chirp-z column kernel with the binning
// (gw_czt2.cuh).
#include "gw_czt2.cuh"

using namespace gwv;
using namespace gwv::czt2;

namespace {

template <int M, int NB, int MINB, bool HALF, bool TMA>
int launch_col_fused(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                     const BinArgs &bn, int s0, int n_sl) {
  constexpr int NT = NB * Fused<M>::R1;
  const size_t smem = ((size_t)ColLayout<M, NB>::AREA) * sizeof(float2);
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_col_fused<M, NB, MINB, HALF, TMA>, smem));
  if (TMA && P->f1_box_cols != NB)
    return gw::fail(GW_ERR_STATE, "fused column kernel: tensor-map box of " +
                                      std::to_string(P->f1_box_cols) +
                                      " columns, blocks of " + std::to_string(NB));
  dim3 grid((P->Nc + NB - 1) / NB, n_sl);
  gw::KTimer tm(P->ctx, GW_K_COLBIN);
  k_col_fused<M, NB, MINB, HALF, TMA><<<grid, NT, smem, P->ctx->stream>>>(
      a, cz, bn, P->d_ftz, s0, P->Nc, P->d_F1, P->f1map);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

// Block-shape variants of the TMA, half-length form (the batched
// workloads' case); every other form runs variant 0.
template <int M, bool HALF, bool TMA>
int col_variant(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                const BinArgs &bn, int s0, int n) {
  constexpr auto V = kFusedVariants;
  if constexpr (HALF && TMA) {
    switch (P->p.block_variant) {
      case 1: return launch_col_fused<M, V[1].nb, V[1].minb, HALF, TMA>(P, a, cz, bn, s0, n);
      case 2: return launch_col_fused<M, V[2].nb, V[2].minb, HALF, TMA>(P, a, cz, bn, s0, n);
      case 3: return launch_col_fused<M, V[3].nb, V[3].minb, HALF, TMA>(P, a, cz, bn, s0, n);
      default: break;
    }
  }
  return launch_col_fused<M, V[0].nb, V[0].minb, HALF, TMA>(P, a, cz, bn, s0, n);
}

template <int M>
int col_fused(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
              const BinArgs &bn, int s0, int n) {
  const bool h = half_fits<M>(cz.L, cz.N);
  if (P->f1_tma) return h ? col_variant<M, true, true>(P, a, cz, bn, s0, n)
                          : col_variant<M, false, true>(P, a, cz, bn, s0, n);
  return h ? col_variant<M, true, false>(P, a, cz, bn, s0, n)
           : col_variant<M, false, false>(P, a, cz, bn, s0, n);
}

}  // namespace

namespace gwv {

int fused_col_block(const gw_voxel_plan *P) {
  // the plan's block shape where it applies (the half-length TMA form,
  // col_variant), else the default
  const bool half = (P->Mz == 1024 && half_fits<1024>(P->Lz, P->Nr)) ||
                    (P->Mz == 1280 && half_fits<1280>(P->Lz, P->Nr));
  return half ? kFusedVariants[P->p.block_variant].nb : kFusedVariants[0].nb;
}

int fused_col_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                       const BinArgs &bn, int s0, int n) {
  switch (P->Mz) {
    case 1024: return col_fused<1024>(P, a, cz, bn, s0, n);
    case 1280: return col_fused<1280>(P, a, cz, bn, s0, n);
  }
  return gw::fail(GW_ERR_ARG, "no fused column transform of this length");
}

}  // namespace gwv
