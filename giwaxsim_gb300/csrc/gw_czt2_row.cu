// Launches of the fused chirp-z row kernel (gw_czt2.cuh) and the fused
// transforms' host tables.
#include <cmath>

#include "gw_czt2.cuh"

using namespace gwv;
using namespace gwv::czt2;

namespace {

template <int M, int NB, int MINB, bool HALF, bool BIL>
int launch_row_fused(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                     int s0, int n_sl) {
  constexpr int NT = NB * Fused<M>::R1;
  const size_t smem = (size_t)NB * FusedLayout<M>::SEQ * sizeof(float2);
  static gw::SmemRecord attr;
  GW_TRY(gw::smem_limit(attr, k_row_fused<M, NB, MINB, HALF, BIL>, smem));
  const int n_rows = batch_rows(P, s0, n_sl);
  gw::KTimer tm(P->ctx, GW_K_ROW);
  k_row_fused<M, NB, MINB, HALF, BIL><<<(n_rows + NB - 1) / NB, NT, smem, P->ctx->stream>>>(
      a, cz, P->d_fty, s0, n_sl, n_rows, P->Nc, P->d_F1);
  GW_LAUNCHED(P->ctx);
  return GW_OK;
}

// Block-shape variants of the nearest-bin, half-length form (the batched
// workloads' case); every other form runs variant 0.
template <int M, bool HALF, bool BIL>
int row_variant(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz, int s0,
                int n) {
  constexpr auto V = kFusedVariants;
  if constexpr (HALF && !BIL) {
    switch (P->p.block_variant) {
      case 1: return launch_row_fused<M, V[1].nb, V[1].minb, HALF, BIL>(P, a, cz, s0, n);
      case 2: return launch_row_fused<M, V[2].nb, V[2].minb, HALF, BIL>(P, a, cz, s0, n);
      case 3: return launch_row_fused<M, V[3].nb, V[3].minb, HALF, BIL>(P, a, cz, s0, n);
      default: break;
    }
  }
  return launch_row_fused<M, V[0].nb, V[0].minb, HALF, BIL>(P, a, cz, s0, n);
}

template <int M>
int row_fused(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz, int s0, int n) {
  const bool h = half_fits<M>(cz.L, cz.N);
  if (a.bil) return h ? row_variant<M, true, true>(P, a, cz, s0, n)
                      : row_variant<M, false, true>(P, a, cz, s0, n);
  return h ? row_variant<M, true, false>(P, a, cz, s0, n)
           : row_variant<M, false, false>(P, a, cz, s0, n);
}

// W_M^{n2 k1} in float64 with the exponent reduced mod M exactly.
std::vector<float2> twiddle_table(int M, int R1, int R2) {
  std::vector<float2> t((size_t)R1 * R2);
  for (int n2 = 0; n2 < R2; ++n2)
    for (int k1 = 0; k1 < R1; ++k1) {
      const long long e = ((long long)n2 * k1) % M;
      const double ang = -2.0 * M_PI * (double)e / (double)M;
      t[(size_t)n2 * R1 + k1] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
  return t;
}

}  // namespace

namespace gwv {

bool fused_supported(int M) { return M == 1024 || M == 1280; }

int fused_variant_count() { return czt2::kFusedVariantCount; }

std::vector<float2> fused_twiddles(int M) {
  switch (M) {
    case 1024: return twiddle_table(1024, Fused<1024>::R1, Fused<1024>::R2);
    case 1280: return twiddle_table(1280, Fused<1280>::R1, Fused<1280>::R2);
  }
  return {};
}

int fused_row_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                       int s0, int n) {
  switch (P->My) {
    case 1024: return row_fused<1024>(P, a, cz, s0, n);
    case 1280: return row_fused<1280>(P, a, cz, s0, n);
  }
  return gw::fail(GW_ERR_ARG, "no fused row transform of this length");
}

}  // namespace gwv
