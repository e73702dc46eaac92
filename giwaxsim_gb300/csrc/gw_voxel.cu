// Voxel stage: atoms -> per-phi projected scattering-factor slices -> 2-D
// DFT -> |F|^2 -> rotational binning -> I(q) average, crop and f0 factor.
//
// Reference: tools/comparison.py:673-788 (voxelgridmaker_fitting), the
// per-slice worker tools/voxelgrids.py:311-416 and the binning
// tools/voxelgrids.py:464-506.
//
// GB300 design (batched mode):
//  * A slice's real-space grid is D + Cbg, with Cbg the constant background
//    that fill_bkg/smoothing paint outside the slab and D compactly
//    supported (slab footprint plus the Gaussian tail).  DFT(Cbg) is a
//    single value at q = 0, added back before |.|^2.  Only D is transformed.
//  * Only the output rows/columns whose pixels land in the cropped cube are
//    produced: each 1-D DFT is a band-limited chirp-z transform
//    X[k0+m] = B[m] * sum_n (D[n] A[n]) h[m-n], evaluated as a circular
//    convolution with mixed-radix shared-memory FFTs (gw_fft.cuh).
//  * Row transforms (along y) write an intermediate F1[slice][z][col];
//    column transforms (along z) finish the DFT and either bin |F|^2 into
//    the float64 sum grid of the cropped cube with atomics, or store each
//    pixel for the gather binning (k_gather: every voxel summed in a fixed
//    order, then finalized in the same pass).
//  * Real grids (one phase per structure): two window rows per row
//    transform, only the columns ky >= 0, mirrored binning
//    (gw_stockham_row.cu, gw_stockham_col.cu).
//  * Counts depend only on geometry and factor as C2[qy,qx] * C1[qz]; the
//    count grid is never materialised.
// Plain mode keeps the reference's structure: the full g x g grid with its
// background, the full transform, binning into the whole q_num^3 cube and a
// crop afterwards, one slice per launch sequence.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "gw_tma.cuh"
#include "gw_voxel_impl.cuh"

using namespace gwv;

namespace {

// ------------------------------------------------------------ structure prep
__global__ void k_zmin(const double *xyz, const gw_structure *st,
                       unsigned long long *zmin_ord) {
  const gw_structure s = st[blockIdx.y];
  unsigned long long best = ~0ULL;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    double z = xyz[3 * (s.atom_begin + i) + 2];
    best = min(best, dbl_ord(z));
  }
  for (int o = 16; o > 0; o >>= 1)
    best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best != ~0ULL)
    atomicMin(zmin_ord + blockIdx.y, best);
}

// z index is phi independent: rotation about z leaves z unchanged
// (fma(z,1,fma(y,0,x*0)) == z), utilities.py:303-317.  Atoms are counted per
// z row (bin g collects z >= g, dropped by every slice's valid mask).
__global__ void k_zidx_hist(const double *xyz, const gw_structure *st,
                            const unsigned long long *zmin_ord, double r,
                            double inv_r, int g, int *zidx, int *hist) {
  const gw_structure s = st[blockIdx.y];
  const double zmin = ord_dbl(zmin_ord[blockIdx.y]);
  int *h = hist + (size_t)blockIdx.y * (g + 1);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = s.atom_begin + i;
    const double z = GW_DSUB(xyz[3 * a + 2], zmin);
    const int zi = (int)floor_div_exact(z, r, inv_r);
    zidx[a] = zi;
    atomicAdd(h + (zi >= 0 && zi < g ? zi : g), 1);
  }
}

// Per structure: exclusive scan of the row histogram into absolute offsets
// rowstart[0..g+1], scatter cursors, and (largest occupied row, all valid).
__global__ void __launch_bounds__(1024)
k_zscan(const gw_structure *st, int g, const int *hist, int *rowstart,
        int *cursor, int2 *zstat) {
  __shared__ int warp_sum[32];
  const int t = blockIdx.x;
  const int *h = hist + (size_t)t * (g + 1);
  int *rs = rowstart + (size_t)t * (g + 2);
  int *cur = cursor + (size_t)t * (g + 1);
  const int nb = g + 1;
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  int local = 0, zmax = -1;
  for (int k = 0; k < per; ++k) {
    const int b = b0 + k;
    if (b < nb) {
      local += h[b];
      if (b < g && h[b] > 0) zmax = b;
    }
  }
  // block exclusive scan of `local`
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int ws = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += v;
    }
    warp_sum[lane] = ws;
  }
  __syncthreads();
  int run = (int)st[t].atom_begin + (wid ? warp_sum[wid - 1] : 0) + incl - local;
  for (int k = 0; k < per; ++k) {
    const int b = b0 + k;
    if (b < nb) {
      rs[b] = run;
      cur[b] = run;
      run += h[b];
    }
  }
  if (threadIdx.x == blockDim.x - 1) rs[nb] = (int)(st[t].atom_begin + st[t].atom_count);
  zmax = __reduce_max_sync(0xffffffffu, zmax);
  __shared__ int zm;
  if (threadIdx.x == 0) zm = -1;
  __syncthreads();
  if (lane == 0) atomicMax(&zm, zmax);
  __syncthreads();
  if (threadIdx.x == 0) zstat[t] = make_int2(zm, h[g] == 0);
}

// Counting-sort scatter by z index.  Also records the permutation (sorted
// position -> input index) and, for the bilinear deposit, the fractional z
// position (z - zmin)/r - zi of each atom.
__global__ void k_zscatter(const double *xyz, const float2 *f,
                           const gw_structure *st, const int *zidx, int g,
                           const unsigned long long *zmin_ord, double inv_r,
                           int *cursor, double *xyz_s, float4 *xyf_s,
                           int *perm, float *fz_s) {
  const gw_structure s = st[blockIdx.y];
  int *cur = cursor + (size_t)blockIdx.y * (g + 1);
  const double zmin = ord_dbl(zmin_ord[blockIdx.y]);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = s.atom_begin + i;
    const int zi = zidx[a];
    const int pos = atomicAdd(cur + (zi >= 0 && zi < g ? zi : g), 1);
    xyz_s[3 * (size_t)pos] = xyz[3 * a];
    xyz_s[3 * (size_t)pos + 1] = xyz[3 * a + 1];
    xyz_s[3 * (size_t)pos + 2] = xyz[3 * a + 2];
    const float2 fa = f[a];
    xyf_s[pos] = make_float4((float)xyz[3 * a], (float)xyz[3 * a + 1], fa.x, fa.y);
    perm[pos] = (int)a;
    if (fz_s) {
      const double v = GW_DMUL(GW_DSUB(xyz[3 * a + 2], zmin), inv_r);
      fz_s[pos] = fminf(fmaxf((float)(v - (double)zi), 0.f), 1.f);
    }
  }
}

// ------------------------------------------------------------ per slice
// Per slice: min and max of the rotated y over all atoms (the shift to the
// minimum, voxelgrids.py:323), and the slice's background constants.
// Per-slice extremes of the rotated y' = x sin(phi) + y cos(phi) over all
// atoms of the structure (voxelgrids.py:325-330: np.min / np.max of
// rot[:, 1]), exact in float64, in two passes over the z-sorted atoms.
// Pass 1 (k_ybound) evaluates y' in float32 with a rigorous error bound d
// (10 u (|x s| + |y c|), u = 2^-24: input, product and fma roundings total
// about 4.1 u of that sum) and keeps lo = min(y' + d) and hi = max(y' - d),
// rounded outward.  Pass 2 (k_yminmax) evaluates the float64 chain only for
// the atoms whose interval reaches below lo or above hi: every other atom's
// exact value is above lo >= the exact minimum (below hi <= the maximum).
__device__ __forceinline__ unsigned flt_ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_flt(unsigned o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ void y_interval(const float4 q, float cs, float sn,
                                           float &lo, float &hi) {
  const float xs = q.x * sn, yc = q.y * cs;
  const float t = fmaf(q.y, cs, xs);
  const float d = 10.f * 5.9604645e-8f * (fabsf(xs) + fabsf(yc));
  lo = __fsub_rd(t, d);
  hi = __fadd_ru(t, d);
}

// lo bounds to the largest ordered value, hi bounds to the smallest
__global__ void k_yreset(unsigned *ybnd, int s0, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    ybnd[2 * (size_t)(s0 + i)] = ~0u;
    ybnd[2 * (size_t)(s0 + i) + 1] = 0u;
  }
}

// Both passes give a block kYS consecutive slices of the batch: a thread
// loads an atom once and evaluates it for each of them (the atoms stay in
// L2; one load per atom and slice made the passes L2-bound).  Slices of
// different structures in one block are taken as runs of the same
// structure, each over its own atoms.
constexpr int kYS = 4;

// Run [kb, ke) of the block's slices k0 + k that share one structure.
__device__ __forceinline__ int y_run_end(const SliceArgs &a, int first, int kb,
                                         int ns) {
  const int t = (first + kb) / a.n_phi;
  int ke = kb + 1;
  while (ke < ns && (first + ke) / a.n_phi == t) ++ke;
  return ke;
}

// Block reduction of kYS (min, max) pairs; thread 0 gets the results.
template <typename T>
__device__ __forceinline__ void y_block_reduce(T (&lo)[kYS], T (&hi)[kYS]) {
  __shared__ T s_lo[kYS][32], s_hi[kYS][32];
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < kYS; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
    if ((threadIdx.x & 31) == 0) { s_lo[k][w] = lo[k]; s_hi[k][w] = hi[k]; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kYS; ++k)
      for (int j = 1; j < nw; ++j) {
        lo[k] = min(lo[k], s_lo[k][j]);
        hi[k] = max(hi[k], s_hi[k][j]);
      }
  }
}

__global__ void k_ybound(SliceArgs a, int slice0, int n) {
  const int first = slice0 + blockIdx.y * kYS;
  const int ns = min(kYS, slice0 + n - first);
  float cs[kYS], sn[kYS];
  unsigned lo[kYS], hi[kYS];  // ordered: min of (y'+d), max of (y'-d)
#pragma unroll
  for (int k = 0; k < kYS; ++k) {
    const int p = (first + min(k, ns - 1)) % a.n_phi;
    cs[k] = (float)a.ph[p].cos_phi;
    sn[k] = (float)a.ph[p].sin_phi;
    lo[k] = ~0u;
    hi[k] = 0u;
  }
  for (int kb = 0; kb < ns;) {
    const int ke = y_run_end(a, first, kb, ns);
    const gw_structure s = a.st[(first + kb) / a.n_phi];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
      const float4 q = a.xyf_s[s.atom_begin + i];
#pragma unroll
      for (int k = 0; k < kYS; ++k) {
        if (k < kb || k >= ke) continue;
        float l, h;
        y_interval(q, cs[k], sn[k], l, h);
        lo[k] = min(lo[k], flt_ord(h));
        hi[k] = max(hi[k], flt_ord(l));
      }
    }
    kb = ke;
  }
  // block reduction, then one atomic per block, slice and bound
  y_block_reduce(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kYS; ++k) {
      if (k >= ns || lo[k] == ~0u) continue;
      atomicMin(a.ybnd + 2 * (size_t)(first + k), lo[k]);
      atomicMax(a.ybnd + 2 * (size_t)(first + k) + 1, hi[k]);
    }
  }
}

__global__ void k_yminmax(SliceArgs a, int slice0, int n) {
  const int first = slice0 + blockIdx.y * kYS;
  const int ns = min(kYS, slice0 + n - first);
  if (blockIdx.x == 0 && threadIdx.x < ns) {
    // background constant C = avg_voxel_f * max_voxels (voxelgrids.py:358,365):
    // Cbg is what the transformed window excludes (batched mode), Cd what
    // stays inside it
    const int sl = first + threadIdx.x;
    const gw_structure s = a.st[sl / a.n_phi];
    const float2 c = make_float2((float)GW_DMUL(s.avg_f_re, s.max_voxels),
                                 (float)GW_DMUL(s.avg_f_im, s.max_voxels));
    const bool bg = !a.plain && (a.fill || a.smooth_on);
    a.sconst[sl] = bg ? make_float4(c.x, c.y, 0.f, 0.f)
                      : make_float4(0.f, 0.f, c.x, c.y);
  }
  double c[kYS], sn[kYS];
  float blo[kYS], bhi[kYS];
  unsigned long long lo[kYS], hi[kYS];
#pragma unroll
  for (int k = 0; k < kYS; ++k) {
    const int sl = first + min(k, ns - 1);
    const int p = sl % a.n_phi;
    c[k] = a.ph[p].cos_phi;
    sn[k] = a.ph[p].sin_phi;
    blo[k] = ord_flt(a.ybnd[2 * (size_t)sl]);
    bhi[k] = ord_flt(a.ybnd[2 * (size_t)sl + 1]);
    lo[k] = ~0ULL;
    hi[k] = 0ULL;
  }
  for (int kb = 0; kb < ns;) {
    const int ke = y_run_end(a, first, kb, ns);
    const gw_structure s = a.st[(first + kb) / a.n_phi];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
      const float4 q = a.xyf_s[s.atom_begin + i];
#pragma unroll
      for (int k = 0; k < kYS; ++k) {
        if (k < kb || k >= ke) continue;
        float l, h;
        y_interval(q, (float)c[k], (float)sn[k], l, h);
        if (l <= blo[k] || h >= bhi[k]) {
          const unsigned long long v =
              dbl_ord(rot_y(a.xyz_s + 3 * (s.atom_begin + i), c[k], sn[k]));
          lo[k] = min(lo[k], v);
          hi[k] = max(hi[k], v);
        }
      }
    }
    kb = ke;
  }
  y_block_reduce(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kYS; ++k) {
      if (k >= ns || lo[k] == ~0ULL) continue;
      atomicMin(a.ymin_ord + first + k, lo[k]);
      atomicMax(a.ymax_ord + first + k, hi[k]);
    }
  }
}

// Per slice extents of the valid atoms (voxelgrids.py:346-349).  y indices
// grow with y (the floor division is monotone), so when every atom is valid
// the extents are (0, index of max y, 0, largest occupied z row); otherwise
// k_ext_exact computes them atom by atom.
__global__ void k_ext(SliceArgs a, int slice0, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sl = slice0 + i;
  const int t = sl / a.n_phi;
  const double ymin = ord_dbl(a.ymin_ord[sl]), ymax = ord_dbl(a.ymax_ord[sl]);
  const double Y = floor_div_exact(GW_DSUB(ymax, ymin), a.r, a.inv_r);
  const int2 zs = a.zstat[t];
  if (Y < (double)a.g && zs.y) {
    a.ext[sl] = make_int4(0, (int)Y, 0, zs.x);
    a.extflag[sl] = 0;
  } else {
    a.ext[sl] = make_int4(INT_MAX, -1, INT_MAX, -1);
    a.extflag[sl] = 1;
  }
}

__global__ void k_ext_exact(SliceArgs a, int slice0) {
  const int sl = slice0 + blockIdx.y;
  if (!a.extflag[sl]) return;
  const int t = sl / a.n_phi, p = sl % a.n_phi;
  const gw_structure s = a.st[t];
  const double c = a.ph[p].cos_phi, sn = a.ph[p].sin_phi;
  const double ymin = ord_dbl(a.ymin_ord[sl]);
  int ymn = INT_MAX, ymx = -1, zmn = INT_MAX, zmx = -1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t at = s.atom_begin + i;
    const double y = GW_DSUB(rot_y(a.xyz + 3 * at, c, sn), ymin);
    const int yi = (int)floor_div_exact(y, a.r, a.inv_r);
    const int zi = a.zidx[at];
    if (yi >= 0 && yi < a.g && zi >= 0 && zi < a.g) {
      ymn = min(ymn, yi); ymx = max(ymx, yi);
      zmn = min(zmn, zi); zmx = max(zmx, zi);
    }
  }
  ymn = __reduce_min_sync(0xffffffffu, ymn);
  ymx = __reduce_max_sync(0xffffffffu, ymx);
  zmn = __reduce_min_sync(0xffffffffu, zmn);
  zmx = __reduce_max_sync(0xffffffffu, zmx);
  if ((threadIdx.x & 31) == 0 && ymx >= 0) {
    int4 *e = a.ext + sl;
    atomicMin(&e->x, ymn); atomicMax(&e->y, ymx);
    atomicMin(&e->z, zmn); atomicMax(&e->w, zmx);
  }
}

// Per-slice profiles: fill_bkg column term (minus the background) and the
// two separable smoothing masks (voxelgrids.py:344-379).
__global__ void k_profile(SliceArgs a, int slice0) {
  const int sl = slice0 + blockIdx.x;
  const int t = sl / a.n_phi, p = sl % a.n_phi;
  const gw_structure s = a.st[t];
  const gw_phi ph = a.ph[p];
  const int4 e = a.ext[sl];
  if (e.y < 0) {  // no valid atom: np.min of an empty array raises
    if (threadIdx.x == 0 && blockIdx.y == 0) dev_error(a.err, GW_DEVERR_NO_ATOMS);
    return;
  }
  const double cre = GW_DMUL(s.avg_f_re, s.max_voxels);
  const double cim = GW_DMUL(s.avg_f_im, s.max_voxels);
  const bool bg = !a.plain && (a.fill || a.smooth_on);
  // blockIdx.y-th part of the columns / rows
  const int i0 = blockIdx.y * blockDim.x + threadIdx.x;
  const int di = gridDim.y * blockDim.x;
  const bool lead = blockIdx.y == 0 && threadIdx.x == 0;
  if (a.fill) {
    const double base = a.clbase[sl];
    for (int yy = i0; yy < a.Ly; yy += di) {
      int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
      const double x = GW_DMUL((double)yi, a.r);
      const double len = collapse_length(ph, s.y_bound, s.x_bound, base, x);
      const double nm = GW_DSUB(s.max_voxels, floor_div_exact(len, a.r, a.inv_r));
      const double n_missing = (double)(long long)nm;
      double re = GW_DMUL(n_missing, s.avg_f_re);
      double im = GW_DMUL(n_missing, s.avg_f_im);
      if (bg) { re -= cre; im -= cim; }
      a.amo[(size_t)blockIdx.x * a.Ly + yy] = make_float2((float)re, (float)im);
    }
  }
  if (a.smooth_on) {
    int ys, ye, zs, ze;
    plateau(a, e, ys, ye, zs, ze);
    for (int yy = i0; yy < a.Ly; yy += di) {
      int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
      a.my[(size_t)blockIdx.x * a.Ly + yy] = smooth_at(yi, ys, ye, a.g, a.radius, a.gw);
    }
    for (int zz = i0; zz < a.Lz; zz += di) {
      int zi = a.z_lo + zz; if (zi < 0) zi += a.g; if (zi >= a.g) zi -= a.g;
      a.mz[(size_t)blockIdx.x * a.Lz + zz] = smooth_at(zi, zs, ze, a.g, a.radius, a.gw);
    }
    // the smoothing support must lie inside the transformed window
    if (lead && a.Ly < a.g) {
      int l = a.y_lo - 1; if (l < 0) l += a.g;
      int r = a.y_lo + a.Ly; r %= a.g; if (r < 0) r += a.g;
      if (smooth_at(l, ys, ye, a.g, a.radius, a.gw) != 0.f ||
          smooth_at(r, ys, ye, a.g, a.radius, a.gw) != 0.f)
        dev_error(a.err, GW_DEVERR_MASK_WRAP);
    }
    if (lead && a.Lz < a.g) {
      const int rows = a.roff ? a.roff[sl + 1] - a.roff[sl] : a.Lz;
      int l = a.z_lo - 1; if (l < 0) l += a.g;
      int r = a.z_lo + rows; r %= a.g; if (r < 0) r += a.g;
      if (smooth_at(l, zs, ze, a.g, a.radius, a.gw) != 0.f ||
          smooth_at(r, zs, ze, a.g, a.radius, a.gw) != 0.f)
        dev_error(a.err, GW_DEVERR_MASK_WRAP);
    }
  }
  if (a.pr) {
    // real grids: the row kernel's per-column table (d_value_row_real);
    // this thread's own amo and my entries, written above
    const float2 u = unit_phase(s);
    const float nan = __int_as_float(0x7fc00000);
    for (int yy = i0; yy < a.Ly; yy += di) {
      const size_t o = (size_t)blockIdx.x * a.Ly + yy;
      float x = 0.f;
      if (a.fill) {
        int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
        const float2 am = a.amo[o];
        x = (yi > e.x && yi < e.y) ? am.x * u.x + am.y * u.y : nan;
      }
      a.pr[o] = make_float2(x, a.smooth_on ? a.my[o] : 1.f);
    }
  }
}

// ---------------------------------------------------------- geometry tables
// Column tables per phi (voxelgrids.py:396-401 slice axes, :475-498 mask and
// indices): window offset ((iy-wlo)*W + (ix-wlo))*W, or -1.
__global__ void k_col_tables(const gw_phi *ph, int g, int k0, int nc,
                             double qmin, double qmax, double dq, double inv_dq,
                             int wlo, int whi, int W, int *colofs,
                             unsigned int *C2) {
  const int p = blockIdx.x;
  const double rqy = ph[p].right_qy, rqx = ph[p].right_qx;
  for (int m = threadIdx.x; m < nc; m += blockDim.x) {
    const int c = k0 + m + g / 2;  // column index of the shifted slice
    int out = -1;
    if (c >= 0 && c < g) {
      const double hy = linspace_at(-rqy, rqy, g, c);
      const double hx = linspace_at(-rqx, rqx, g, c);
      if (hx <= qmax && hx >= qmin && hy <= qmax && hy >= qmin) {
        const int ix = (int)floor_div_exact(GW_DSUB(hx, qmin), dq, inv_dq);
        const int iy = (int)floor_div_exact(GW_DSUB(hy, qmin), dq, inv_dq);
        if (ix >= wlo && ix <= whi && iy >= wlo && iy <= whi) {
          out = ((iy - wlo) * W + (ix - wlo)) * W;
          atomicAdd(C2 + (iy - wlo) * W + (ix - wlo), 1u);
        }
      }
    }
    colofs[(size_t)p * nc + m] = out;
  }
}

// I = sum / count (0 where count == 0), crop, f0 factor (comparison.py:765-786,
// voxelgrids.py:16-48, :828-857).  Output in crop coordinates (qy,qx,qz).
// One warp per (qy, qx) line, lanes along qz (the contiguous axis), lines
// in a grid-stride loop.  The count grid factorises, count = C2[line] *
// C1[z]; a voxel's factor is (inv_nstruct / C2) (1 / C1) (count_factors),
// with the z reciprocals and the four f0 z factors staged in shared memory
// per block and, per line, C2's factor and the (qx, qy) part of the
// separable f0 sum in registers.  A line with C2 = 0 holds no binned pixel:
// zeros, no sum read; a voxel with C1 = 0 gets a zero factor.  F64: the float64 I(q)
// (the sum times the float32 factor, one float64 multiply); otherwise the
// float32 I(q) the detector gathers from, computed in float32 from the sum
// rounded to float (no float64 arithmetic: on this GPU the float64 pipe is
// the slow one), within 1.5 float32 ulps of the float64 I(q) rounded (both
// use the same factor).  Dynamic shared memory: Qc float4 (use_f0) + Qc
// floats.
constexpr int kFinU = 8;  // voxels per lane per round of k_finalize

template <bool F64>
__global__ void __launch_bounds__(256)
k_finalize(const double *__restrict__ sum, const float2 *__restrict__ sumk, int kahan,
           const unsigned int *__restrict__ C2, const int *__restrict__ C1, int W,
           int off, int Qc, float inv_nstruct, const float *__restrict__ f0tab,
           const float4 *__restrict__ zf0, int use_f0, float f0_c, float f0_invz,
           double *__restrict__ out64, float *__restrict__ out32) {
  extern __shared__ float4 s_zf0[];
  float *s_rc1 = reinterpret_cast<float *>(s_zf0 + (use_f0 ? Qc : 0));
  for (int iz = threadIdx.x; iz < Qc; iz += blockDim.x) {
    s_rc1[iz] = z_count_factor((unsigned)C1[iz + off]);
    if (use_f0) s_zf0[iz] = zf0[iz];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int n_lines = Qc * Qc;
  const int stride = gridDim.x * (blockDim.x >> 5);
  for (int line = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       line < n_lines; line += stride) {
    const int iy = line / Qc, ix = line - iy * Qc;
    const int wy = iy + off, wx = ix + off;
    const unsigned c2 = C2[(size_t)wy * W + wx];
    const size_t obase = (size_t)line * Qc;
    if (c2 == 0u) {
      for (int iz = lane; iz < Qc; iz += 32) {
        if (F64) out64[obase + iz] = 0.0;
        else out32[obase + iz] = 0.f;
      }
      continue;
    }
    const size_t wbase = ((size_t)wy * W + wx) * W + off;
    const float r2 = line_count_factor(c2, inv_nstruct);
    float fxy[4] = {0.f, 0.f, 0.f, 0.f};
    if (use_f0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float *t = f0tab + i * 3 * Qc;
        fxy[i] = __ldg(t + ix) * __ldg(t + Qc + iy);
      }
    }
    // kFinU voxels per lane per round: every sum load of the round is
    // issued before the first is used (a voxel with C1 = 0 loads its zero
    // sum too), so each warp keeps kFinU loads in flight.  Both sum kinds
    // are 8 bytes a voxel: loaded as raw words, read as a float64 or as a
    // (sum, compensation) float pair.
    const unsigned long long *raw =
        kahan ? reinterpret_cast<const unsigned long long *>(sumk) + wbase
              : reinterpret_cast<const unsigned long long *>(sum) + wbase;
    for (int iz0 = 0; iz0 < Qc; iz0 += 32 * kFinU) {
      unsigned long long w[kFinU];
#pragma unroll
      for (int u = 0; u < kFinU; ++u) {
        const int iz = iz0 + u * 32 + lane;
        w[u] = iz < Qc ? raw[iz] : 0ull;
      }
#pragma unroll
      for (int u = 0; u < kFinU; ++u) {
        const int iz = iz0 + u * 32 + lane;
        if (iz >= Qc) break;
        double s = 0.0;
        float s32 = 0.f;
        if (kahan) {
          const float sx = __uint_as_float((unsigned)w[u]);
          const float sc = __uint_as_float((unsigned)(w[u] >> 32));
          if (F64) s = f2d_exact(sx) - f2d_exact(sc);
          else s32 = sx - sc;
        } else if (F64) {
          s = __longlong_as_double((long long)w[u]);
        } else {
          s32 = d2f_rn(__longlong_as_double((long long)w[u]));
        }
        float scale = r2 * s_rc1[iz];
        if (use_f0) {
          const float4 z = s_zf0[iz];
          float acc = f0_c;
          acc += fxy[0] * z.x;
          acc += fxy[1] * z.y;
          acc += fxy[2] * z.z;
          acc += fxy[3] * z.w;
          const float fq = acc * f0_invz;
          scale *= fq * fq;
        }
        if (F64) out64[obase + iz] = s * f2d_exact(scale);
        else out32[obase + iz] = s32 * scale;
      }
    }
  }
}

size_t finalize_smem(int Qc, bool use_f0) {
  return (size_t)Qc * ((use_f0 ? sizeof(float4) : 0) + sizeof(float));
}

// Gather binning: the sums of one voxel line in a fixed order, then the
// finalize of k_finalize.  A warp runs along qz in spans of 32 U voxels
// (qz = z0 + lane + 32 u).  A line's entries (phi, F1 column,
// mirrored) are taken in table order (phi, then band column), kGatherP at
// a time with the pixel loads of all their voxels issued together, each
// over the structures t0 .. t1-1 (the slice t n_phi + phi); the pixel of
// voxel qz is output row mr of the z table (mirrored: row 2 r_zero - mr).
// Pixels are float32 and the running sum is compensated (Kahan) float32:
// the exact sum to about one float32 ulp, the same bits on every run.
// Voxels with further output rows (C1 > 1) are summed again over all rows
// by k_gather_multi.  Lines with up to kGatherHeavy pixels per voxel
// (entries times structures) take one warp each (grid-stride); the heavier
// lines (near the rotation axis every phi meets) are listed in `heavy` and
// take one block each, its warps
// splitting the entries in eight fixed parts whose partial sums are added
// in warp order.  Three blocks per SM (measured faster than two without
// the few spilled registers of U = 13).
// MODE 0: the float32 I(q) (crop, factor, f0 as k_finalize); 1: the float64
// I(q) from the same sums; 2: the float64 sums into the window grid (crop
// = window, off = 0; no factor).
constexpr int kGatherHeavy = 64;

__device__ __forceinline__ void kahan_step(float &hi, float &lo, float x) {
  const float y = x - lo;
  const float s = hi + y;
  lo = (s - hi) - y;
  hi = s;
}

// A warp's pass over a span of up to 32 U voxels of a line (qz = z0 +
// lane + 32 u): kGatherP entries at a time, the pixel loads of all their
// voxels issued together, then added (compensated) in entry order.  U is
// picked per launch so that a span covers a whole line (U = 13: lines of up
// to 416 voxels; U = 7: up to 224).
constexpr int kGatherP = 1;

template <int U>
__device__ __forceinline__ void gather_span(const float *__restrict__ G,
                                            const int2 *__restrict__ lent, int e0,
                                            int e1, int t0, int t1, int n_phi, int nf,
                                            int nr, int r_zero, const int *s_row, int z0,
                                            int lane, int Qc, float (&hi)[U],
                                            float (&lo)[U]) {
  const unsigned tstep = (unsigned)n_phi * (unsigned)nf * (unsigned)nr;
  int mr[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int iz = z0 + lane + 32 * u;
    mr[u] = iz < Qc ? s_row[iz] : -1;
  }
#pragma unroll 1
  for (int e = e0; e < e1; e += kGatherP) {
    const int ne = min(kGatherP, e1 - e);
    unsigned col[kGatherP];
    bool flip[kGatherP];
#pragma unroll
    for (int k = 0; k < kGatherP; ++k) {
      const int2 en = k < ne ? __ldg(lent + e + k) : make_int2(0, 0);
      col[k] = ((unsigned)(t0 * n_phi + en.x) * (unsigned)nf + (unsigned)(en.y >> 1)) *
               (unsigned)nr;
      flip[k] = en.y & 1;
    }
#pragma unroll 1
    for (int t = t0; t < t1; ++t) {
      float v[kGatherP][U];
#pragma unroll
      for (int k = 0; k < kGatherP; ++k)
#pragma unroll
        for (int u = 0; u < U; ++u)
          v[k][u] = (k < ne && mr[u] >= 0)
                        ? __ldg(G + col[k] + (unsigned)(flip[k] ? 2 * r_zero - mr[u] : mr[u]))
                        : 0.f;
#pragma unroll
      for (int k = 0; k < kGatherP; ++k) {
        if (k >= ne) break;
#pragma unroll
        for (int u = 0; u < U; ++u) kahan_step(hi[u], lo[u], v[k][u]);
        col[k] += tstep;
      }
    }
  }
}

template <int MODE>
__device__ __forceinline__ void gather_store(float hi, float lo, int iz, size_t obase,
                                             float r2, const float *s_rc1,
                                             const float4 *s_zf0, const float (&fxy)[4],
                                             int use_f0, float f0_c, float f0_invz,
                                             double *out64, float *out32) {
  if (MODE == 2) {
    out64[obase + iz] = f2d_exact(hi) - f2d_exact(lo);
    return;
  }
  float scale = r2 * s_rc1[iz];
  if (use_f0) {
    const float4 z = s_zf0[iz];
    float acc = f0_c;
    acc += fxy[0] * z.x;
    acc += fxy[1] * z.y;
    acc += fxy[2] * z.z;
    acc += fxy[3] * z.w;
    const float fq = acc * f0_invz;
    scale *= fq * fq;
  }
  if (MODE == 1) out64[obase + iz] = (f2d_exact(hi) - f2d_exact(lo)) * f2d_exact(scale);
  else out32[obase + iz] = (hi - lo) * scale;
}

template <int MODE, int U>
__global__ void __launch_bounds__(256, 3)
k_gather(const float *__restrict__ G, const int *__restrict__ lptr,
         const int2 *__restrict__ lent, const int *__restrict__ zptr,
         const int *__restrict__ zrows, const int *__restrict__ heavy, int n_heavy,
         int heavy_on, int line_lo, int line_hi, int nf, int nr, int r_zero, int n_phi,
         int t0, int t1, const unsigned int *__restrict__ C2, const int *__restrict__ C1,
         int W, int off, int Qc, float inv_nstruct, const float *__restrict__ f0tab,
         const float4 *__restrict__ zf0, int use_f0, float f0_c, float f0_invz,
         double *__restrict__ out64, float *__restrict__ out32) {
  extern __shared__ float4 s_zf0[];
  float *s_rc1 = reinterpret_cast<float *>(s_zf0 + (use_f0 ? Qc : 0));
  int *s_row = reinterpret_cast<int *>(s_rc1 + Qc);  // first output row per qz
  // [8][Qc] partial sums: 8-byte aligned (20 Qc or 4 Qc bytes before s_row)
  float2 *s_part = reinterpret_cast<float2 *>(s_row + Qc);
  for (int iz = threadIdx.x; iz < Qc; iz += blockDim.x) {
    s_rc1[iz] = z_count_factor((unsigned)C1[iz + off]);
    if (use_f0) s_zf0[iz] = zf0[iz];
    const int r0 = zptr[iz + off];
    s_row[iz] = zptr[iz + off + 1] > r0 ? zrows[r0] : -1;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto line_consts = [&](int iy, int ix, int wl, float &r2, float (&fxy)[4]) {
    r2 = 0.f;
    fxy[0] = fxy[1] = fxy[2] = fxy[3] = 0.f;
    if (MODE != 2) {
      r2 = line_count_factor(C2[wl], inv_nstruct);
      if (use_f0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float *t = f0tab + i * 3 * Qc;
          fxy[i] = __ldg(t + ix) * __ldg(t + Qc + iy);
        }
      }
    }
  };
  if ((int)blockIdx.x < n_heavy) {
    // a heavy line: the block's eight warps split its entries
    const int wl = heavy[blockIdx.x];
    const int iy = wl / W - off, ix = wl % W - off;
    if (iy < 0 || iy >= Qc || ix < 0 || ix >= Qc) return;
    const int e0 = lptr[wl], ne = lptr[wl + 1] - e0;
    const int nw = blockDim.x >> 5;
    const int eb = e0 + (int)((int64_t)ne * warp / nw);
    const int ee = e0 + (int)((int64_t)ne * (warp + 1) / nw);
    for (int z0 = 0; z0 < Qc; z0 += 32 * U) {
      float hi[U], lo[U];
#pragma unroll
      for (int u = 0; u < U; ++u) hi[u] = lo[u] = 0.f;
      gather_span(G, lent, eb, ee, t0, t1, n_phi, nf, nr, r_zero, s_row, z0, lane, Qc, hi,
                  lo);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int iz = z0 + lane + 32 * u;
        if (iz < Qc) s_part[warp * Qc + iz] = make_float2(hi[u], lo[u]);
      }
    }
    __syncthreads();
    float r2, fxy[4];
    line_consts(iy, ix, wl, r2, fxy);
    const size_t obase = MODE == 2 ? (size_t)wl * W : ((size_t)iy * Qc + ix) * Qc;
    for (int iz = threadIdx.x; iz < Qc; iz += blockDim.x) {
      float hi = 0.f, lo = 0.f;
      for (int w = 0; w < nw; ++w) {
        const float2 p = s_part[w * Qc + iz];
        kahan_step(hi, lo, p.x);
        kahan_step(hi, lo, -p.y);
      }
      gather_store<MODE>(hi, lo, iz, obase, r2, s_rc1, s_zf0, fxy, use_f0, f0_c, f0_invz,
                         out64, out32);
    }
    return;
  }
  // the other lines of [line_lo, line_hi), one warp each, in spans of 32 U
  // voxels
  const int wpb = blockDim.x >> 5;
  const int stride = (gridDim.x - n_heavy) * wpb;
  for (int line = line_lo + (blockIdx.x - n_heavy) * wpb + warp; line < line_hi;
       line += stride) {
    const int iy = line / Qc, ix = line - iy * Qc;
    const int wl = (iy + off) * W + ix + off;
    const size_t obase = MODE == 2 ? (size_t)wl * W : (size_t)line * Qc;
    const int e0 = lptr[wl], e1 = lptr[wl + 1];
    if (heavy_on && (e1 - e0) * (t1 - t0) > kGatherHeavy) continue;  // a heavy block's
    if (e0 == e1) {
      for (int iz = lane; iz < Qc; iz += 32) {
        if (MODE == 0) out32[obase + iz] = 0.f;
        else out64[obase + iz] = 0.0;
      }
      continue;
    }
    float r2, fxy[4];
    line_consts(iy, ix, wl, r2, fxy);
    for (int z0 = 0; z0 < Qc; z0 += 32 * U) {
      float hi[U], lo[U];
#pragma unroll
      for (int u = 0; u < U; ++u) hi[u] = lo[u] = 0.f;
      gather_span(G, lent, e0, e1, t0, t1, n_phi, nf, nr, r_zero, s_row, z0, lane, Qc, hi,
                  lo);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int iz = z0 + lane + 32 * u;
        if (iz < Qc)
          gather_store<MODE>(hi[u], lo[u], iz, obase, r2, s_rc1, s_zf0, fxy, use_f0, f0_c,
                             f0_invz, out64, out32);
      }
    }
  }
}

// Voxels with more than one output row (C1 > 1, the window z listed in
// zmulti): their whole sum again over every row, in the order entry, then
// structure, then row, replacing the first-row value k_gather wrote.  One
// warp per line with entries, lanes over the listed z.
template <int MODE>
__global__ void __launch_bounds__(256)
k_gather_multi(const float *__restrict__ G, const int *__restrict__ lptr,
               const int2 *__restrict__ lent, const int *__restrict__ zptr,
               const int *__restrict__ zrows, const int *__restrict__ zmulti,
               int n_zmulti, int line_lo, int line_hi, int nf, int nr, int r_zero,
               int n_phi, int t0, int t1, const unsigned int *__restrict__ C2,
               const int *__restrict__ C1, int W, int off, int Qc, float inv_nstruct,
               const float *__restrict__ f0tab, const float4 *__restrict__ zf0,
               int use_f0, float f0_c, float f0_invz, double *__restrict__ out64,
               float *__restrict__ out32) {
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * (blockDim.x >> 5);
  for (int line = line_lo + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       line < line_hi; line += stride) {
    const int iy = line / Qc, ix = line - iy * Qc;
    const int wl = (iy + off) * W + ix + off;
    const int e0 = lptr[wl], e1 = lptr[wl + 1];
    if (e0 == e1) continue;
    const size_t obase = MODE == 2 ? (size_t)wl * W : (size_t)line * Qc;
    for (int i = lane; i < n_zmulti; i += 32) {
      const int wz = zmulti[i], iz = wz - off;
      if (iz < 0 || iz >= Qc) continue;
      float hi = 0.f, lo = 0.f;
      for (int e = e0; e < e1; ++e) {
        const int2 en = __ldg(lent + e);
        for (int t = t0; t < t1; ++t) {
          const float *col = G + ((size_t)(t * n_phi + en.x) * nf + (en.y >> 1)) * nr;
          for (int rr = zptr[wz]; rr < zptr[wz + 1]; ++rr) {
            const int m = zrows[rr];
            kahan_step(hi, lo, __ldg(col + ((en.y & 1) ? 2 * r_zero - m : m)));
          }
        }
      }
      if (MODE == 2) {
        out64[obase + iz] = f2d_exact(hi) - f2d_exact(lo);
        continue;
      }
      float scale = line_count_factor(C2[wl], inv_nstruct) * z_count_factor((unsigned)C1[wz]);
      if (use_f0) {
        const float4 z = zf0[iz];
        float fxy[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float *t = f0tab + k * 3 * Qc;
          fxy[k] = __ldg(t + ix) * __ldg(t + Qc + iy);
        }
        float acc = f0_c;
        acc += fxy[0] * z.x;
        acc += fxy[1] * z.y;
        acc += fxy[2] * z.z;
        acc += fxy[3] * z.w;
        const float fq = acc * f0_invz;
        scale *= fq * fq;
      }
      if (MODE == 1) out64[obase + iz] = (f2d_exact(hi) - f2d_exact(lo)) * f2d_exact(scale);
      else out32[obase + iz] = (hi - lo) * scale;
    }
  }
}

// Dynamic shared memory of k_gather: the finalize tables, the first output
// row per qz, and (heavy lines) eight partial sums per qz.
size_t gather_smem(int Qc, bool use_f0, bool heavy) {
  return finalize_smem(Qc, use_f0) + (size_t)Qc * sizeof(int) +
         (heavy ? (size_t)8 * Qc * sizeof(float2) : 0);
}

// Shell code of every window voxel (voxelgrids.py:651-652, :659-664, :706):
// |q| = sqrt((qx^2 + qy^2) + qz^2) as numpy evaluates the meshgrid sum, and
// shell k holds lower[k] < |q| <= upper[k].  Shells are increasing, so a
// voxel lies in at most two adjacent ones.
__global__ void k_shell_codes(const double *qw, int W, const double *lower,
                              const double *upper, int K, unsigned short *codes) {
  const int64_t n = (int64_t)W * W * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(i % W);
    const int64_t line = i / W;
    const int ix = (int)(line % W), iy = (int)(line / W);
    const double qx = qw[ix], qy = qw[iy], qz = qw[iz];
    const double qr = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(qx, qx), __dmul_rn(qy, qy)),
                                           __dmul_rn(qz, qz)));
    unsigned short c = kNoShell;
    for (int k = 0; k < K; ++k)
      if (qr <= upper[k] && qr > lower[k]) {
        const bool next = k + 1 < K && qr <= upper[k + 1] && qr > lower[k + 1];
        c = (unsigned short)(2 * k + (next ? 1 : 0));
        break;
      }
    codes[i] = c;
  }
}

// The reference's multi-q result (voxelgrids.py:703-707): the last shell's
// I(q) everywhere, doubled inside that shell.  Doubling is exact in float64
// and float32.
__global__ void k_shell_double(const unsigned short *codes, int W, int off,
                               int Qc, int k, double *out64, float *out32) {
  const int64_t n = (int64_t)Qc * Qc * Qc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(i % Qc);
    const int64_t line = i / Qc;
    const int ix = (int)(line % Qc), iy = (int)(line / Qc);
    const int64_t w = ((int64_t)(iy + off) * W + (ix + off)) * W + (iz + off);
    if (shell_member(codes[w], k)) {
      if (out64) out64[i] *= 2.0;
      if (out32) out32[i] *= 2.f;
    }
  }
}

// The deposited window of one slice (row zz, column yy) through the same
// sorted arrays and index code the row kernel uses.
__global__ void k_debug_window(SliceArgs a, int sl, float2 *win) {
  const int t = sl / a.n_phi;
  for (int zz = blockIdx.x; zz < a.Lz; zz += gridDim.x) {
    int lo, mid, hi;
    row_atoms(a, t, zz, lo, mid, hi);
    float2 *row = win + (size_t)zz * a.Ly;
    for (int at = lo + threadIdx.x; at < hi; at += blockDim.x) {
      if (!a.bil) {
        int yy;
        if (deposit_column(a, at, sl, yy) && yy < a.Ly) {
          atomicAdd(&row[yy].x, a.xyf_s[at].z);
          atomicAdd(&row[yy].y, a.xyf_s[at].w);
        }
      } else {
        int i0;
        float fu;
        if (bilinear_column(a, at, sl, i0, fu)) {
          const float wz = at >= mid ? 1.f - a.fz_s[at] : a.fz_s[at];
          const float2 fv = make_float2(a.xyf_s[at].z, a.xyf_s[at].w);
          for (int c = 0; c < 2; ++c) {
            const int i = i0 + c;
            const int yy = window_col(a, i);
            const float w = wz * (c ? fu : 1.f - fu);
            if (i < a.g && yy < a.Ly) {
              atomicAdd(&row[yy].x, fv.x * w);
              atomicAdd(&row[yy].y, fv.y * w);
            }
          }
        }
      }
    }
  }
}

// per-slice extents start empty: min fields INT_MAX, max fields -1
__global__ void k_ext_init(int4 *ext, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ext[i] = make_int4(INT_MAX, -1, INT_MAX, -1);
}

__global__ void k_debug_deposit(SliceArgs a, int sl, int *yo, int *zo) {
  const int t = sl / a.n_phi, p = sl % a.n_phi;
  const gw_structure s = a.st[t];
  const double c = a.ph[p].cos_phi, sn = a.ph[p].sin_phi;
  const double ymin = ord_dbl(a.ymin_ord[sl]);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < s.atom_count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t at = s.atom_begin + i;
    const double y = GW_DSUB(rot_y(a.xyz + 3 * at, c, sn), ymin);
    const int yi = (int)floor_div_exact(y, a.r, a.inv_r);
    const int zi = a.zidx[at];
    const bool ok = yi >= 0 && yi < a.g && zi >= 0 && zi < a.g;
    yo[i] = ok ? yi : -1;
    zo[i] = ok ? zi : -1;
  }
}

// ------------------------------------------------------------ host tables
using cd = std::complex<double>;

// Forward DFT (exp(-2 pi i/n)) in float64 for n = 2^k * odd: radix-2
// decimation in time down to the odd length, done directly.
void fft_inplace_host(std::vector<cd> &a) {
  const size_t n = a.size();
  if (n <= 1) return;
  if (n & 1) {
    std::vector<cd> out(n);
    for (size_t k = 0; k < n; ++k) {
      cd s(0, 0);
      for (size_t j = 0; j < n; ++j) {
        const double ang = -2.0 * M_PI * (double)((j * k) % n) / (double)n;
        s += a[j] * cd(std::cos(ang), std::sin(ang));
      }
      out[k] = s;
    }
    a.swap(out);
    return;
  }
  std::vector<cd> ev(n / 2), od(n / 2);
  for (size_t i = 0; i < n / 2; ++i) { ev[i] = a[2 * i]; od[i] = a[2 * i + 1]; }
  fft_inplace_host(ev);
  fft_inplace_host(od);
  for (size_t k = 0; k < n / 2; ++k) {
    const double ang = -2.0 * M_PI * (double)k / (double)n;
    const cd t = cd(std::cos(ang), std::sin(ang)) * od[k];
    a[k] = ev[k] + t;
    a[k + n / 2] = ev[k] - t;
  }
}

// exp(-i*pi*e/g) with e reduced mod 2g exactly
cd chirp(long long e, long long g) {
  long long m = e % (2 * g);
  if (m < 0) m += 2 * g;
  const double ang = -M_PI * (double)m / (double)g;
  return cd(std::cos(ang), std::sin(ang));
}

// Per-pass twiddle tables of gw_fft.cuh's plan for length M: for every pass
// with stride Ns > 1 and radix R, tw[k*(R-1) + r-1] = exp(-2 pi i r k/(Ns R)).
// Odd-radix passes store their table r-major: tw[(r-1)*Ns + k].
std::vector<float2> fft_twiddles(int M) {
  int F = M;
  while (!(F & 1)) F >>= 1;
  const int P2 = M / F;
  int l2 = 0;
  while ((1 << l2) < P2) ++l2;
  const int n16 = l2 / 4, r2 = 1 << (l2 - 4 * n16);
  std::vector<float2> tw;
  auto w = [](long long e, long long span) {
    const double ang = -2.0 * M_PI * (double)(e % span) / (double)span;
    return make_float2((float)std::cos(ang), (float)std::sin(ang));
  };
  auto add = [&](int ns, int R) {
    const long long span = (long long)ns * R;
    if (R & 1) {
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < ns; ++k) tw.push_back(w((long long)r * k, span));
    } else {
      for (int k = 0; k < ns; ++k)
        for (int r = 1; r < R; ++r) tw.push_back(w((long long)r * k, span));
    }
  };
  int ns = 16;
  for (int p = 1; p < n16; ++p) { add(ns, 16); ns *= 16; }
  if (r2 > 1) { add(ns, r2); ns *= r2; }
  if (F > 1) add(ns, F);
  if (tw.empty()) tw.push_back(make_float2(1.f, 0.f));
  return tw;
}

}  // namespace

namespace gwv {

CztTables make_czt(int g, int lo, int L, int k0, int N, int M) {
  CztTables t;
  t.A.resize(L); t.B.resize(N); t.H.resize(M);
  for (int n = 0; n < L; ++n) {
    const cd w = chirp(2LL * n * k0 + 1LL * n * n, g);  // W^{n k0 + n^2/2}
    t.A[n] = make_float2((float)w.real(), (float)w.imag());
  }
  for (int m = 0; m < N; ++m) {  // W^{lo (k0+m) + m^2/2}
    const cd w = chirp(2LL * lo * (k0 + m) + 1LL * m * m, g);
    t.B[m] = make_float2((float)w.real(), (float)w.imag());
  }
  std::vector<cd> h(M, cd(0, 0));
  for (int j = -(L - 1); j <= N - 1; ++j) {  // W^{-j^2/2}
    const cd w = chirp(-1LL * j * j, g);
    h[(j % M + M) % M] = w;
  }
  fft_inplace_host(h);
  for (int i = 0; i < M; ++i) {
    const cd v = h[i] / (double)M;
    t.H[i] = make_float2((float)v.real(), (float)v.imag());
  }
  t.tw = fft_twiddles(M);
  return t;
}

int next_fft_size(int n, bool pow2_only) {
  for (int m : kFftSizes)
    if (m >= n && m >= kMinM && (!pow2_only || (m & (m - 1)) == 0)) return m;
  return 0;
}

bool fft_size_supported(int m) {
  for (int s : kFftSizes)
    if (s == m) return true;
  return false;
}

int batch_rows(gw_voxel_plan *P, int s0, int n) {
  if (P->roff_host.empty()) return n * P->Lz;
  return P->roff_host[s0 + n] - P->roff_host[s0];
}

SliceArgs slice_args(gw_voxel_plan *P) {
  SliceArgs a{};
  a.g = P->g; a.r = P->r; a.inv_r = P->inv_r; a.n_phi = P->n_phi;
  a.y_lo = P->y_lo; a.Ly = P->Ly; a.z_lo = P->z_lo; a.Lz = P->Lz;
  a.fill = P->p.fill_bkg != 0; a.smooth_on = P->p.smooth != 0.0;
  a.sigma = (float)P->p.smooth; a.radius = P->radius; a.plain = P->plain;
  a.xyz = P->d_xyz; a.f = P->d_f; a.zidx = P->d_zidx; a.st = P->d_structs;
  a.xyz_s = P->d_xyz_s; a.xyf_s = P->d_xyf_s; a.rowstart = P->d_rowstart;
  a.fz_s = P->d_fz_s; a.bil = P->bil;
  a.ybnd = P->d_ybnd;
  a.roff = P->d_roff;
  a.zstat = P->d_zstat; a.ymax_ord = P->d_ymax; a.extflag = P->d_extflag;
  a.ph = P->d_phis; a.clbase = P->d_clbase; a.ymin_ord = P->d_ymin;
  a.ext = P->d_ext; a.amo = P->d_amo; a.my = P->d_my; a.pr = P->d_pr;
  a.mz = P->d_mz; a.gw = P->d_gw; a.sconst = P->d_sconst; a.err = P->ctx->d_err;
  return a;
}

int atom_blocks(gw_voxel_plan *P) {
  int64_t max_atoms = 0;
  for (auto &s : P->structs) max_atoms = std::max(max_atoms, s.atom_count);
  return (int)std::min<int64_t>(std::max<int64_t>(1, (max_atoms + 255) / 256),
                                4 * P->ctx->sm_count);
}

int enqueue_prep(gw_voxel_plan *P) {
  gw_ctx *ctx = P->ctx;
  cudaStream_t st = ctx->stream;
  k_ext_init<<<(P->n_slices + 255) / 256, 256, 0, st>>>(P->d_ext, P->n_slices);
  GW_LAUNCHED(ctx);
  GW_CUDA(cudaMemsetAsync(P->d_zmin, 0xff, P->n_struct * sizeof(unsigned long long), st));
  GW_CUDA(cudaMemsetAsync(P->d_ymin, 0xff, P->n_slices * sizeof(unsigned long long), st));
  GW_CUDA(cudaMemsetAsync(P->d_ymax, 0, P->n_slices * sizeof(unsigned long long), st));
  GW_CUDA(cudaMemsetAsync(P->d_zhist, 0, (size_t)P->n_struct * (P->g + 1) * sizeof(int), st));
  const int nblk_at = atom_blocks(P);
  {
    gw::KTimer tm(ctx, GW_K_PREP);
    k_zmin<<<dim3(nblk_at, P->n_struct), 256, 0, st>>>(P->d_xyz, P->d_structs, P->d_zmin);
    GW_LAUNCHED(ctx);
  }
  {
    gw::KTimer tm(ctx, GW_K_PREP);
    k_zidx_hist<<<dim3(nblk_at, P->n_struct), 256, 0, st>>>(
        P->d_xyz, P->d_structs, P->d_zmin, P->r, P->inv_r, P->g, P->d_zidx,
        P->d_zhist);
    GW_LAUNCHED(ctx);
  }
  {
    gw::KTimer tm(ctx, GW_K_PREP);
    k_zscan<<<P->n_struct, 1024, 0, st>>>(P->d_structs, P->g, P->d_zhist,
                                          P->d_rowstart, P->d_cursor, P->d_zstat);
    GW_LAUNCHED(ctx);
  }
  {
    gw::KTimer tm(ctx, GW_K_PREP);
    k_zscatter<<<dim3(nblk_at, P->n_struct), 256, 0, st>>>(
        P->d_xyz, P->d_f, P->d_structs, P->d_zidx, P->g, P->d_zmin, P->inv_r,
        P->d_cursor, P->d_xyz_s, P->d_xyf_s, P->d_perm, P->d_fz_s);
    GW_LAUNCHED(ctx);
  }
  return GW_OK;
}

// Slice arguments whose fill/smoothing profile arrays start at slice s0
// (the setup kernels and the row stage index them by batch slot).
SliceArgs profile_view(const SliceArgs &a, int s0) {
  SliceArgs v = a;
  v.amo = a.amo + (size_t)s0 * a.Ly;
  if (a.pr) v.pr = a.pr + (size_t)s0 * a.Ly;
  v.my = a.my + (size_t)s0 * a.Ly;
  v.mz = a.mz + (size_t)s0 * a.Lz;
  return v;
}

int enqueue_slice_setup(gw_voxel_plan *P, const SliceArgs &a, int s0, int n) {
  gw_ctx *ctx = P->ctx;
  cudaStream_t st = ctx->stream;
  const int nblk_at = atom_blocks(P);
  {
    gw::KTimer tm(ctx, GW_K_DEPOSIT);
    // bounds of slice s live at ybnd[2s], ybnd[2s+1]: reset this range
    k_yreset<<<(n + 255) / 256, 256, 0, st>>>(P->d_ybnd, s0, n);
    GW_LAUNCHED(ctx);
    // a few blocks per slice (grid-stride over the atoms), one atomic per
    // block: the slice's two words are the only targets
    const int nblk_y = std::min(nblk_at, 16);
    const int ngrp = (n + kYS - 1) / kYS;
    k_ybound<<<dim3(nblk_y, ngrp), 256, 0, st>>>(a, s0, n);
    GW_LAUNCHED(ctx);
    k_yminmax<<<dim3(nblk_y, ngrp), 256, 0, st>>>(a, s0, n);
    GW_LAUNCHED(ctx);
  }
  {
    gw::KTimer tm(ctx, GW_K_DEPOSIT);
    k_ext<<<(n + 127) / 128, 128, 0, st>>>(a, s0, n);
    GW_LAUNCHED(ctx);
  }
  {
    gw::KTimer tm(ctx, GW_K_DEPOSIT);
    // rarely needed (a slice with atoms outside the grid): a small grid
    // that exits at once otherwise
    k_ext_exact<<<dim3(std::min(nblk_at, 16), n), 256, 0, st>>>(a, s0);
    GW_LAUNCHED(ctx);
  }
  if (a.fill || a.smooth_on) {
    gw::KTimer tm(ctx, GW_K_PROFILE);
    // several blocks per slice when the slices alone would not fill the GPU
    const int parts = std::max(1, std::min(8, (2 * ctx->sm_count + n - 1) / n));
    k_profile<<<dim3(n, parts), 256, 0, st>>>(a, s0);
    GW_LAUNCHED(ctx);
  }
  return GW_OK;
}

// Slices per launch of the setup kernels (their grids index slices in y).
constexpr int kSetupChunk = 32768;

// Average, crop and f0 factor of every I(q) grid the plan produces: the
// float32 grid the detector reads (f64 false; part of every execute) or the
// float64 grid (f64 true; made when a caller asks for float64 I(q)).
// Whether this execute bins by gather (multi-q shells bin atomically).
bool gathering(const gw_voxel_plan *P) { return P->gather && P->n_shells == 0; }

// k_gather over the structures of output t (all of them when averaged):
// mode 0 / 1 into the float32 / float64 I(q) of output t, mode 2 into sum
// grid t (window).
// Output lines [line_lo, line_hi) of the crop (line = iy Q + ix; -1: all):
// the light lines in that range and the heavy lines among them (a run of the
// ascending heavy list), then the C1 > 1 voxels of the same lines.
int enqueue_gather(gw_voxel_plan *P, int mode, int t, int line_lo, int line_hi) {
  gw_ctx *ctx = P->ctx;
  const bool sep = P->p.average == GW_STRUCTS_SEPARATE;
  const int t0 = sep ? t : 0, t1 = sep ? t + 1 : P->n_struct;
  const bool sums = mode == 2;
  const bool use_f0 = !sums && P->p.f0_z > 0;
  const int Q = sums ? P->W : P->Qc, off = sums ? 0 : P->lo - P->wlo;
  const float f0c = (float)P->p.f0_coef[8];
  const float f0iz = P->p.f0_z > 0 ? (float)(1.0 / P->p.f0_z) : 1.f;
  const float inv_ns = P->p.average == GW_STRUCTS_AVERAGE ? 1.0f / (float)P->n_struct : 1.0f;
  // heavy lines take a block each when the block's partial sums fit
  const bool heavy = P->n_heavy > 0 && gather_smem(Q, use_f0, true) <= (200u << 10);
  if (line_hi < 0) line_hi = Q * Q;
  if (line_lo >= line_hi) return GW_OK;
  int h0 = 0, n_heavy = 0;
  if (heavy) {
    // window line of crop line L; heavy lines outside the crop, listed
    // between two crop lines, are skipped by the kernel
    auto wline = [&](int L) {
      return L >= Q * Q ? P->W * P->W : (L / Q + off) * P->W + L % Q + off;
    };
    const auto b = P->h_heavy.begin(), e = P->h_heavy.end();
    h0 = (int)(std::lower_bound(b, e, wline(line_lo)) - b);
    n_heavy = (int)(std::lower_bound(b, e, wline(line_hi)) - b) - h0;
  }
  const size_t smem = gather_smem(Q, use_f0, heavy);
  // above the default 48 KB: the launch's own kernel (mode, span length)
  static gw::SmemRecord attr[3][2];
  const bool u7 = Q <= 7 * 32;
  if (smem > (48u << 10)) {
    auto &r = attr[mode][u7];
    if (mode == 0) GW_TRY(u7 ? gw::smem_limit(r, k_gather<0, 7>, smem)
                             : gw::smem_limit(r, k_gather<0, 13>, smem));
    else if (mode == 1) GW_TRY(u7 ? gw::smem_limit(r, k_gather<1, 7>, smem)
                                  : gw::smem_limit(r, k_gather<1, 13>, smem));
    else GW_TRY(u7 ? gw::smem_limit(r, k_gather<2, 7>, smem)
                   : gw::smem_limit(r, k_gather<2, 13>, smem));
  }
  const int n_lines = line_hi - line_lo;
  const int blocks = n_heavy + std::max(1, std::min((n_lines + 7) / 8, 16 * ctx->sm_count));
  float *o32 = mode == 0 ? P->d_iq32 + t * P->iq_stride : nullptr;
  double *o64 = mode == 1 ? P->d_iq64 + t * P->iq_stride
              : mode == 2 ? P->d_sum + t * P->sum_stride : nullptr;
  gw::KTimer tm(ctx, GW_K_FINALIZE);
#define GW_GATHER_ARGS                                                             \
  P->d_G, P->d_lptr, P->d_lent, P->d_zptr, P->d_zrows, P->d_heavy + h0, n_heavy,    \
      (int)heavy, line_lo, line_hi, P->Nf, P->Nr, P->r_zero, P->n_phi, t0, t1,       \
      P->d_C2, P->d_C1, P->W, off, Q, inv_ns, P->d_f0, P->d_zf0, use_f0, f0c, f0iz, \
      o64, o32
  // spans covering a whole line: 7 voxels a lane up to 224 a line, else 13
  if (mode == 0) {
    if (u7) k_gather<0, 7><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
    else k_gather<0, 13><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
  } else if (mode == 1) {
    if (u7) k_gather<1, 7><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
    else k_gather<1, 13><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
  } else {
    if (u7) k_gather<2, 7><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
    else k_gather<2, 13><<<blocks, 256, smem, ctx->stream>>>(GW_GATHER_ARGS);
  }
#undef GW_GATHER_ARGS
  GW_LAUNCHED(ctx);
  if (P->n_zmulti > 0) {
    const int mb = std::max(1, std::min((n_lines + 7) / 8, 4 * ctx->sm_count));
#define GW_GATHER_MULTI_ARGS                                                         \
  P->d_G, P->d_lptr, P->d_lent, P->d_zptr, P->d_zrows, P->d_zmulti, P->n_zmulti,     \
      line_lo, line_hi, P->Nf, P->Nr, P->r_zero, P->n_phi, t0, t1, P->d_C2, P->d_C1, \
      P->W, off, Q, inv_ns, P->d_f0, P->d_zf0, use_f0, f0c, f0iz, o64, o32
    if (mode == 0) k_gather_multi<0><<<mb, 256, 0, ctx->stream>>>(GW_GATHER_MULTI_ARGS);
    else if (mode == 1) k_gather_multi<1><<<mb, 256, 0, ctx->stream>>>(GW_GATHER_MULTI_ARGS);
    else k_gather_multi<2><<<mb, 256, 0, ctx->stream>>>(GW_GATHER_MULTI_ARGS);
#undef GW_GATHER_MULTI_ARGS
    GW_LAUNCHED(ctx);
  }
  return GW_OK;
}

int enqueue_finalize(gw_voxel_plan *P, bool f64) {
  gw_ctx *ctx = P->ctx;
  cudaStream_t st = ctx->stream;
  if (gathering(P)) {
    for (int t = 0; t < P->n_out; ++t) GW_TRY(enqueue_gather(P, f64 ? 1 : 0, t));
    return GW_OK;
  }
  const int K = P->n_shells;
  const float f0c = (float)P->p.f0_coef[8];
  const float f0iz = P->p.f0_z > 0 ? (float)(1.0 / P->p.f0_z) : 1.f;
  const float inv_ns = P->p.average == GW_STRUCTS_AVERAGE ? 1.0f / (float)P->n_struct : 1.0f;
  const int kahan = P->p.accum == GW_ACCUM_KAHAN32;
  const size_t Qc3 = (size_t)P->Qc * P->Qc * P->Qc;
  for (int t = 0; t < P->n_out; ++t) {  // one I(q) per structure when separate
    double *sum = P->d_sum ? P->d_sum + t * P->sum_stride : nullptr;
    float2 *sumk = P->d_sumk ? P->d_sumk + t * P->sum_stride : nullptr;
    double *o64 = f64 ? P->d_iq64 + t * P->iq_stride : nullptr;
    float *o32 = f64 ? nullptr : P->d_iq32 + t * P->iq_stride;
    {
      gw::KTimer tm(ctx, GW_K_FINALIZE);
      const bool use_f0 = P->p.f0_z > 0;
      const size_t smem = finalize_smem(P->Qc, use_f0);
      // above the default 48 KB (crops beyond about 2400 voxels a side)
      static gw::SmemRecord attr64, attr32;
      if (smem > (48u << 10)) {
        if (f64) GW_TRY(gw::smem_limit(attr64, k_finalize<true>, smem));
        else GW_TRY(gw::smem_limit(attr32, k_finalize<false>, smem));
      }
      const int blocks = std::min((P->Qc * P->Qc + 7) / 8, 16 * ctx->sm_count);
      if (f64)
        k_finalize<true><<<blocks, 256, smem, st>>>(
            sum, sumk, kahan, P->d_C2, P->d_C1, P->W, P->lo - P->wlo, P->Qc,
            inv_ns, P->d_f0, P->d_zf0, use_f0, f0c, f0iz, o64, o32);
      else
        k_finalize<false><<<blocks, 256, smem, st>>>(
            sum, sumk, kahan, P->d_C2, P->d_C1, P->W, P->lo - P->wlo, P->Qc,
            inv_ns, P->d_f0, P->d_zf0, use_f0, f0c, f0iz, o64, o32);
      GW_LAUNCHED(ctx);
    }
    if (K > 0 && P->shell_mode == GW_SHELLS_REFERENCE) {
      gw::KTimer tm(ctx, GW_K_FINALIZE);
      const int blocks = (int)std::min<int64_t>(((int64_t)Qc3 + 255) / 256, 16 * ctx->sm_count);
      k_shell_double<<<blocks, 256, 0, st>>>(P->d_shell, P->W, P->lo - P->wlo,
                                             P->Qc, K - 1, o64, o32);
      GW_LAUNCHED(ctx);
    }
  }
  return GW_OK;
}

// Enqueue the whole chain (no synchronisation).
int enqueue(gw_voxel_plan *P) {
  gw_ctx *ctx = P->ctx;
  cudaStream_t st = ctx->stream;
  // gather binning stores every pixel and sums afterwards: no sum grid to
  // clear
  if (P->p.accum == GW_ACCUM_KAHAN32)
    GW_CUDA(cudaMemsetAsync(P->d_sumk, 0, P->sum_stride * P->n_out * sizeof(float2), st));
  else if (!gathering(P))
    GW_CUDA(cudaMemsetAsync(P->d_sum, 0, P->sum_stride * P->n_out * sizeof(double), st));
  SliceArgs a = slice_args(P);
  CztArgs cy{P->My, P->Ly, P->Nc, P->d_Ay, P->d_Hy, P->d_By, P->d_twy};
  CztArgs cz{P->Mz, P->Lz, P->Nr, P->d_Az, P->d_Hz, P->d_Bz, P->d_twz};
  BinArgs bn{P->d_colofs, P->d_rowofs, P->d_sum, P->d_sumk,
             P->p.accum == GW_ACCUM_KAHAN32, P->k0, P->kz0,
             (float)((double)P->g * (double)P->g),
             P->n_out > 1 ? (int64_t)P->sum_stride : 0, nullptr, 0,
             P->wait_polls, P->real ? 1 : 0, P->m_zero, P->r_zero,
             gathering(P) ? P->d_G : nullptr};
  // Multi-q form factors: one pass per shell with that shell's atom f
  // values and average voxel f, binning only the shell's voxels into the
  // common sums (GW_SHELLS_PER_SHELL); or the reference's single pass with
  // the last shell's values (GW_SHELLS_REFERENCE).
  const int K = P->n_shells;
  const int k_first = K > 0 && P->shell_mode == GW_SHELLS_PER_SHELL ? 0 : K - 1;
  for (int k = std::max(k_first, 0); k < std::max(K, 1); ++k) {
    if (K > 0) {
      GW_CUDA(cudaMemcpyAsync(P->d_f, P->d_f_shells + (size_t)k * P->n_atoms,
                              (size_t)P->n_atoms * sizeof(float2),
                              cudaMemcpyDeviceToDevice, st));
      GW_CUDA(cudaMemcpyAsync(P->d_structs, P->d_structs_shells + (size_t)k * P->n_struct,
                              (size_t)P->n_struct * sizeof(gw_structure),
                              cudaMemcpyDeviceToDevice, st));
      bn.shell = P->shell_mode == GW_SHELLS_PER_SHELL ? P->d_shell : nullptr;
      bn.shell_k = k;
    }
    {
      gw::Range r("giwaxsim: voxel prep (z sort)");
      GW_TRY(enqueue_prep(P));
    }
    // Batched: the per-slice setup of every slice at once (fuller grids,
    // fewer launches); the profile arrays hold every slice and each batch
    // sees its part.  Plain mode keeps the reference's per-rotation order.
    if (!P->plain)
      for (int c0 = 0; c0 < P->n_slices; c0 += kSetupChunk)
        GW_TRY(enqueue_slice_setup(P, profile_view(a, c0), c0,
                                   std::min(kSetupChunk, P->n_slices - c0)));
    for (int s0 = 0; s0 < P->n_slices; s0 += P->S) {
      const int n = std::min(P->S, P->n_slices - s0);
      const SliceArgs ab = profile_view(a, s0);
      if (P->plain) GW_TRY(enqueue_slice_setup(P, ab, s0, n));
      {
        gw::Range r("giwaxsim: voxel rows (deposit + y chirp-z)");
        GW_TRY(row_dispatch(P, ab, cy, s0, n));
      }
      {
        gw::Range r("giwaxsim: voxel columns (z chirp-z + binning)");
        GW_TRY(col_dispatch(P, ab, cz, bn, s0, n));
      }
    }
  }
  gw::Range r("giwaxsim: voxel finalize");
  return enqueue_finalize(P, false);
}

}  // namespace


extern "C" int gw_voxel_plan_create(gw_ctx *ctx, const gw_voxel_params *p,
                                    const gw_structure *structs,
                                    int32_t n_struct, const gw_phi *phis,
                                    int32_t n_phi, gw_voxel_plan **out) {
  if (!ctx || !p || !structs || !phis || !out)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: null argument");
  if (n_struct < 1 || n_phi < 1)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: need >= 1 structure and >= 1 phi");
  if (p->grid_size < 2 || p->r_voxel_size <= 0 || p->dq <= 0 || p->q_num < 3 ||
      p->crop_lo < 0 || p->crop_hi >= p->q_num || p->crop_lo > p->crop_hi)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: invalid geometry");
  if (p->smooth < 0)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: smooth must be >= 0");
  // real grids take each structure's phase from its average voxel f
  if (p->real_grids)
    for (int t = 0; t < n_struct; ++t) {
      const double re = structs[t].avg_f_re, im = structs[t].avg_f_im;
      if (!std::isfinite(re) || !std::isfinite(im) || (re == 0.0 && im == 0.0))
        return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: real_grids needs a finite, "
                                    "nonzero average voxel f for every structure");
    }
  if (p->binning < GW_BINNING_AUTO || p->binning > GW_BINNING_GATHER)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: binning must be GW_BINNING_AUTO, "
                                "_ATOMIC or _GATHER");
  if (p->block_variant < 0 || p->block_variant >= gwv::fused_variant_count())
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: block_variant must be 0.." +
                                    std::to_string(gwv::fused_variant_count() - 1));
  if (p->deposit != GW_DEPOSIT_NEAREST && p->deposit != GW_DEPOSIT_BILINEAR)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: unknown deposit mode");
  if (p->deposit == GW_DEPOSIT_BILINEAR && p->mode == GW_VOXEL_PLAIN)
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: the bilinear deposit needs the batched mode");
  GW_CUDA(cudaSetDevice(ctx->device));
  auto *P = new gw_voxel_plan();
  P->ctx = ctx;
  P->p = *p;
  P->n_struct = n_struct;
  P->n_phi = n_phi;
  P->n_slices = n_struct * n_phi;
  P->structs.assign(structs, structs + n_struct);
  P->phis.assign(phis, phis + n_phi);
  P->g = p->grid_size;
  P->plain = p->mode == GW_VOXEL_PLAIN;
  P->bil = p->deposit == GW_DEPOSIT_BILINEAR;
  P->n_out = p->average == GW_STRUCTS_SEPARATE ? n_struct : 1;
  P->r = p->r_voxel_size;
  P->inv_r = 1.0 / P->r;
  P->dq = p->dq;
  P->inv_dq = 1.0 / P->dq;
  P->lo = p->crop_lo;
  P->hi = p->crop_hi;
  P->Qc = P->hi - P->lo + 1;
  if (P->plain) { P->wlo = 0; P->whi = p->q_num - 1; }
  else { P->wlo = P->lo; P->whi = P->hi; }
  P->W = P->whi - P->wlo + 1;
  const int g = P->g;
  const double sigma = p->smooth;
  P->radius = sigma > 0 ? (int)(4.0 * sigma + 0.5) : 0;

  // row table (phi independent): fftshift(fftfreq(g, r)) * 2pi
  std::vector<int> rowofs_all(g, -1);
  P->C1host.assign(P->W, 0);
  {
    const double val = 1.0 / ((double)g * P->r);
    for (int i = 0; i < g; ++i) {
      const long long k = (long long)i - g / 2;
      const double q = (((double)k * val) * 2.0) * M_PI;
      if (q <= p->q_max && q >= p->q_min) {
        const int iz = (int)floor_div_exact(q - p->q_min, P->dq, P->inv_dq);
        if (iz >= P->wlo && iz <= P->whi) rowofs_all[i] = iz - P->wlo;
      }
    }
  }
  int r0 = -1, r1 = -1;
  if (P->plain) {
    r0 = 0; r1 = g - 1;
  } else {
    for (int i = 0; i < g; ++i)
      if (rowofs_all[i] >= 0) { if (r0 < 0) r0 = i; r1 = i; }
    if (r0 < 0) { delete P; return gw::fail(GW_ERR_ARG, "no slice row lands in the cropped cube"); }
  }
  // real grids: bands symmetric around q = 0 (kz from -Kz to Kz), so that
  // every output row has its mirror
  const bool want_real = p->real_grids != 0 && !P->plain && !P->bil;
  if (want_real) {
    const int Kz = std::max(g / 2 - r0, r1 - g / 2);
    if (g / 2 - Kz < 0 || g / 2 + Kz > g - 1) {
      delete P;
      return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: real-grid band wider than the grid");
    }
    r0 = g / 2 - Kz;
    r1 = g / 2 + Kz;
    P->r_zero = Kz;
  }
  P->kz0 = r0 - g / 2;
  P->Nr = r1 - r0 + 1;
  std::vector<int> rowofs(P->Nr);
  for (int i = 0; i < P->Nr; ++i) {
    rowofs[i] = rowofs_all[r0 + i];
    if (rowofs[i] >= 0) P->C1host[rowofs[i]]++;
  }
  // column band
  if (P->plain) {
    P->k0 = -(g / 2);
    P->Nc = g;
  } else {
    // |q| reached by the binned window, then the widest column band over
    // phi (45 degrees), plus a margin; exact per-column validity comes from
    // k_col_tables.
    const double qa = std::max(std::fabs(p->q_min + P->lo * P->dq),
                               std::fabs(p->q_min + (P->hi + 1) * P->dq));
    const double hcap = (qa + 2 * P->dq) * std::sqrt(2.0);
    const double dh = 2.0 * p->h_max / (g - 1);
    const int K = (int)std::ceil(hcap / dh) + 2;
    int c_lo = std::max(0, (g - 1) / 2 - K);
    int c_hi = std::min(g - 1, g / 2 + K);
    if (want_real) {
      // symmetric: ky from -K to K, m_zero = K; F1 keeps the columns
      // ky >= 0, an even number of them (one past K if needed: beyond the
      // margin of K, so unbinned)
      c_lo = g / 2 - K;
      c_hi = g / 2 + K;
      if (c_lo < 0 || c_hi > g - 1) {
        delete P;
        return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: real-grid band wider than the grid");
      }
      P->m_zero = K;
      if ((K + 1) % 2) ++c_hi;
    } else if ((c_hi - c_lo + 1) % 2) {
      // an even band keeps F1's rows 16-byte aligned for tensor-map loads;
      // a column past the grid (c_hi = g) is marked unbinned by
      // k_col_tables
      ++c_hi;
    }
    P->k0 = c_lo - g / 2;
    P->Nc = c_hi - c_lo + 1;
  }
  // real-space windows
  if (P->plain) {
    P->y_lo = 0; P->Ly = g; P->z_lo = 0; P->Lz = g;
  } else {
    int ybound = 0, zbound = 0;
    for (int t = 0; t < n_struct; ++t) {
      const gw_structure &s = structs[t];
      zbound = std::max(zbound, (int)std::floor(s.z_bound * P->inv_r + 1e-6) + 1);
      for (int q = 0; q < n_phi; ++q) {
        const double ext = s.x_bound * std::fabs(phis[q].sin_phi) +
                           s.y_bound * std::fabs(phis[q].cos_phi);
        ybound = std::max(ybound, (int)std::floor(ext * P->inv_r + 1e-6) + 1);
      }
    }
    const int tail = P->radius;
    const int lo_off = sigma > 0 ? std::min(0, (int)std::ceil(sigma) - P->radius) : 0;
    P->y_lo = lo_off;
    P->Ly = ybound + tail - lo_off + 1;
    if (P->Ly >= g) { P->Ly = g; P->y_lo = 0; }
    P->z_lo = lo_off;
    P->Lz = zbound + tail - lo_off + 1;
    if (P->Lz >= g) { P->Lz = g; P->z_lo = 0; }
    // structures of uneven height: each keeps the rows of its own z window
    // (same origin z_lo; the window never wraps the grid when Lz < g)
    if (P->Lz < g && n_struct > 1) {
      std::vector<int> lz(n_struct);
      bool uneven = false;
      for (int t = 0; t < n_struct; ++t) {
        const int zb = (int)std::floor(structs[t].z_bound * P->inv_r + 1e-6) + 1;
        lz[t] = std::min(P->Lz, zb + tail - lo_off + 1);
        uneven = uneven || lz[t] != P->Lz;
      }
      if (uneven) {
        P->roff_host.assign((size_t)P->n_slices + 1, 0);
        for (int sl = 0; sl < P->n_slices; ++sl)
          P->roff_host[sl + 1] = P->roff_host[sl] + lz[sl / n_phi];
      }
    }
  }
  // transform lengths: the smallest supported >= L+N-1, or the caller's
  // choice (an autotuner compares the candidates)
  const int need_y = P->Ly + P->Nc - 1, need_z = P->Lz + P->Nr - 1;
  P->My = p->fft_y > 0 ? p->fft_y : next_fft_size(need_y, false);
  P->Mz = p->fft_z > 0 ? p->fft_z : next_fft_size(need_z, false);
  if (P->My == 0 || P->Mz == 0) {
    delete P;
    return gw::fail(GW_ERR_ARG, "slice transform larger than 8192 points");
  }
  if (!fft_size_supported(P->My) || !fft_size_supported(P->Mz) ||
      P->My < need_y || P->Mz < need_z) {
    delete P;
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: fft_y/fft_z must be a supported length >= L+N-1");
  }
  // real grids: two window rows share one row transform buffer (a window
  // of at most half the buffer) and the Stockham kernels run both axes (a
  // fused kernel asked for by name keeps the general path)
  P->real = want_real && 2 * P->Ly <= fft_ldm(P->My) && P->My <= 2048 &&
            p->transform_y != GW_TRANSFORM_FUSED && p->transform_z != GW_TRANSFORM_FUSED;
  P->Nf = P->real ? P->Nc - P->m_zero : P->Nc;
  // batch size: keep the per-batch intermediates near L2 size
  {
    const size_t per = (size_t)P->Lz * P->Nf * sizeof(float2) +
                       (P->Ly + P->Lz) * 12;
    int S = p->batch_slices > 0 ? p->batch_slices
                                : (int)std::max<size_t>(1, (96u << 20) / per);
    if (P->plain) S = 1;
    P->S = std::min(std::min(S, P->n_slices), 4096);  // grid.y limit margin
  }

  int st = GW_OK;
  size_t &B = P->bytes;
  // per-slice collapse base (pow on the host, as numpy's scalar ** does)
  std::vector<double> clbase(P->n_slices, 0.0);
  if (p->fill_bkg) {
    std::vector<double> ver(P->n_slices), cost(P->n_slices);
    for (int t = 0; t < n_struct; ++t)
      for (int q = 0; q < n_phi; ++q) {
        const gw_phi &ph = phis[q];
        ver[(size_t)t * n_phi + q] = ph.cl_swap ? structs[t].y_bound : structs[t].x_bound;
        cost[(size_t)t * n_phi + q] = ph.cos_t;
      }
    GW_TRY(gw_collapse_base(ver.data(), cost.data(), P->n_slices, clbase.data()));
  }
  // Gaussian weights (scipy.ndimage._gaussian_kernel1d, order 0)
  std::vector<float> gwv;
  if (sigma > 0) {
    std::vector<double> w(2 * P->radius + 1);
    double sum = 0;
    for (int j = -P->radius; j <= P->radius; ++j) {
      w[j + P->radius] = std::exp(-0.5 / (sigma * sigma) * (double)j * j);
      sum += w[j + P->radius];
    }
    for (double v : w) gwv.push_back((float)(v / sum));
  }
  // f0 tables (separable exp factors) on the cropped axis
  std::vector<float> f0tab;
  if (p->f0_z > 0) {
    f0tab.resize(4 * 3 * P->Qc);
    const double s16 = 16.0 * M_PI * M_PI;
    for (int i = 0; i < 4; ++i)
      for (int ax = 0; ax < 3; ++ax)
        for (int k = 0; k < P->Qc; ++k) {
          const double q = linspace_at(p->q_min, p->q_max, p->q_num, P->lo + k);
          double e = std::exp(-p->f0_coef[2 * i + 1] * q * q / s16);
          if (ax == 0) e *= p->f0_coef[2 * i];  // a_i folded into the x factor
          f0tab[(i * 3 + ax) * P->Qc + k] = (float)e;
        }
  }
  // the z factors of the four terms, packed per qz
  std::vector<float4> zf0;
  if (p->f0_z > 0)
    for (int k = 0; k < P->Qc; ++k)
      zf0.push_back(make_float4(f0tab[2 * P->Qc + k], f0tab[5 * P->Qc + k],
                                f0tab[8 * P->Qc + k], f0tab[11 * P->Qc + k]));
  CztTables ty = make_czt(g, P->y_lo, P->Ly, P->k0, P->Nc, P->My);
  CztTables tz = make_czt(g, P->z_lo, P->Lz, P->kz0, P->Nr, P->Mz);
  // fused chirp-z kernels where the caller asks for them (and the length
  // has a fused shape); the Stockham kernels otherwise (measured faster on
  // GB300 for every length with a fused shape; an autotuner may still pick
  // the fused ones)
  P->fused_y = !P->real && p->transform_y == GW_TRANSFORM_FUSED && fused_supported(P->My);
  P->fused_z = !P->real && p->transform_z == GW_TRANSFORM_FUSED && fused_supported(P->Mz);
  if ((p->transform_y == GW_TRANSFORM_FUSED && !P->fused_y) ||
      (p->transform_z == GW_TRANSFORM_FUSED && !P->fused_z)) {
    const int m = (p->transform_y == GW_TRANSFORM_FUSED && !P->fused_y) ? P->My : P->Mz;
    delete P;
    return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: no fused transform of length " +
                                    std::to_string(m));
  }
  const std::vector<float2> fty = P->fused_y ? fused_twiddles(P->My) : std::vector<float2>();
  const std::vector<float2> ftz = P->fused_z ? fused_twiddles(P->Mz) : std::vector<float2>();
  const size_t W3 = (size_t)P->W * P->W * P->W;
  const size_t Qc3 = (size_t)P->Qc * P->Qc * P->Qc;
  P->sum_stride = (W3 + 3) & ~(size_t)3;
  P->iq_stride = (Qc3 + 3) & ~(size_t)3;
  if ((st = upload(&P->d_structs, P->structs, &B)) ||
      (st = upload(&P->d_phis, P->phis, &B)) ||
      (st = upload(&P->d_clbase, clbase, &B)) ||
      (st = upload(&P->d_gw, gwv, &B)) || (st = upload(&P->d_f0, f0tab, &B)) ||
      (st = upload(&P->d_zf0, zf0, &B)) ||
      (st = upload(&P->d_rowofs, rowofs, &B)) ||
      (st = upload(&P->d_C1, P->C1host, &B)) ||
      (st = upload(&P->d_Ay, ty.A, &B)) || (st = upload(&P->d_Hy, ty.H, &B)) ||
      (st = upload(&P->d_By, ty.B, &B)) || (st = upload(&P->d_twy, ty.tw, &B)) ||
      (st = upload(&P->d_Az, tz.A, &B)) || (st = upload(&P->d_Hz, tz.H, &B)) ||
      (st = upload(&P->d_Bz, tz.B, &B)) || (st = upload(&P->d_twz, tz.tw, &B)) ||
      (st = upload(&P->d_fty, fty, &B)) || (st = upload(&P->d_ftz, ftz, &B)) ||
      (st = alloc(&P->d_zmin, n_struct, &B)) ||
      (st = alloc(&P->d_ymin, P->n_slices, &B)) ||
      (st = alloc(&P->d_ext, P->n_slices, &B)) ||
      (st = alloc(&P->d_sconst, P->n_slices, &B)) ||
      (st = alloc(&P->d_colofs, (size_t)n_phi * P->Nc, &B)) ||
      (st = alloc(&P->d_C2, (size_t)P->W * P->W, &B)) ||
      (st = (p->accum == GW_ACCUM_KAHAN32
                 ? alloc(&P->d_sumk, P->sum_stride * P->n_out, &B)
                 : alloc(&P->d_sum, P->sum_stride * P->n_out, &B))) ||
      (st = alloc(&P->d_iq64, P->iq_stride * P->n_out, &B)) ||
      (st = alloc(&P->d_iq32, P->iq_stride * P->n_out, &B)) ||
      (st = alloc(&P->d_ymax, P->n_slices, &B)) ||
      (st = alloc(&P->d_ybnd, 2 * (size_t)P->n_slices, &B)) ||
      (st = alloc(&P->d_extflag, P->n_slices, &B)) ||
      (st = alloc(&P->d_zhist, (size_t)n_struct * (g + 1), &B)) ||
      (st = alloc(&P->d_rowstart, (size_t)n_struct * (g + 2), &B)) ||
      (st = alloc(&P->d_cursor, (size_t)n_struct * (g + 1), &B)) ||
      (st = alloc(&P->d_zstat, n_struct, &B)) ||
      (st = alloc(&P->d_F1, (size_t)P->S * P->Lz * P->Nf, &B)) ||
      (st = alloc(&P->d_amo, (size_t)P->n_slices * P->Ly, &B)) ||
      (P->real && (st = alloc(&P->d_pr, (size_t)P->n_slices * P->Ly, &B))) ||
      (st = alloc(&P->d_my, (size_t)P->n_slices * P->Ly, &B)) ||
      (st = alloc(&P->d_mz, (size_t)P->n_slices * P->Lz, &B)) ||
      (st = upload(&P->d_roff, P->roff_host, &B)) ||
      (st = col_map_dispatch(P))) {
    gw_voxel_plan_destroy(P);
    return st;
  }
  // column bin tables and the (qy,qx) count factor: geometry only, made once
  {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMemsetAsync(P->d_C2, 0, (size_t)P->W * P->W * sizeof(unsigned), s);
    if (e == cudaSuccess) {
      k_col_tables<<<P->n_phi, 256, 0, s>>>(P->d_phis, P->g, P->k0, P->Nc,
                                           P->p.q_min, P->p.q_max, P->dq,
                                           P->inv_dq, P->wlo, P->whi, P->W,
                                           P->d_colofs, P->d_C2);
      ctx->launches++;
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      gw_voxel_plan_destroy(P);
      return gw::cuda_fail(e, "column tables", __FILE__, __LINE__);
    }
  }
  // gather binning: where it applies and the pixel store fits the budget
  // (GW_GATHER_MAX_MB, default 8192)
  {
    const size_t g_bytes = (size_t)P->n_slices * P->Nf * P->Nr * sizeof(float);
    const char *env = getenv("GW_GATHER_MAX_MB");
    const size_t cap = (env ? (size_t)std::max(0L, atol(env)) : (size_t)8192) << 20;
    // (and fewer than 2^31 pixels: the gather addresses them with 32 bits)
    const bool can = !P->plain && p->accum == GW_ACCUM_FP64 && !P->fused_z &&
                     g_bytes <= cap && g_bytes / sizeof(float) < ((size_t)1 << 31);
    if (p->binning == GW_BINNING_GATHER && !can) {
      gw_voxel_plan_destroy(P);
      return gw::fail(GW_ERR_ARG, "gw_voxel_plan_create: gather binning needs a batched, "
                                  "float64-accumulating plan without the fused column "
                                  "kernel, and a pixel store within GW_GATHER_MAX_MB");
    }
    // auto: gather for one structure on real grids whose float64 sum grid
    // is larger than L2 -- each atomic is then a DRAM read-modify-write and
    // the grid's clearing a DRAM pass, while each stored pixel serves two
    // voxels (its mirror) -- measured faster there (si-100A) and slower
    // with the grid in L2, several structures (the gather loops over the
    // structures of every entry) or complex grids (lamellar-200A)
    const size_t sum_bytes = P->sum_stride * P->n_out * sizeof(double);
    const bool want = p->binning == GW_BINNING_GATHER ||
                      (p->binning == GW_BINNING_AUTO && P->real && n_struct == 1 &&
                       sum_bytes > ctx->l2_bytes);
    if (want && can) {
      // the line entries, in table order (phi, band column): counting sort
      // by window line
      std::vector<int> cof((size_t)n_phi * P->Nc);
      cudaError_t e = cudaMemcpy(cof.data(), P->d_colofs, cof.size() * sizeof(int),
                                 cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        gw_voxel_plan_destroy(P);
        return gw::cuda_fail(e, "column tables", __FILE__, __LINE__);
      }
      const int W = P->W;
      std::vector<int> lptr((size_t)W * W + 1, 0);
      for (int co : cof)
        if (co >= 0) ++lptr[co / W + 1];
      for (size_t i = 1; i < lptr.size(); ++i) lptr[i] += lptr[i - 1];
      std::vector<int2> lent(std::max(lptr.back(), 1));
      std::vector<int> fill(lptr.begin(), lptr.end() - 1);
      for (int q = 0; q < n_phi; ++q)
        for (int m = 0; m < P->Nc; ++m) {
          const int co = cof[(size_t)q * P->Nc + m];
          if (co < 0) continue;
          // F1 column of table column m: itself, or with real grids its
          // mirror's (rows mirrored) below m_zero
          int j = m, flip = 0;
          if (P->real) {
            if (m >= P->m_zero) j = m - P->m_zero;
            else { j = P->m_zero - m; flip = 1; }
          }
          lent[fill[co / W]++] = make_int2(q, 2 * j + flip);
        }
      // output rows of every window z, ascending
      std::vector<int> zptr((size_t)W + 1, 0);
      for (int ro : rowofs)
        if (ro >= 0) ++zptr[ro + 1];
      for (int i = 1; i <= W; ++i) zptr[i] += zptr[i - 1];
      std::vector<int> zrows(std::max(zptr.back(), 1));
      std::vector<int> zfill(zptr.begin(), zptr.end() - 1);
      for (int mr = 0; mr < P->Nr; ++mr)
        if (rowofs[mr] >= 0) zrows[zfill[rowofs[mr]]++] = mr;
      // window z with more than one output row
      std::vector<int> zmulti;
      for (int z = 0; z < W; ++z)
        if (zptr[z + 1] - zptr[z] > 1) zmulti.push_back(z);
      P->n_zmulti = (int)zmulti.size();
      if (zmulti.empty()) zmulti.push_back(0);
      // lines with more than kGatherHeavy pixels per voxel (entries times
      // the structures each output sums; near the rotation axis)
      const int per_entry = p->average == GW_STRUCTS_SEPARATE ? 1 : n_struct;
      std::vector<int> heavy;
      for (int l = 0; l < W * W; ++l)
        if ((int64_t)(lptr[l + 1] - lptr[l]) * per_entry > kGatherHeavy) heavy.push_back(l);
      P->n_heavy = (int)heavy.size();
      P->h_heavy = heavy;
      if (heavy.empty()) heavy.push_back(0);
      if ((st = upload(&P->d_heavy, heavy, &B)) || (st = upload(&P->d_zmulti, zmulti, &B)) ||
          (st = upload(&P->d_lptr, lptr, &B)) || (st = upload(&P->d_lent, lent, &B)) ||
          (st = upload(&P->d_zptr, zptr, &B)) || (st = upload(&P->d_zrows, zrows, &B)) ||
          (st = alloc(&P->d_G, g_bytes / sizeof(float), &B))) {
        gw_voxel_plan_destroy(P);
        return st;
      }
      P->gather = true;
    }
  }
  *out = P;
  return GW_OK;
}

extern "C" int gw_voxel_plan_destroy(gw_voxel_plan *P) {
  if (!P) return GW_OK;
  if (P->gexec) cudaGraphExecDestroy(P->gexec);
  if (P->graph) cudaGraphDestroy(P->graph);
  gwv::grad_state_destroy(P->grad);
  void *ptrs[] = {P->d_xyz, P->d_f, P->d_zidx, P->d_structs, P->d_phis,
                  P->d_clbase, P->d_zmin, P->d_ymin, P->d_ext, P->d_Ay,
                  P->d_Hy, P->d_By, P->d_twy, P->d_Az, P->d_Hz, P->d_Bz,
                  P->d_twz, P->d_gw, P->d_colofs, P->d_rowofs, P->d_C1,
                  P->d_C2, P->d_sum, P->d_sumk, P->d_f0, P->d_iq64,
                  P->d_iq32, P->d_F1, P->d_amo, P->d_my, P->d_mz,
                  P->d_sconst, P->d_xyz_s, P->d_xyf_s, P->d_fz_s,
                  P->d_perm, P->d_ybnd, P->d_roff, P->d_zhist, P->d_rowstart,
                  P->d_cursor, P->d_zstat, P->d_ymax, P->d_extflag,
                  P->d_shell, P->d_f_shells, P->d_structs_shells, P->d_zf0,
                  P->d_fty, P->d_ftz, P->d_G, P->d_lptr, P->d_lent, P->d_zptr,
                  P->d_zrows, P->d_heavy, P->d_zmulti, P->d_pr};
  for (void *q : ptrs) gw::dev_free(q);
  delete P;
  return GW_OK;
}

extern "C" int gw_voxel_set_atoms(gw_voxel_plan *P, const double *xyz,
                                  const float *f, int64_t n, int32_t on_device) {
  if (!P || !xyz || !f || n < 1)
    return gw::fail(GW_ERR_ARG, "gw_voxel_set_atoms: null argument or no atoms");
  for (auto &s : P->structs)
    if (s.atom_begin < 0 || s.atom_count < 1 || s.atom_begin + s.atom_count > n)
      return gw::fail(GW_ERR_ARG, "gw_voxel_set_atoms: structure atom range outside the atom arrays");
  if (n != P->n_atoms) {
    void *old[] = {P->d_xyz, P->d_f, P->d_zidx, P->d_xyz_s, P->d_xyf_s,
                   P->d_perm, P->d_fz_s};
    for (void *q : old) gw::dev_free(q);
    P->d_xyz = nullptr; P->d_f = nullptr; P->d_zidx = nullptr;
    P->d_xyz_s = nullptr; P->d_xyf_s = nullptr;
    P->d_perm = nullptr; P->d_fz_s = nullptr;
    P->n_atoms = -1;
    if (n > INT_MAX / 4)
      return gw::fail(GW_ERR_ARG, "gw_voxel_set_atoms: more than 2^29 atoms");
    GW_CUDA(gw::dev_malloc((void **)&P->d_xyz, (size_t)n * 3 * sizeof(double)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_f, (size_t)n * sizeof(float2)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_zidx, (size_t)n * sizeof(int)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_xyz_s, (size_t)n * 3 * sizeof(double)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_xyf_s, (size_t)n * sizeof(float4)));
    GW_CUDA(gw::dev_malloc((void **)&P->d_perm, (size_t)n * sizeof(int)));
    if (P->bil)
      GW_CUDA(gw::dev_malloc((void **)&P->d_fz_s, (size_t)n * sizeof(float)));
    P->n_atoms = n;
    if (P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    if (P->graph) { cudaGraphDestroy(P->graph); P->graph = nullptr; }
  }
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  GW_CUDA(cudaMemcpyAsync(P->d_xyz, xyz, (size_t)n * 3 * sizeof(double), kind, P->ctx->stream));
  GW_CUDA(cudaMemcpyAsync(P->d_f, f, (size_t)n * sizeof(float2), kind, P->ctx->stream));
  P->f_stale = false;
  return GW_OK;
}

extern "C" int gw_voxel_set_shells(gw_voxel_plan *P, int32_t n_shells,
                                   int32_t mode, const double *q_axis,
                                   const double *lower, const double *upper,
                                   const float *f, const double *avg_f) {
  if (P && P->real)
    return gw::fail(GW_ERR_STATE, "gw_voxel_set_shells: the plan was made with "
                                  "real_grids (per-shell f values): make it with real_grids 0");
  if (!P) return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: null plan");
  auto drop = [P]() {
    gw::dev_free(P->d_shell); gw::dev_free(P->d_f_shells);
    gw::dev_free(P->d_structs_shells);
    P->d_shell = nullptr; P->d_f_shells = nullptr; P->d_structs_shells = nullptr;
    if (P->n_shells > 0) P->f_stale = true;
    P->n_shells = 0;
    P->shell_atoms = -1;
    if (P->gexec) { cudaGraphExecDestroy(P->gexec); P->gexec = nullptr; }
    if (P->graph) { cudaGraphDestroy(P->graph); P->graph = nullptr; }
  };
  GW_CUDA(cudaSetDevice(P->ctx->device));
  GW_CUDA(cudaStreamSynchronize(P->ctx->stream));  // no pass reads the tables
  if (n_shells == 0) { drop(); return GW_OK; }
  if (n_shells < 0 || n_shells > 32767)
    return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: n_shells outside [0, 32767]");
  if (mode != GW_SHELLS_PER_SHELL && mode != GW_SHELLS_REFERENCE)
    return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: unknown mode");
  if (!q_axis || !lower || !upper || !f || !avg_f)
    return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: null argument");
  if (P->n_atoms < 1)
    return gw::fail(GW_ERR_STATE, "gw_voxel_set_shells: set the atoms first");
  if (P->grad) return gw::fail(GW_ERR_STATE, "gw_voxel_set_shells: plan has gradient state");
  for (int k = 0; k < n_shells; ++k) {
    if (!(lower[k] < upper[k]))
      return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: shell with lower >= upper");
    if (k + 1 < n_shells && !(lower[k + 1] > lower[k] && upper[k + 1] > upper[k]))
      return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: shells must increase");
    if (k + 2 < n_shells && !(lower[k + 2] >= upper[k]))
      return gw::fail(GW_ERR_ARG, "gw_voxel_set_shells: a shell overlaps the one after next");
  }
  drop();
  const int K = n_shells;
  const size_t W3 = (size_t)P->W * P->W * P->W;
  std::vector<gw_structure> st((size_t)K * P->n_struct);
  for (int k = 0; k < K; ++k)
    for (int t = 0; t < P->n_struct; ++t) {
      gw_structure s = P->structs[t];
      s.avg_f_re = avg_f[2 * ((size_t)k * P->n_struct + t)];
      s.avg_f_im = avg_f[2 * ((size_t)k * P->n_struct + t) + 1];
      st[(size_t)k * P->n_struct + t] = s;
    }
  std::vector<double> qw(q_axis + P->wlo, q_axis + P->whi + 1);
  std::vector<double> bounds(lower, lower + K);
  bounds.insert(bounds.end(), upper, upper + K);
  double *d_qw = nullptr, *d_bounds = nullptr;
  cudaStream_t s = P->ctx->stream;
  cudaError_t e = gw::dev_malloc((void **)&P->d_shell, W3 * sizeof(unsigned short));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&P->d_f_shells, (size_t)K * P->n_atoms * sizeof(float2));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&P->d_structs_shells, st.size() * sizeof(gw_structure));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_qw, qw.size() * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_bounds, bounds.size() * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->d_f_shells, f, (size_t)K * P->n_atoms * sizeof(float2),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->d_structs_shells, st.data(), st.size() * sizeof(gw_structure),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_qw, qw.data(), qw.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_bounds, bounds.data(), bounds.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int blocks = (int)std::min<int64_t>(((int64_t)W3 + 255) / 256, 16 * P->ctx->sm_count);
    k_shell_codes<<<blocks, 256, 0, s>>>(d_qw, P->W, d_bounds, d_bounds + K, K, P->d_shell);
    P->ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  gw::dev_free(d_qw);
  gw::dev_free(d_bounds);
  if (e != cudaSuccess) {
    drop();
    return gw::cuda_fail(e, "gw_voxel_set_shells", __FILE__, __LINE__);
  }
  P->n_shells = K;
  P->shell_mode = mode;
  P->shell_atoms = P->n_atoms;
  return GW_OK;
}

static int voxel_enqueue_all(gw_voxel_plan *P) { return enqueue(P); }

static int shell_state(gw_voxel_plan *P, const char *who) {
  if (P->n_shells > 0 && P->shell_atoms != P->n_atoms)
    return gw::fail(GW_ERR_STATE, std::string(who) +
                                      ": the atom count changed after gw_voxel_set_shells");
  if (P->n_shells == 0 && P->f_stale)
    return gw::fail(GW_ERR_STATE, std::string(who) +
                                      ": shells were cleared; set the atoms again");
  return GW_OK;
}

extern "C" int gw_voxel_execute(gw_voxel_plan *P) {
  if (!P) return gw::fail(GW_ERR_ARG, "gw_voxel_execute: null plan");
  if (P->n_atoms < 0) return gw::fail(GW_ERR_STATE, "gw_voxel_execute: atoms not set");
  GW_TRY(shell_state(P, "gw_voxel_execute"));
  GW_CUDA(cudaSetDevice(P->ctx->device));
  gw::Range r("giwaxsim: voxel execute");
  if (P->gexec) {
    GW_CUDA(cudaGraphLaunch(P->gexec, P->ctx->stream));
    P->ctx->launches += P->graph_kernels;
  } else {
    GW_TRY(voxel_enqueue_all(P));
  }
  P->executed = true;
  P->iq64_valid = false;
  return GW_OK;
}

extern "C" int32_t gw_voxel_block_variants(void) { return gwv::fused_variant_count(); }

extern "C" int gw_voxel_set_wait_limit(gw_voxel_plan *P, uint32_t polls) {
  if (!P) return gw::fail(GW_ERR_ARG, "gw_voxel_set_wait_limit: null plan");
  P->wait_polls = polls;
  // a captured graph holds the old limit in its kernel arguments
  if (P->gexec) cudaGraphExecDestroy(P->gexec);
  if (P->graph) cudaGraphDestroy(P->graph);
  P->gexec = nullptr;
  P->graph = nullptr;
  return GW_OK;
}

extern "C" int gw_voxel_capture_graph(gw_voxel_plan *P) {
  if (!P) return gw::fail(GW_ERR_ARG, "gw_voxel_capture_graph: null plan");
  if (P->n_atoms < 0) return gw::fail(GW_ERR_STATE, "gw_voxel_capture_graph: atoms not set");
  GW_TRY(shell_state(P, "gw_voxel_capture_graph"));
  if (P->gexec) return GW_OK;
  GW_CUDA(cudaSetDevice(P->ctx->device));
  // first-launch attributes must be set outside capture
  GW_TRY(voxel_enqueue_all(P));
  GW_CUDA(cudaStreamSynchronize(P->ctx->stream));
  const int64_t before = P->ctx->launches;
  GW_CUDA(cudaStreamBeginCapture(P->ctx->stream, cudaStreamCaptureModeThreadLocal));
  int st = voxel_enqueue_all(P);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(P->ctx->stream, &graph);
  if (st != GW_OK) { if (graph) cudaGraphDestroy(graph); return st; }
  if (e != cudaSuccess) return gw::cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  P->graph_kernels = P->ctx->launches - before;
  P->ctx->launches = before;
  P->graph = graph;
  GW_CUDA(cudaGraphInstantiate(&P->gexec, graph, 0));
  return GW_OK;
}

extern "C" int gw_voxel_get_iq(gw_voxel_plan *P, double *iq, int32_t on_device) {
  if (!P || !iq) return gw::fail(GW_ERR_ARG, "gw_voxel_get_iq: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_get_iq: plan not executed");
  const size_t n = (size_t)P->Qc * P->Qc * P->Qc;
  // Gather binning into a resident host array: the float64 grid is made in
  // GW_IQ_CHUNKS runs of lines (default 8; 1 or less: in one launch), each
  // copied out on the copy stream as soon as it is made, so that the
  // gather and the device-to-host copy overlap.
  const char *kc = getenv("GW_IQ_CHUNKS");
  const int K = std::min(16, kc ? atoi(kc) : 8);
  if (!P->iq64_valid && !on_device && P->n_out == 1 && K > 1 && gwv::gathering(P) &&
      gw::host_resident(iq, n * sizeof(double))) {
    GW_CUDA(cudaSetDevice(P->ctx->device));
    gw_ctx *c = P->ctx;
    GW_TRY(gw::copy_stream_ready(c));
    const int lines = P->Qc * P->Qc;
    int st = GW_OK;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < K && st == GW_OK && e == cudaSuccess; ++k) {
      const int l0 = (int)((int64_t)lines * k / K);
      const int l1 = (int)((int64_t)lines * (k + 1) / K);
      st = gwv::enqueue_gather(P, 1, 0, l0, l1);
      if (st != GW_OK) break;
      e = cudaEventRecord(c->copy_ev[k], c->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->copy_ev[k], 0);
      const size_t o = (size_t)l0 * P->Qc;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(iq + o, P->d_iq64 + o, (size_t)(l1 - l0) * P->Qc * sizeof(double),
                            cudaMemcpyDeviceToHost, c->copy_stream);
    }
    // the stream waits for every copy (also after a failed launch)
    cudaError_t j = cudaEventRecord(c->copy_ev[16], c->copy_stream);
    if (j == cudaSuccess) j = cudaStreamWaitEvent(c->stream, c->copy_ev[16], 0);
    if (st != GW_OK) return st;
    if (e != cudaSuccess) return gw::cuda_fail(e, "chunked result copy", __FILE__, __LINE__);
    if (j != cudaSuccess) return gw::cuda_fail(j, "chunked result copy", __FILE__, __LINE__);
    P->iq64_valid = true;
    return gw::check_device_error(P->ctx, "voxel stage");
  }
  // the float64 grid is made when asked for: an execute writes only the
  // float32 grid the detector reads
  if (!P->iq64_valid) {
    GW_CUDA(cudaSetDevice(P->ctx->device));
    GW_TRY(gwv::enqueue_finalize(P, true));
    P->iq64_valid = true;
  }
  if (!on_device && P->n_out == 1) {
    GW_TRY(gw::copy_to_host(iq, P->d_iq64, n * sizeof(double), P->ctx->stream));
    return gw::check_device_error(P->ctx, "voxel stage");
  }
  if (!on_device) gw::prefault_host(iq, n * P->n_out * sizeof(double));
  // one 2-D copy packs the structures' padded grids back to back
  GW_CUDA(cudaMemcpy2DAsync(iq, n * sizeof(double), P->d_iq64,
                            P->iq_stride * sizeof(double), n * sizeof(double),
                            P->n_out,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            P->ctx->stream));
  return gw::check_device_error(P->ctx, "voxel stage");
}

extern "C" int gw_voxel_get_iq32(gw_voxel_plan *P, float *iq32) {
  if (!P || !iq32) return gw::fail(GW_ERR_ARG, "gw_voxel_get_iq32: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_get_iq32: plan not executed");
  const size_t n = (size_t)P->Qc * P->Qc * P->Qc;
  gw::prefault_host(iq32, n * P->n_out * sizeof(float));
  GW_CUDA(cudaMemcpy2DAsync(iq32, n * sizeof(float), P->d_iq32,
                            P->iq_stride * sizeof(float), n * sizeof(float),
                            P->n_out, cudaMemcpyDeviceToHost, P->ctx->stream));
  return gw::check_device_error(P->ctx, "voxel stage");
}

extern "C" int gw_voxel_device_iq32(gw_voxel_plan *P, int32_t structure,
                                    const float **iq32) {
  if (!P || !iq32) return gw::fail(GW_ERR_ARG, "gw_voxel_device_iq32: null argument");
  if (structure < 0 || structure >= P->n_out)
    return gw::fail(GW_ERR_ARG, "gw_voxel_device_iq32: structure " +
                                    std::to_string(structure) + " outside [0, " +
                                    std::to_string(P->n_out) + ")");
  *iq32 = P->d_iq32 + (size_t)structure * P->iq_stride;
  return GW_OK;
}

extern "C" int gw_voxel_get_counts(gw_voxel_plan *P, double *counts) {
  if (!P || !counts) return gw::fail(GW_ERR_ARG, "gw_voxel_get_counts: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_get_counts: plan not executed");
  std::vector<unsigned> C2((size_t)P->W * P->W);
  GW_CUDA(cudaMemcpyAsync(C2.data(), P->d_C2, C2.size() * sizeof(unsigned),
                          cudaMemcpyDeviceToHost, P->ctx->stream));
  GW_TRY(gw::check_device_error(P->ctx, "voxel stage"));
  const int off = P->lo - P->wlo, Q = P->Qc;
  for (int y = 0; y < Q; ++y)
    for (int x = 0; x < Q; ++x)
      for (int z = 0; z < Q; ++z)
        counts[((size_t)y * Q + x) * Q + z] =
            (double)C2[(size_t)(y + off) * P->W + x + off] *
            (double)P->C1host[z + off] * (double)P->n_struct;
  return GW_OK;
}

extern "C" int gw_voxel_get_sums(gw_voxel_plan *P, double *sums) {
  if (!P || !sums) return gw::fail(GW_ERR_ARG, "gw_voxel_get_sums: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_get_sums: plan not executed");
  const size_t W3 = (size_t)P->W * P->W * P->W;
  std::vector<double> s(W3);
  if (P->p.accum == GW_ACCUM_KAHAN32) {
    std::vector<float2> k(W3);
    GW_CUDA(cudaMemcpyAsync(k.data(), P->d_sumk, W3 * sizeof(float2),
                            cudaMemcpyDeviceToHost, P->ctx->stream));
    GW_TRY(gw::check_device_error(P->ctx, "voxel stage"));
    for (size_t i = 0; i < W3; ++i) s[i] = (double)k[i].x - (double)k[i].y;
  } else {
    // gather binning keeps no sum grid: made from the stored pixels here
    if (gwv::gathering(P)) GW_TRY(gwv::enqueue_gather(P, 2, 0));
    GW_CUDA(cudaMemcpyAsync(s.data(), P->d_sum, W3 * sizeof(double),
                            cudaMemcpyDeviceToHost, P->ctx->stream));
    GW_TRY(gw::check_device_error(P->ctx, "voxel stage"));
  }
  const int off = P->lo - P->wlo, Q = P->Qc;
  for (int y = 0; y < Q; ++y)
    for (int x = 0; x < Q; ++x)
      for (int z = 0; z < Q; ++z)
        sums[((size_t)y * Q + x) * Q + z] =
            s[((size_t)(y + off) * P->W + x + off) * P->W + z + off];
  return GW_OK;
}

extern "C" int gw_voxel_info(gw_voxel_plan *P, int64_t *info, int32_t n) {
  if (!P || !info) return gw::fail(GW_ERR_ARG, "gw_voxel_info: null argument");
  const int64_t v[] = {P->Qc, P->S, P->Ly, P->Lz, P->Nc, P->Nr, P->My, P->Mz,
                       P->y_lo, P->z_lo, P->k0, P->kz0, P->n_slices,
                       (int64_t)P->bytes, P->graph_kernels,
                       (int64_t)P->f1_tma, (int64_t)P->fused_y,
                       (int64_t)P->fused_z, (int64_t)P->real, (int64_t)P->gather,
                       P->gather ? P->n_heavy : 0, P->gather ? P->n_zmulti : 0};
  const int k = std::min<int>(n, (int)(sizeof v / sizeof v[0]));
  for (int i = 0; i < k; ++i) info[i] = v[i];
  return k;
}

extern "C" int gw_voxel_debug_deposit(gw_voxel_plan *P, int32_t slice,
                                      int32_t *y_idx, int32_t *z_idx) {
  if (!P || !y_idx || !z_idx) return gw::fail(GW_ERR_ARG, "gw_voxel_debug_deposit: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_debug_deposit: plan not executed");
  if (slice < 0 || slice >= P->n_slices) return gw::fail(GW_ERR_ARG, "gw_voxel_debug_deposit: slice out of range");
  const gw_structure &s = P->structs[slice / P->n_phi];
  int *dy = nullptr, *dz = nullptr;
  GW_CUDA(gw::dev_malloc((void **)&dy, s.atom_count * sizeof(int)));
  cudaError_t e = gw::dev_malloc((void **)&dz, s.atom_count * sizeof(int));
  if (e != cudaSuccess) { gw::dev_free(dy); return gw::cuda_fail(e, "dev_malloc", __FILE__, __LINE__); }
  SliceArgs a = slice_args(P);
  k_debug_deposit<<<256, 256, 0, P->ctx->stream>>>(a, slice, dy, dz);
  P->ctx->launches++;
  e = cudaMemcpyAsync(y_idx, dy, s.atom_count * sizeof(int), cudaMemcpyDeviceToHost, P->ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(z_idx, dz, s.atom_count * sizeof(int), cudaMemcpyDeviceToHost, P->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->ctx->stream);
  gw::dev_free(dy);
  gw::dev_free(dz);
  if (e != cudaSuccess) return gw::cuda_fail(e, "debug deposit", __FILE__, __LINE__);
  return GW_OK;
}

extern "C" int gw_voxelgrid(gw_ctx *ctx, const gw_voxel_params *p,
                            const gw_structure *structs, int32_t n_struct,
                            const gw_phi *phis, int32_t n_phi,
                            const double *xyz, const float *f, int64_t n_atoms,
                            double *iq_out) {
  gw_voxel_plan *P = nullptr;
  GW_TRY(gw_voxel_plan_create(ctx, p, structs, n_struct, phis, n_phi, &P));
  int st = gw_voxel_set_atoms(P, xyz, f, n_atoms, 0);
  if (st == GW_OK) st = gw_voxel_execute(P);
  if (st == GW_OK) st = gw_voxel_get_iq(P, iq_out, 0);
  gw_voxel_plan_destroy(P);
  return st;
}

extern "C" int gw_voxel_debug_window(gw_voxel_plan *P, int32_t slice,
                                     float *window) {
  if (!P || !window) return gw::fail(GW_ERR_ARG, "gw_voxel_debug_window: null argument");
  if (!P->executed) return gw::fail(GW_ERR_STATE, "gw_voxel_debug_window: plan not executed");
  if (slice < 0 || slice >= P->n_slices) return gw::fail(GW_ERR_ARG, "gw_voxel_debug_window: slice out of range");
  const size_t n = (size_t)P->Lz * P->Ly;
  float2 *d = nullptr;
  GW_CUDA(gw::dev_malloc((void **)&d, n * sizeof(float2)));
  cudaError_t e = cudaMemsetAsync(d, 0, n * sizeof(float2), P->ctx->stream);
  SliceArgs a = slice_args(P);
  if (e == cudaSuccess) {
    k_debug_window<<<256, 128, 0, P->ctx->stream>>>(a, slice, d);
    P->ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(window, d, n * sizeof(float2), cudaMemcpyDeviceToHost, P->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->ctx->stream);
  gw::dev_free(d);
  if (e != cudaSuccess) return gw::cuda_fail(e, "debug window", __FILE__, __LINE__);
  return GW_OK;
}
