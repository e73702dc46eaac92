// Internal declarations of the voxel stage shared by the forward kernels
// (gw_voxel.cu) and the adjoint kernels (gw_grad.cu): the per-slice argument
// block, the chirp-z argument block, the plan object, and the device helpers
// that both sides must evaluate identically (deposit index, window mapping,
// smoothing profile).
#pragma once

#include <algorithm>
#include <climits>
#include <complex>
#include <vector>

#include <cuda.h>

#include "gw_common.cuh"
#include "gw_fft.cuh"
#include "gw_slice.cuh"

namespace gwv {

constexpr int kMinM = 64, kMaxM = 8192;

struct SliceArgs {
  // geometry
  int g;
  double r, inv_r;
  int n_phi;
  int y_lo, Ly, z_lo, Lz;
  int fill, smooth_on;
  float sigma;
  int radius;
  int plain;
  int bil;             // bilinear deposit (two rows x two columns per atom)
  // arrays
  const double *xyz;   // atoms in input order
  const float2 *f;
  const int *zidx;
  const double *xyz_s; // atoms sorted by z index within each structure
  const float4 *xyf_s; // sorted atoms: float32 (x, y) and f (re, im)
  const float *fz_s;   // bilinear: fractional z position of the sorted atoms
  unsigned *ybnd;      // per slice: float32 bounds on the y extremes (ordered)
  const int *roff;     // per slice: first window row (n_slices+1 entries),
                       // when structures have their own z windows; else null
  const int *rowstart; // per structure: g+2 offsets into the sorted arrays
  const int2 *zstat;   // per structure: (max valid z index, all z valid)
  const gw_structure *st;
  const gw_phi *ph;
  const double *clbase;  // per slice
  unsigned long long *ymin_ord, *ymax_ord;
  int *extflag;          // per slice: 1 = extents need the exact pass
  int4 *ext;  // y_min, y_max, z_min, z_max (valid atoms)
  float2 *amo;
  float *my, *mz;
  // real grids: per slot and window column, (the fill value projected on
  // the structure's phase, NaN outside the slice's y extent; the y
  // smoothing factor, 1 without smoothing), made by k_profile
  float2 *pr;
  const float *gw;  // gaussian weights, 2*radius+1
  float4 *sconst;   // per slice: (Cbg.re, Cbg.im, Cd.re, Cd.im)
  int *err;
};

struct CztArgs {
  int M;
  int L, N;  // input length, output length
  const float2 *A, *H, *B, *tw;
};

struct BinArgs {
  const int *colofs;  // [n_phi][Nc], -1 = not binned
  const int *rowofs;  // [Nr], -1 = not binned
  double *sum;        // window^3 float64
  float2 *sumk;       // window^3 (sum, compensation) for Kahan float32
  int kahan;
  int k0, kz0;        // frequency of output column 0 / row 0
  float dc_scale;     // g*g
  int64_t sstride;    // window^3 per structure in separate mode, else 0
  // q-shell pass (multi-q form factors): bin only the voxels of shell
  // shell_k; null = every voxel
  const unsigned short *shell;
  int shell_k;
  // polls of the column kernel's bounded wait for its tile load
  unsigned wait_polls;
  // real grids (only the columns ky >= 0 are transformed): F1 column j is
  // table column m_zero + j, and every pixel (m, mr) with m > m_zero is
  // binned again at its mirror (2 m_zero - m, 2 r_zero - mr), where
  // |F(-ky, -kz)|^2 = |F(ky, kz)|^2
  int mirror, m_zero, r_zero;
  // gather binning: store |F|^2 of (slice, F1 column, output row) at
  // G[(slice * nf + column) * Nr + row] instead of adding it (null: add)
  float *G;
};

// Default poll limit of a bounded wait for an asynchronous tile load: far
// beyond any load's latency (a few microseconds), short of a hang.
constexpr unsigned kTileWaitPolls = 1u << 22;

// Shell code of a voxel: 2 k + 1 if it lies in shells k and k + 1 (a
// boundary rounding case), 2 k if in shell k only, kNoShell if in none.
constexpr unsigned short kNoShell = 0xFFFF;
__device__ __forceinline__ bool shell_member(unsigned short c, int k) {
  if (c == kNoShell) return false;
  const int k1 = c >> 1;
  return k == k1 || ((c & 1) && k == k1 + 1);
}

struct SliceConst {
  float2 cbg, cd;
};

__device__ __forceinline__ SliceConst slice_const(const SliceArgs &a, int sl) {
  const float4 v = a.sconst[sl];
  SliceConst k;
  k.cbg = make_float2(v.x, v.y);
  k.cd = make_float2(v.z, v.w);
  return k;
}

__device__ __forceinline__ double rot_y(const double *p, double c, double s) {
  // column 1 of np.dot(coords, Rz.T): fma(z,0,fma(y,c,x*s)) == fma(y,c,x*s)
  return GW_DFMA(p[1], c, GW_DMUL(p[0], s));
}

// Python slice normalisation of [start:stop] on a length-n axis.
__device__ __forceinline__ void py_slice(int start, int stop, int n, int &s,
                                         int &e) {
  if (start < 0) { start += n; if (start < 0) start = 0; }
  else if (start > n) start = n;
  if (stop < 0) { stop += n; if (stop < 0) stop = 0; }
  else if (stop > n) stop = n;
  s = start;
  e = stop;
}

// gaussian_filter1d(mask, sigma, mode='wrap') of the plateau [ms, me), with
// the kernel weights w (or their sigma derivative).
__device__ __forceinline__ float smooth_at(int i, int ms, int me, int g,
                                           int radius, const float *w) {
  float acc = 0.f;
  for (int j = -radius; j <= radius; ++j) {
    int k = i + j;
    k %= g; if (k < 0) k += g;
    if (k >= ms && k < me) acc += w[j + radius];
  }
  return acc;
}

// Smoothing plateau bounds of slice extents e (voxelgrids.py:369-370, with
// ceil() for non-integer sigma).
__device__ __forceinline__ void plateau(const SliceArgs &a, int4 e, int &ys,
                                        int &ye, int &zs, int &ze) {
  const float sg = a.sigma;
  py_slice((int)ceilf((float)e.x + sg), (int)ceilf((float)e.y - sg), a.g, ys, ye);
  py_slice((int)ceilf((float)e.z + sg), (int)ceilf((float)e.w - sg), a.g, zs, ze);
}

// Batch-relative window row -> (slot, zz).  Every slice has Lz rows, or,
// with per-structure windows, roff[s+1] - roff[s] rows.
__device__ __forceinline__ void row_slot(const SliceArgs &a, int slice0,
                                         int n_sl, int row, int &slot,
                                         int &zz) {
  if (!a.roff) {
    slot = row / a.Lz;
    zz = row - slot * a.Lz;
    return;
  }
  const int R = a.roff[slice0] + row;
  int lo = 0, hi = n_sl - 1;  // last slot whose first row is <= R
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.roff[slice0 + mid] <= R) lo = mid;
    else hi = mid - 1;
  }
  slot = lo;
  zz = R - a.roff[slice0 + lo];
}

// Window rows of slice sl and the first of them relative to slice0.
__device__ __forceinline__ void slice_rows(const SliceArgs &a, int slice0,
                                           int sl, int &first, int &count) {
  if (!a.roff) {
    first = (sl - slice0) * a.Lz;
    count = a.Lz;
  } else {
    first = a.roff[sl] - a.roff[slice0];
    count = a.roff[sl + 1] - a.roff[sl];
  }
}

__device__ __forceinline__ int window_row_to_z(const SliceArgs &a, int zz) {
  int zi = a.z_lo + zz;
  if (zi < 0) zi += a.g;
  if (zi >= a.g) zi -= a.g;
  return zi;
}

// Window column of grid column yi (yi in [0, g)); >= Ly flags an overflow.
__device__ __forceinline__ int window_col(const SliceArgs &a, int yi) {
  int yy = yi - a.y_lo;
  if (yy >= a.g) yy -= a.g;
  return yy;
}

// D value of box element (zz, yy) of slice slot `slot`.
__device__ __forceinline__ float2 d_value(const SliceArgs &a, int slot, int sl,
                                          int zz, int yy, float2 dep, float2 cd,
                                          float2 cbg, int4 e) {
  float2 v;
  if (a.fill) {
    int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
    int zi = a.z_lo + zz; if (zi < 0) zi += a.g; if (zi >= a.g) zi -= a.g;
    const bool inside = zi >= e.z && zi < e.w && yi > e.x && yi < e.y;
    v = inside ? cadd(dep, a.amo[(size_t)slot * a.Ly + yy]) : cd;
  } else {
    v = csub(dep, cbg);
  }
  if (a.smooth_on) {
    const float m = a.mz[(size_t)slot * a.Lz + zz] * a.my[(size_t)slot * a.Ly + yy];
    v = make_float2(v.x * m + cd.x * (1.f - m), v.y * m + cd.y * (1.f - m));
  }
  return v;
}

// The per-row part of d_value, hoisted: a block that transforms whole rows
// evaluates it once per row.
struct RowConst {
  float2 cd, cbg;  // slice constants (sconst)
  int4 e;          // slice extents
  float mz;        // z smoothing factor of the row (1 when smoothing is off)
  int zin;         // the row's z lies inside [e.z, e.w)
  int slot;
  float2 u;        // unit phase of the structure's average voxel f (real
                   // grids: the row is u times a real row)
};

// Unit phase of a structure's average voxel f (real grids: its slice grids
// are this phase times real grids).
__device__ __forceinline__ float2 unit_phase(const gw_structure &st) {
  const double mag = sqrt(st.avg_f_re * st.avg_f_re + st.avg_f_im * st.avg_f_im);
  return mag > 0.0 ? make_float2((float)(st.avg_f_re / mag), (float)(st.avg_f_im / mag))
                   : make_float2(1.f, 0.f);
}

__device__ __forceinline__ RowConst row_const(const SliceArgs &a, int slot,
                                              int sl, int zz) {
  RowConst k;
  const SliceConst c = slice_const(a, sl);
  k.cd = c.cd;
  k.cbg = c.cbg;
  k.e = a.ext[sl];
  k.mz = a.smooth_on ? a.mz[(size_t)slot * a.Lz + zz] : 1.f;
  const int zi = window_row_to_z(a, zz);
  k.zin = zi >= k.e.z && zi < k.e.w;
  k.slot = slot;
  k.u = unit_phase(a.st[sl / a.n_phi]);
  return k;
}

// d_value of element yy of a row with constants k: the same operations in
// the same order.
// The slice arguments the per-element grid value reads, by value: a
// transform functor holding them in registers reads no field through a
// pointer to the kernel's parameter block (a generic load per element).
struct RowValueArgs {
  const float2 *amo;
  const float *my;
  const float2 *pr;
  int fill, smooth_on, y_lo, g, Ly;
};

__device__ __forceinline__ RowValueArgs row_value_args(const SliceArgs &a) {
  return RowValueArgs{a.amo, a.my, a.pr, a.fill, a.smooth_on, a.y_lo, a.g, a.Ly};
}

__device__ __forceinline__ float2 d_value_row(const RowValueArgs &a,
                                              const RowConst &k, int yy,
                                              float2 dep) {
  float2 v;
  if (a.fill) {
    int yi = a.y_lo + yy; if (yi < 0) yi += a.g; if (yi >= a.g) yi -= a.g;
    const bool inside = k.zin && yi > k.e.x && yi < k.e.y;
    v = inside ? cadd(dep, a.amo[(size_t)k.slot * a.Ly + yy]) : k.cd;
  } else {
    v = csub(dep, k.cbg);
  }
  if (a.smooth_on) {
    const float m = k.mz * a.my[(size_t)k.slot * a.Ly + yy];
    v = make_float2(v.x * m + k.cd.x * (1.f - m), v.y * m + k.cd.y * (1.f - m));
  }
  return v;
}

__device__ __forceinline__ float2 d_value_row(const SliceArgs &a,
                                              const RowConst &k, int yy,
                                              float2 dep) {
  return d_value_row(row_value_args(a), k, yy, dep);
}

// Real grids: Re(d_value_row(a, k, yy, r u) conj(u)) for the real row sum
// r.  The fill and smoothing values (amo, cd, cbg) are multiples of u, so
// the projection is taken term by term, in float32 (|u| = 1); the slot's
// projected fill value, its y-extent test and the y smoothing factor come
// as one 8-byte load of the k_profile table pr.
__device__ __forceinline__ float d_value_row_real(const RowValueArgs &a,
                                                  const RowConst &k, int yy,
                                                  float r) {
  const float cdr = k.cd.x * k.u.x + k.cd.y * k.u.y;
  // (k_profile runs, and makes the table, with fill or smoothing only)
  const float2 t = (a.fill || a.smooth_on) ? a.pr[(size_t)k.slot * a.Ly + yy]
                                           : make_float2(0.f, 1.f);
  float v;
  if (a.fill) v = (k.zin && t.x == t.x) ? r + t.x : cdr;
  else v = r - (k.cbg.x * k.u.x + k.cbg.y * k.u.y);
  if (a.smooth_on) {
    const float m = k.mz * t.y;
    v = v * m + cdr * (1.f - m);
  }
  return v;
}

// Window column of sorted atom `at` in slice `sl` (nearest-bin deposit):
// false when the valid mask drops it (y index outside [0, g)); yy >= Ly
// flags a window overflow.
// The index is first estimated in float32: t = (x s + y c - ymin)/r with an
// error below d = 10 u (|x s| + |y c| + |ymin|)/r + 1e-6 (u = 2^-24; the
// input roundings, four arithmetic roundings and those of t -+ d total at
// most 7 u times that sum).  Only when [t-d, t+d] contains an integer is the
// exact float64 chain replayed.
// The per-slice constants of the deposit (a block evaluates them once per
// row).
struct DepRow {
  double ymin, cphi, sphi;
  float cs, sn, ym;
};

__device__ __forceinline__ DepRow dep_row(const SliceArgs &a, int sl) {
  const gw_phi &ph = a.ph[sl % a.n_phi];
  DepRow k;
  k.ymin = ord_dbl(a.ymin_ord[sl]);
  k.cphi = ph.cos_phi;
  k.sphi = ph.sin_phi;
  k.cs = (float)ph.cos_phi;
  k.sn = (float)ph.sin_phi;
  k.ym = (float)k.ymin;
  return k;
}

// xy: the atom's float32 (x, y) (xyf_s[at].x, .y).
__device__ __forceinline__ bool deposit_column(const SliceArgs &a,
                                               const DepRow &k, float2 xy,
                                               int at, int &yy) {
  const float ir = (float)a.inv_r;
  const float t = (fmaf(xy.y, k.cs, xy.x * k.sn) - k.ym) * ir;
  const float d = 10.f * 5.9604645e-8f *
                      (fabsf(xy.x * k.sn) + fabsf(xy.y * k.cs) + fabsf(k.ym)) * ir +
                  1e-6f;
  int klo, khi, yi;
  if (floor_to_int(t - d, klo) && floor_to_int(t + d, khi) && klo == khi) {
    yi = klo;
  } else {
    const double y = GW_DSUB(rot_y(a.xyz_s + 3 * (size_t)at, k.cphi, k.sphi), k.ymin);
    yi = (int)floor_div_exact(y, a.r, a.inv_r);
  }
  if (yi < 0 || yi >= a.g) return false;
  yy = window_col(a, yi);
  return true;
}

__device__ __forceinline__ bool deposit_column(const SliceArgs &a, int at,
                                               int sl, int &yy) {
  const float4 q = a.xyf_s[at];
  return deposit_column(a, dep_row(a, sl), make_float2(q.x, q.y), at, yy);
}

// Bilinear deposit of sorted atom `at` in slice `sl`: the atom's shifted
// position u = (y' - ymin)/r splits between columns i0 = floor(u) (weight
// 1-fu) and i0+1 (weight fu).  The atom is valid when i0 is inside the grid
// (the nearest-bin valid mask); a corner at g is dropped.
__device__ __forceinline__ bool bilinear_column(const SliceArgs &a, int at,
                                                int sl, int &i0, float &fu) {
  const gw_phi &ph = a.ph[sl % a.n_phi];
  const double ymin = ord_dbl(a.ymin_ord[sl]);
  const double y = GW_DSUB(rot_y(a.xyz_s + 3 * (size_t)at, ph.cos_phi,
                                 ph.sin_phi), ymin);
  const double k = floor_div_exact(y, a.r, a.inv_r);
  if (k < 0.0 || k >= (double)a.g) return false;
  i0 = (int)k;
  const float t = (float)(GW_DMUL(y, a.inv_r) - k);
  fu = fminf(fmaxf(t, 0.f), 1.f);
  return true;
}

// Atom range of window row zz: nearest-bin rows hold the atoms of z index
// zi; bilinear rows also those of zi-1 (their upper z corner).  `mid` is the
// first atom of index zi.
__device__ __forceinline__ void row_atoms(const SliceArgs &a, int t, int zz,
                                          int &lo, int &mid, int &hi) {
  const int zi = window_row_to_z(a, zz);
  const int *rs = a.rowstart + (size_t)t * (a.g + 2);
  mid = rs[zi];
  hi = rs[zi + 1];
  lo = (a.bil && zi > 0) ? rs[zi - 1] : mid;
}

// Add w * fv at grid column i of a shared-memory row.
__device__ __forceinline__ void deposit_at(const SliceArgs &a, float2 *row,
                                           int i, float2 fv, float w) {
  const int yy = window_col(a, i);
  if (yy < a.Ly) {
    atomicAdd(&row[yy].x, fv.x * w);
    atomicAdd(&row[yy].y, fv.y * w);
  } else {
    dev_error(a.err, GW_DEVERR_BOX);
  }
}

// Per-row state of a row-transform block (shared memory).
template <int NB>
struct RowShared {
  int lo[NB], mid[NB], cnt[NB + 1], slot[NB];
  RowConst k[NB];
  DepRow d[NB];
};

// The deposit of a row-transform block (voxelgrids.py:319-341: shift,
// floor division, valid mask, np.add.at): NB window rows starting at row0
// of the batch, row f into buf[f * ldm + 0 .. L) (zeroed first), by shared
// atomics.  Sets up rs (slot, window row, atom range and constants of every
// row) and leaves the block synchronised.  REAL (real grids, nearest bin):
// each atom adds Re(f conj(u)) to the .x of its element only, u the row's
// unit phase (the row is u times that real row): one shared atomic per atom.
template <int NB, int NT, bool BIL, bool REAL = false>
__device__ __forceinline__ void deposit_rows(const SliceArgs &a, int L,
                                             int slice0, int n_sl, int n_rows,
                                             int row0, float2 *buf, int ldm,
                                             RowShared<NB> &rs) {
  // only the window columns [0, L) are deposited into and read back; a
  // real row (REAL) is a float array, row f at float offset f ldm
  float *rbuf = reinterpret_cast<float *>(buf);
  for (int f = 0; f < NB; ++f)
    for (int n = threadIdx.x; n < L; n += NT) {
      if constexpr (REAL) rbuf[f * ldm + n] = 0.f;
      else buf[f * ldm + n] = make_float2(0.f, 0.f);
    }
  // the block's rows: slot, window row and atom range, one thread per row
  // (independent loads), then a scan of the atom counts
  static_assert(NB <= 32, "one warp sets the rows up");
  if (threadIdx.x < NB) {
    const int f = threadIdx.x, row = row0 + f;
    int lo = 0, mid = 0, hi = 0, slot = 0, zz = 0;
    if (row < n_rows) {
      row_slot(a, slice0, n_sl, row, slot, zz);
      const int sl = slice0 + slot, t = sl / a.n_phi;
      if (a.ext[sl].y < 0) dev_error(a.err, GW_DEVERR_NO_ATOMS);
      row_atoms(a, t, zz, lo, mid, hi);
    }
    rs.lo[f] = lo;
    rs.mid[f] = mid;
    rs.cnt[f + 1] = hi - lo;
    rs.slot[f] = slot;
    if (row < n_rows) {
      rs.k[f] = row_const(a, slot, slice0 + slot, zz);
      rs.d[f] = dep_row(a, slice0 + slot);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    rs.cnt[0] = 0;
    for (int f = 0; f < NB; ++f) rs.cnt[f + 1] += rs.cnt[f];
  }
  __syncthreads();
  const int total = rs.cnt[NB];
  for (int i = threadIdx.x; i < total; i += NT) {
    int f = 0;
    while (f + 1 < NB && i >= rs.cnt[f + 1]) ++f;
    const int at = rs.lo[f] + (i - rs.cnt[f]);
    const int sl = slice0 + rs.slot[f];
    if constexpr (!BIL) {
      int yy;
      const float4 q = a.xyf_s[at];
      if (deposit_column(a, rs.d[f], make_float2(q.x, q.y), at, yy)) {
        if (yy < a.Ly) {
          if constexpr (REAL) {
            const float2 u = rs.k[f].u;
            atomicAdd(rbuf + f * ldm + yy, fmaf(q.z, u.x, q.w * u.y));
          } else {
            atomicAdd(&buf[f * ldm + yy].x, q.z);
            atomicAdd(&buf[f * ldm + yy].y, q.w);
          }
        } else {
          dev_error(a.err, GW_DEVERR_BOX);
        }
      }
    } else {
      int i0;
      float fu;
      if (bilinear_column(a, at, sl, i0, fu)) {
        const float fz = a.fz_s[at];
        const float wz = at >= rs.mid[f] ? 1.f - fz : fz;
        const float4 q = a.xyf_s[at];
        const float2 fv = make_float2(q.z, q.w);
        deposit_at(a, buf + f * ldm, i0, fv, wz * (1.f - fu));
        if (i0 + 1 < a.g) deposit_at(a, buf + f * ldm, i0 + 1, fv, wz * fu);
      }
    }
  }
  __syncthreads();
}

// Kahan-compensated float32 accumulation into a (sum, compensation) pair,
// as one 64-bit compare-and-swap.
__device__ __forceinline__ void kahan_add(float2 *addr, float x) {
  unsigned long long *p = reinterpret_cast<unsigned long long *>(addr);
  unsigned long long old = *p, assumed;
  do {
    assumed = old;
    float2 sc;
    memcpy(&sc, &assumed, 8);
    const float y = x - sc.y;
    const float t = sc.x + y;
    const float c = (t - sc.x) - y;
    float2 nw = make_float2(t, c);
    unsigned long long nv;
    memcpy(&nv, &nw, 8);
    old = atomicCAS(p, assumed, nv);
  } while (old != assumed);
}

// Rows per TMA box for transform length M: a divisor of M of at most 256,
// so the boxes covering a slice's rows (at most M) fit the FFT buffer.
__host__ __device__ constexpr int tma_box_rows(int M) {
  return M % 256 == 0 ? 256 : M % 192 == 0 ? 192 : M % 160 == 0 ? 160
                                                                 : M % 128 == 0 ? 128 : 64;
}

// ------------------------------------------------------------ host helpers
struct CztTables {
  std::vector<float2> A, H, B, tw;
};

// X[k0+m] = sum_{n<L} x[lo+n] W^{(lo+n)(k0+m)}, W = exp(-2 pi i/g), via
// B[m] * conv(x*A, h)[m], h[j] = W^{-j^2/2}, j in [-(L-1), N-1].
CztTables make_czt(int g, int lo, int L, int k0, int N, int M);
// Smallest supported transform length >= n (0 if none).
int next_fft_size(int n, bool pow2_only);
bool fft_size_supported(int m);

template <typename T>
int upload(T **dst, const std::vector<T> &v, size_t *bytes) {
  if (v.empty()) { *dst = nullptr; return GW_OK; }
  GW_CUDA(gw::dev_malloc((void **)dst, v.size() * sizeof(T)));
  *bytes += v.size() * sizeof(T);
  GW_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T),
                     cudaMemcpyHostToDevice));
  return GW_OK;
}

template <typename T>
int alloc(T **dst, size_t n, size_t *bytes) {
  if (n == 0) { *dst = nullptr; return GW_OK; }
  GW_CUDA(gw::dev_malloc((void **)dst, n * sizeof(T)));
  *bytes += n * sizeof(T);
  return GW_OK;
}

}  // namespace gwv

struct gw_grad_state;

// ================================================================== plan
struct gw_voxel_plan {
  gw_ctx *ctx = nullptr;
  gw_voxel_params p{};
  int n_struct = 0, n_phi = 0, n_slices = 0;
  std::vector<gw_structure> structs;
  std::vector<gw_phi> phis;
  int g = 0, plain = 0, Qc = 0, lo = 0, hi = 0, wlo = 0, whi = 0, W = 0;
  double r = 0, inv_r = 0, dq = 0, inv_dq = 0;
  int radius = 0, bil = 0;
  int y_lo = 0, Ly = 0, z_lo = 0, Lz = 0, k0 = 0, Nc = 0, kz0 = 0, Nr = 0;
  int My = 0, Mz = 0, S = 1;
  int n_out = 1;           // I(q) grids produced: n_struct in separate mode
  // element strides between the structures' sum and I(q) grids, rounded up
  // to 4 so that every grid starts 16-byte aligned for the vector loads and
  // stores of the finalize kernel
  size_t sum_stride = 0, iq_stride = 0;
  // multi-q form factors: n_shells passes with per-shell atom f values and
  // structure tables (0 = off)
  int n_shells = 0, shell_mode = 0;
  int64_t shell_atoms = -1;    // n_atoms the shell tables were made for
  bool f_stale = false;        // d_f holds a shell's f values, not the atoms'
  unsigned short *d_shell = nullptr;  // window^3 shell codes
  float2 *d_f_shells = nullptr;       // [n_shells][n_atoms]
  gw_structure *d_structs_shells = nullptr;  // [n_shells][n_struct]
  int64_t n_atoms = -1;
  size_t bytes = 0;
  std::vector<int> C1host;
  // device
  double *d_xyz = nullptr;
  float2 *d_f = nullptr;
  int *d_zidx = nullptr;
  gw_structure *d_structs = nullptr;
  gw_phi *d_phis = nullptr;
  double *d_clbase = nullptr;
  unsigned long long *d_zmin = nullptr, *d_ymin = nullptr;
  int4 *d_ext = nullptr;
  float2 *d_Ay = nullptr, *d_Hy = nullptr, *d_By = nullptr, *d_twy = nullptr;
  float2 *d_Az = nullptr, *d_Hz = nullptr, *d_Bz = nullptr, *d_twz = nullptr;
  float *d_gw = nullptr;
  int *d_colofs = nullptr, *d_rowofs = nullptr, *d_C1 = nullptr;
  unsigned int *d_C2 = nullptr;
  double *d_sum = nullptr;
  float2 *d_sumk = nullptr;
  float *d_f0 = nullptr;
  float4 *d_zf0 = nullptr;  // f0 z factors of the four terms per qz (or null)
  double *d_iq64 = nullptr;
  float *d_iq32 = nullptr;
  float2 *d_F1 = nullptr, *d_amo = nullptr;
  // 2-D tensor map of d_F1 (columns inner) for the column kernel's tile
  // loads; f1_tma false when the band or the block width does not allow them
  CUtensorMap f1map{};
  bool f1_tma = false;
  unsigned wait_polls = gwv::kTileWaitPolls;  // gw_voxel_set_wait_limit
  int f1_box_cols = 0;  // columns per box of f1map
  // real grids (gw_voxel_params.real_grids and the shape allows it): two
  // window rows per row transform, only the columns ky >= 0 in F1 (Nf of
  // them, table columns m_zero ..), mirrored binning; the bands are
  // symmetric around ky = 0 (m_zero) and kz = 0 (r_zero)
  bool real = false;
  int m_zero = 0, r_zero = 0;
  int Nf = 0;  // F1 row pitch (columns stored): Nc, or Nc - m_zero
  // gather binning (gw_voxel_params.binning): the column kernels store each
  // slice's |F|^2 pixels in d_G ([slice][F1 column][output row], float32)
  // and k_gather adds every voxel line's pixels in a fixed order.  Window
  // line l takes the entries d_lent[d_lptr[l] .. d_lptr[l+1]) = (phi, F1
  // column * 2 + mirrored), each over every structure's slice of that phi;
  // window z takes the output rows d_zrows[d_zptr[z] .. d_zptr[z+1]) (a
  // mirrored entry reads row 2 r_zero - mr)
  float2 *d_pr = nullptr;  // real grids: the row kernel's column table
  bool gather = false;
  float *d_G = nullptr;
  int *d_lptr = nullptr, *d_zptr = nullptr, *d_zrows = nullptr;
  int2 *d_lent = nullptr;
  // window lines with many entries (each takes a whole block)
  int *d_heavy = nullptr;
  int n_heavy = 0;
  std::vector<int> h_heavy;  // the heavy window lines, ascending (host copy)
  // window z with more than one output row (their voxels are summed again
  // over every row)
  int *d_zmulti = nullptr;
  int n_zmulti = 0;
  // fused chirp-z kernels (gw_czt2.cuh) along y / z, with their twiddles
  bool fused_y = false, fused_z = false;
  float2 *d_fty = nullptr, *d_ftz = nullptr;
  double *d_xyz_s = nullptr;
  float4 *d_xyf_s = nullptr;
  float *d_fz_s = nullptr;
  int *d_perm = nullptr;   // sorted position -> input atom index
  unsigned *d_ybnd = nullptr;  // 2 per slice (see k_ybound)
  std::vector<int> roff_host;  // per-slice first window row (n_slices+1)
  int *d_roff = nullptr;       // null when every slice has Lz rows
  int *d_zhist = nullptr, *d_rowstart = nullptr, *d_cursor = nullptr;
  int2 *d_zstat = nullptr;
  unsigned long long *d_ymax = nullptr;
  int *d_extflag = nullptr;
  float *d_my = nullptr, *d_mz = nullptr;
  float4 *d_sconst = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_kernels = 0;
  bool executed = false;
  // d_iq64 holds the last execute's float64 I(q) (made on request)
  bool iq64_valid = false;
  gw_grad_state *grad = nullptr;  // adjoint workspace (gw_grad.cu)
};

namespace gwv {
SliceArgs slice_args(gw_voxel_plan *P);
// Structure preparation: extents reset, z sort, column tables.
int enqueue_prep(gw_voxel_plan *P);
// Per-slice min/max, extents and profiles of slices [s0, s0+n).
int enqueue_slice_setup(gw_voxel_plan *P, const SliceArgs &a, int s0, int n);
// Row transforms of the window rows of slices [s0, s0+n_sl), into d_F1.
int row_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 int s0, int n_sl);
// The pruned Stockham forms (window and band within M/2) for the batched
// lengths.
template <int M>
bool pruned(const CztArgs &cz) {
  return M <= 2048 && cz.L <= M / 2 && cz.N <= M / 2;
}
// Column transforms and binning of slices [s0, s0+n_sl) (gw_stockham_col.cu).
int col_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                 const BinArgs &bn, int s0, int n_sl);
// The F1 tensor map for the column kernels' tile loads (gw_stockham_col.cu).
int col_map_dispatch(gw_voxel_plan *P);
// Fused chirp-z kernels (gw_czt2_row.cu, gw_czt2_col.cu): lengths with a
// fused shape, the number of block shapes, their twiddle tables, and the
// launches for the plan's My / Mz.
bool fused_supported(int M);
int fused_variant_count();
std::vector<float2> fused_twiddles(int M);
int fused_row_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                       int s0, int n);
int fused_col_dispatch(gw_voxel_plan *P, const SliceArgs &a, const CztArgs &cz,
                       const BinArgs &bn, int s0, int n);
// Columns per block the fused column kernel will run with (the tensor map's
// box width).
int fused_col_block(const gw_voxel_plan *P);
// Average, crop and f0 factor into the float32 (f64 false) or the float64
// I(q) grids.
int enqueue_finalize(gw_voxel_plan *P, bool f64);
int enqueue_gather(gw_voxel_plan *P, int mode, int t, int line_lo = 0, int line_hi = -1);
// Number of window rows of slices [s0, s0+n).
int batch_rows(gw_voxel_plan *P, int s0, int n);
void grad_state_destroy(gw_grad_state *g);
}  // namespace gwv

#define GW_DISPATCH_M(M_, fn, ...)                                        \
  switch (M_) {                                                         \
    case 64: return fn<64>(__VA_ARGS__);                                \
    case 128: return fn<128>(__VA_ARGS__);                              \
    case 256: return fn<256>(__VA_ARGS__);                              \
    case 384: return fn<384>(__VA_ARGS__);                              \
    case 512: return fn<512>(__VA_ARGS__);                              \
    case 640: return fn<640>(__VA_ARGS__);                              \
    case 768: return fn<768>(__VA_ARGS__);                              \
    case 1024: return fn<1024>(__VA_ARGS__);                            \
    case 1280: return fn<1280>(__VA_ARGS__);                            \
    case 1536: return fn<1536>(__VA_ARGS__);                            \
    case 2048: return fn<2048>(__VA_ARGS__);                            \
    case 2560: return fn<2560>(__VA_ARGS__);                            \
    case 3072: return fn<3072>(__VA_ARGS__);                            \
    case 4096: return fn<4096>(__VA_ARGS__);                            \
    case 5120: return fn<5120>(__VA_ARGS__);                            \
    case 6144: return fn<6144>(__VA_ARGS__);                            \
    case 8192: return fn<8192>(__VA_ARGS__);                            \
    default: return gw::fail(GW_ERR_ARG, "unsupported FFT size");       \
  }
