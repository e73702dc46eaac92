// Slab construction on the device: tools/comparison.py:595-671
// (slabmaker_fitting).  A unit cell of n_cell atoms is replicated
// (nx+1) x (ny+1) x (nz+1) times along the cell vectors, shifted to the
// origin, cropped to the central x_size x y_size x z_size box and shifted to
// the origin again.  The result stays on the device, where the voxel stage
// can take it directly (gw_voxel_set_atoms with on_device).
//
// Bit-exact with the reference: every copy is made as the reference makes
// it, by float64 additions of the shift vectors axis by axis --
// ((p + (a_x i, 0, 0)) + (b_x j, b_y j, 0)) + (c_x k, c_y k, c_z k), each
// shift component a float64 product of a vector component and the copy
// number -- and the crop keeps the reference's atom order (a stable
// compaction).  Atom t of the replicated set is copy (k, j, i) of cell atom
// a with t = ((k (ny+1) + j)(nx+1) + i) n_cell + a, the order the
// reference's concatenations produce.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gw_common.cuh"

struct gw_slab {
  gw_ctx *ctx = nullptr;
  int64_t n = 0;            // atoms kept
  double bounds[3] = {0, 0, 0};
  double *d_xyz = nullptr;  // kept atoms, (n, 3)
  int *d_src = nullptr;     // cell atom of each kept atom
};

namespace {

constexpr int kSlabThreads = 256, kSlabItems = 4;
constexpr int kSlabChunk = kSlabThreads * kSlabItems;

struct SlabArgs {
  const double *cell;
  int n_cell;
  int nx1, ny1;        // copies along a and b (nx+1, ny+1)
  int64_t total;
  double ax, bx, by, cx, cy, cz;
};

__device__ __forceinline__ void slab_atom(const SlabArgs &s, int64_t t,
                                          double &x, double &y, double &z,
                                          int &a) {
  a = (int)(t % s.n_cell);
  int64_t r = t / s.n_cell;
  const int i = (int)(r % s.nx1);
  r /= s.nx1;
  const int j = (int)(r % s.ny1);
  const int k = (int)(r / s.ny1);
  x = s.cell[3 * a];
  y = s.cell[3 * a + 1];
  z = s.cell[3 * a + 2];
  // the copies add exact zeros too (which turn -0.0 into +0.0)
  if (i) {  // + (a_x i, 0, 0)
    x = GW_DADD(x, GW_DMUL(s.ax, (double)i));
    y = GW_DADD(y, 0.0);
    z = GW_DADD(z, 0.0);
  }
  if (j) {  // + (b_x j, b_y j, 0)
    x = GW_DADD(x, GW_DMUL(s.bx, (double)j));
    y = GW_DADD(y, GW_DMUL(s.by, (double)j));
    z = GW_DADD(z, 0.0);
  }
  if (k) {
    x = GW_DADD(x, GW_DMUL(s.cx, (double)k));
    y = GW_DADD(y, GW_DMUL(s.cy, (double)k));
    z = GW_DADD(z, GW_DMUL(s.cz, (double)k));
  }
}

// min and max of every axis over the replicated set
__global__ void k_slab_extents(SlabArgs s, unsigned long long *mn,
                               unsigned long long *mx) {
  unsigned long long lo[3] = {~0ULL, ~0ULL, ~0ULL}, hi[3] = {0, 0, 0};
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < s.total;
       t += (int64_t)gridDim.x * blockDim.x) {
    double p[3];
    int a;
    slab_atom(s, t, p[0], p[1], p[2], a);
    for (int c = 0; c < 3; ++c) {
      const unsigned long long v = dbl_ord(p[c]);
      lo[c] = min(lo[c], v);
      hi[c] = max(hi[c], v);
    }
  }
  for (int c = 0; c < 3; ++c) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(mn + c, lo[c]);
      atomicMax(mx + c, hi[c]);
    }
  }
}

struct CropArgs {
  double mn[3];   // minima of the replicated set (first shift)
  double lo[3];   // buffers (ext - size)/2
  double hi[3];   // ext - buffer
};

__device__ __forceinline__ bool slab_keep(const SlabArgs &s, const CropArgs &c,
                                          int64_t t, double p[3], int &a) {
  slab_atom(s, t, p[0], p[1], p[2], a);
  bool keep = true;
  for (int k = 0; k < 3; ++k) {
    p[k] = GW_DSUB(p[k], c.mn[k]);
    keep = keep && p[k] >= c.lo[k] && p[k] <= c.hi[k];
  }
  return keep;
}

// kept atoms per chunk of kSlabChunk consecutive atoms
__global__ void __launch_bounds__(kSlabThreads)
k_slab_count(SlabArgs s, CropArgs c, int *chunk_count) {
  __shared__ int warp_n[kSlabThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kSlabChunk;
  int n = 0;
  for (int it = 0; it < kSlabItems; ++it) {
    const int64_t t = base + it * kSlabThreads + threadIdx.x;
    double p[3];
    int a;
    if (t < s.total && slab_keep(s, c, t, p, a)) ++n;
  }
  n = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < kSlabThreads / 32; ++w) tot += warp_n[w];
    chunk_count[blockIdx.x] = tot;
  }
}

// exclusive scan of the chunk counts in place (one block); total at [n]
__global__ void __launch_bounds__(1024) k_slab_scan(int *cnt, int n) {
  __shared__ int part[1024];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  int local = 0;
  for (int k = 0; k < per; ++k)
    if (b0 + k < n) local += cnt[b0 + k];
  part[threadIdx.x] = local;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - local;
  for (int k = 0; k < per; ++k)
    if (b0 + k < n) {
      const int v = cnt[b0 + k];
      cnt[b0 + k] = run;
      run += v;
    }
  if (threadIdx.x == blockDim.x - 1) cnt[n] = part[threadIdx.x];
}

// stable compaction of the kept atoms (coordinates after the first shift),
// with the minima and maxima of what is kept
__global__ void __launch_bounds__(kSlabThreads)
k_slab_scatter(SlabArgs s, CropArgs c, const int *chunk_off, double *xyz,
               int *src, unsigned long long *kmn, unsigned long long *kmx) {
  __shared__ int warp_base[kSlabThreads / 32 + 1];
  const int64_t base = (int64_t)blockIdx.x * kSlabChunk;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int out = chunk_off[blockIdx.x];
  unsigned long long lo[3] = {~0ULL, ~0ULL, ~0ULL}, hi[3] = {0, 0, 0};
  for (int it = 0; it < kSlabItems; ++it) {
    const int64_t t = base + it * kSlabThreads + threadIdx.x;
    double p[3];
    int a = 0;
    const bool keep = t < s.total && slab_keep(s, c, t, p, a);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_base[wid] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int run = 0;
      for (int w = 0; w < kSlabThreads / 32; ++w) {
        const int v = warp_base[w];
        warp_base[w] = run;
        run += v;
      }
      warp_base[kSlabThreads / 32] = run;
    }
    __syncthreads();
    if (keep) {
      const int64_t o = out + warp_base[wid] + __popc(m & ((1u << lane) - 1u));
      xyz[3 * o] = p[0];
      xyz[3 * o + 1] = p[1];
      xyz[3 * o + 2] = p[2];
      src[o] = a;
      for (int k = 0; k < 3; ++k) {
        lo[k] = min(lo[k], dbl_ord(p[k]));
        hi[k] = max(hi[k], dbl_ord(p[k]));
      }
    }
    out += warp_base[kSlabThreads / 32];
    __syncthreads();
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
    if (lane == 0) {
      atomicMin(kmn + k, lo[k]);
      atomicMax(kmx + k, hi[k]);
    }
  }
}

// second shift to the origin
__global__ void k_slab_shift(double *xyz, int64_t n, double m0, double m1,
                             double m2) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    xyz[3 * t] = GW_DSUB(xyz[3 * t], m0);
    xyz[3 * t + 1] = GW_DSUB(xyz[3 * t + 1], m1);
    xyz[3 * t + 2] = GW_DSUB(xyz[3 * t + 2], m2);
  }
}

}  // namespace

extern "C" int gw_slab_destroy(gw_slab *S) {
  if (!S) return GW_OK;
  gw::dev_free(S->d_xyz);
  gw::dev_free(S->d_src);
  delete S;
  return GW_OK;
}

extern "C" int gw_slab_create(gw_ctx *ctx, const double *cell_xyz,
                              int32_t n_cell, const double *vecs,
                              const double *size, gw_slab **out) {
  if (!ctx || !cell_xyz || !vecs || !size || !out || n_cell < 1)
    return gw::fail(GW_ERR_ARG, "gw_slab_create: invalid argument");
  GW_CUDA(cudaSetDevice(ctx->device));
  // replication numbers (comparison.py:608-610)
  const double av0 = vecs[0], bv0 = vecs[3], bv1 = vecs[4];
  const double cv0 = vecs[6], cv1 = vecs[7], cv2 = vecs[8];
  if (!(av0 > 0) || !(bv1 > 0) || !(cv2 > 0))
    return gw::fail(GW_ERR_ARG, "gw_slab_create: cell vectors must have a_x, b_y, c_z > 0");
  const double nxd = std::ceil(2 * size[0] / av0), nyd = std::ceil(2 * size[1] / bv1),
               nzd = std::ceil(2 * size[2] / cv2);
  const double total_d = (nxd + 1) * (nyd + 1) * (nzd + 1) * (double)n_cell;
  if (!(nxd >= 0 && nyd >= 0 && nzd >= 0) || total_d > 1.5e9)
    return gw::fail(GW_ERR_ARG, "gw_slab_create: slab too large or negative size");
  SlabArgs s{};
  s.n_cell = n_cell;
  s.nx1 = (int)nxd + 1;
  s.ny1 = (int)nyd + 1;
  s.total = (int64_t)total_d;
  s.ax = av0; s.bx = bv0; s.by = bv1; s.cx = cv0; s.cy = cv1; s.cz = cv2;
  const int64_t nchunk = (s.total + kSlabChunk - 1) / kSlabChunk;
  if (nchunk > (1 << 30))
    return gw::fail(GW_ERR_ARG, "gw_slab_create: slab too large");

  cudaStream_t st = ctx->stream;
  double *d_cell = nullptr;
  unsigned long long *d_ord = nullptr;  // mn[3], mx[3], kmn[3], kmx[3]
  int *d_cnt = nullptr;
  auto *S = new gw_slab();
  S->ctx = ctx;
  int status = GW_OK;
  cudaError_t e = gw::dev_malloc((void **)&d_cell, (size_t)n_cell * 3 * sizeof(double));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_ord, 12 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = gw::dev_malloc((void **)&d_cnt, (size_t)(nchunk + 1) * sizeof(int));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_cell, cell_xyz, (size_t)n_cell * 3 * sizeof(double),
                        cudaMemcpyHostToDevice, st);
  unsigned long long h_ord[12];
  for (int k = 0; k < 3; ++k) {
    h_ord[k] = ~0ULL; h_ord[3 + k] = 0ULL; h_ord[6 + k] = ~0ULL; h_ord[9 + k] = 0ULL;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_ord, h_ord, sizeof h_ord, cudaMemcpyHostToDevice, st);
  const int gblocks = (int)std::min<int64_t>((s.total + 255) / 256, 8 * ctx->sm_count);
  if (e == cudaSuccess) {
    s.cell = d_cell;
    k_slab_extents<<<gblocks, 256, 0, st>>>(s, d_ord, d_ord + 3);
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_ord, d_ord, sizeof h_ord, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  CropArgs c{};
  if (e == cudaSuccess) {
    const char *msg[3] = {"x_max must be greater than x_size",
                          "y_max must be greater than y_size",
                          "z_max must be greater than z_size"};
    for (int k = 0; k < 3 && status == GW_OK; ++k) {
      const double mn = ord_dbl(h_ord[k]), mx = ord_dbl(h_ord[3 + k]);
      const double ext = mx - mn;  // comparison.py:639-641
      if (!(ext > size[k])) status = gw::fail(GW_ERR_ARG, msg[k]);
      const double buf = (ext - size[k]) / 2;  // comparison.py:649-651
      c.mn[k] = mn;
      c.lo[k] = buf;
      c.hi[k] = ext - buf;
    }
  }
  if (e == cudaSuccess && status == GW_OK) {
    k_slab_count<<<(unsigned)nchunk, kSlabThreads, 0, st>>>(s, c, d_cnt);
    ctx->launches++;
    k_slab_scan<<<1, 1024, 0, st>>>(d_cnt, (int)nchunk);
    ctx->launches++;
    e = cudaGetLastError();
    int kept = 0;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&kept, d_cnt + nchunk, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && kept < 1) status = gw::fail(GW_ERR_ARG, "gw_slab_create: the crop keeps no atom");
    if (e == cudaSuccess && status == GW_OK) {
      S->n = kept;
      e = gw::dev_malloc((void **)&S->d_xyz, (size_t)kept * 3 * sizeof(double));
      if (e == cudaSuccess) e = gw::dev_malloc((void **)&S->d_src, (size_t)kept * sizeof(int));
      if (e == cudaSuccess) {
        k_slab_scatter<<<(unsigned)nchunk, kSlabThreads, 0, st>>>(
            s, c, d_cnt, S->d_xyz, S->d_src, d_ord + 6, d_ord + 9);
        ctx->launches++;
        e = cudaGetLastError();
      }
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_ord, d_ord, sizeof h_ord, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e == cudaSuccess) {
        double m[3];
        for (int k = 0; k < 3; ++k) {
          m[k] = ord_dbl(h_ord[6 + k]);
          // extent of the final coordinates: max(c - m) - min(c - m)
          S->bounds[k] = ord_dbl(h_ord[9 + k]) - m[k];
        }
        const int sb = (int)std::min<int64_t>((kept + 255) / 256, 8 * ctx->sm_count);
        k_slab_shift<<<sb, 256, 0, st>>>(S->d_xyz, kept, m[0], m[1], m[2]);
        ctx->launches++;
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
  }
  gw::dev_free(d_cell);
  gw::dev_free(d_ord);
  gw::dev_free(d_cnt);
  if (e != cudaSuccess) status = gw::cuda_fail(e, "gw_slab_create", __FILE__, __LINE__);
  if (status != GW_OK) {
    gw_slab_destroy(S);
    return status;
  }
  *out = S;
  return GW_OK;
}

extern "C" int gw_slab_info(gw_slab *S, int64_t *n, double *bounds) {
  if (!S || !n) return gw::fail(GW_ERR_ARG, "gw_slab_info: null argument");
  *n = S->n;
  if (bounds)
    for (int k = 0; k < 3; ++k) bounds[k] = S->bounds[k];
  return GW_OK;
}

extern "C" int gw_slab_get(gw_slab *S, double *xyz, int32_t *src,
                           int32_t on_device) {
  if (!S || !xyz) return gw::fail(GW_ERR_ARG, "gw_slab_get: null argument");
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  GW_CUDA(cudaMemcpyAsync(xyz, S->d_xyz, (size_t)S->n * 3 * sizeof(double), k, S->ctx->stream));
  if (src)
    GW_CUDA(cudaMemcpyAsync(src, S->d_src, (size_t)S->n * sizeof(int), k, S->ctx->stream));
  GW_CUDA(cudaStreamSynchronize(S->ctx->stream));
  return GW_OK;
}

extern "C" int gw_slab_device_xyz(gw_slab *S, const double **xyz) {
  if (!S || !xyz) return gw::fail(GW_ERR_ARG, "gw_slab_device_xyz: null argument");
  *xyz = S->d_xyz;
  return GW_OK;
}
