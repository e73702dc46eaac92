/*
 * giwaxs_gb300.h -- C ABI of the GB300 (sm_103a) GIWAXS forward path.
 *
 * The reference (tchaney97/giwaxsim) is pure Python/numpy; its hot path is
 * reached through these Python entry points, which this library replaces:
 *
 *   tools/comparison.py:673  voxelgridmaker_fitting(...)  -> gw_voxel_*
 *   tools/voxelgrids.py:311  rotate_project_fft_coords(args)  (per slice)
 *   tools/voxelgrids.py:464  process_file2(...)               (binning)
 *   tools/comparison.py:790  detectormaker_fitting(...)   -> gw_detector_*
 *   tools/detector.py:278    generate_detector_ints(args)     (per orientation)
 *   tools/detector.py:194    intersect_detector(...)
 *
 * A reference-side binding is plain ctypes; the package
 * giwaxsim_gb300.tools.* is that binding, with the reference's signatures.
 * All entry points return a gw_status; gw_last_error() gives the message of
 * the last failure on the calling thread.  Pointers are plain
 * host or device addresses; a flag says which.  No call allocates pinned
 * host memory or keeps host pointers after it returns.
 *
 * Threading: a gw_ctx owns one CUDA stream; calls on one context must not
 * overlap.  Different contexts may be used from different threads.
 */
#ifndef GIWAXS_GB300_H
#define GIWAXS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ------------------------------------------------------------ */
enum gw_status {
  GW_OK = 0,
  GW_ERR_ARG = 1,     /* invalid argument; message names it                */
  GW_ERR_OOM = 2,     /* device allocation failed (or GW_FAIL_ALLOC_AFTER)  */
  GW_ERR_CUDA = 3,    /* a CUDA runtime call failed                         */
  GW_ERR_TIMEOUT = 4, /* a bounded device wait ran out                      */
  GW_ERR_BOUNDS = 5,  /* a device-side range check failed                   */
  GW_ERR_STATE = 6    /* call out of order (e.g. execute before set_atoms)  */
};

int gw_version(void);
const char *gw_status_string(int status);
/* Copies the calling thread's last error message (NUL-terminated, truncated
 * to len-1).  Returns the full message length. */
size_t gw_last_error(char *buf, size_t len);
/* Allocation-failure injection, a test hook with no counterpart in the
 * reference: from this call on, the (after+1)-th device allocation the
 * library makes and every later one fail with GW_ERR_OOM, as if the device
 * were out of memory (after < 0 turns it off).  The environment variable
 * GW_FAIL_ALLOC_AFTER=n does the same counting from process start. */
int gw_set_alloc_fault(int64_t after);
/* Page-lock an existing host buffer (cudaHostRegister) so that the copies of
 * results into it and of inputs from it run at the link's speed, and release
 * it again (before the buffer is freed).  No counterpart in the reference
 * (its results are numpy arrays on the host).  GW_ERR_CUDA when the driver
 * refuses (the buffer stays usable, unpinned). */
int gw_host_pin(void *ptr, uint64_t bytes);
int gw_host_unpin(void *ptr);

/* ---- context ----------------------------------------------------------- */
typedef struct gw_ctx gw_ctx;
int gw_ctx_create(int device, gw_ctx **out);
int gw_ctx_destroy(gw_ctx *ctx);
int gw_ctx_synchronize(gw_ctx *ctx);
/* The context's cudaStream_t, for callers that order their own work. */
int gw_ctx_stream(gw_ctx *ctx, void **stream);
/* Number of kernels this library launched on the context so far (graph
 * replays count the kernels inside the graph). */
int64_t gw_ctx_launch_count(gw_ctx *ctx);
/* "<device name> sm_XY xN" of the context's device (keys tuning caches). */
int gw_ctx_device_name(gw_ctx *ctx, char *buf, size_t n);
/* Device-side stopwatch on the context stream: record mark 0 and mark 1
 * (gw_ctx_mark), then gw_ctx_elapsed_ms waits for mark 1 and returns the
 * time between them. */
int gw_ctx_mark(gw_ctx *ctx, int32_t slot);
int gw_ctx_elapsed_ms(gw_ctx *ctx, float *ms);

/* Per-kernel device timing.  When on, every kernel launch of the library on
 * this context is bracketed by CUDA events on the context stream (eager
 * execution only; graph replays are not instrumented).  gw_ctx_kernel_times
 * synchronises, then fills total milliseconds and launch counts per kernel
 * category (names from gw_kernel_category_name) and returns the number of
 * categories; the totals accumulate until timing is switched on again. */
int gw_ctx_set_timing(gw_ctx *ctx, int32_t on);
int gw_ctx_kernel_times(gw_ctx *ctx, double *ms, int64_t *launches,
                        int32_t n);
const char *gw_kernel_category_name(int32_t category);

/* ---- host helpers ------------------------------------------------------ */
/* out[k*3+i] = fma(p2,R[i][2], fma(p1,R[i][1], p0*R[i][0])): the fused
 * order OpenBLAS uses for np.dot(coords, R.T) (tools/utilities.py:315) and
 * R @ vstack (tools/detector.py:71).  R row-major 3x3, pts (n,3). */
int gw_rotate_points(const double *R, const double *pts, int64_t n,
                     double *out);
/* rectangular_collapse_lengths' per-slice constant
 * sqrt(ver**2 - (ver*cos_t)**2) (tools/voxelgrids.py:292) with the host
 * libm pow(), which is what numpy's scalar ** calls. */
int gw_collapse_base(const double *ver, const double *cos_t, int64_t n,
                     double *out);

/* ---- voxel stage: I(qx,qy,qz) from atoms ----------------------------- */
enum { GW_VOXEL_BATCHED = 0, GW_VOXEL_PLAIN = 1 };
enum { GW_ACCUM_FP64 = 0, GW_ACCUM_KAHAN32 = 1 };
enum { GW_STRUCTS_SUM = 0, GW_STRUCTS_AVERAGE = 1, GW_STRUCTS_SEPARATE = 2 };
enum { GW_DEPOSIT_NEAREST = 0, GW_DEPOSIT_BILINEAR = 1 };
enum { GW_SHELLS_PER_SHELL = 1, GW_SHELLS_REFERENCE = 2 };

enum { GW_TRANSFORM_AUTO = 0, GW_TRANSFORM_STOCKHAM = 1, GW_TRANSFORM_FUSED = 2 };

enum { GW_BINNING_AUTO = 0, GW_BINNING_ATOMIC = 1, GW_BINNING_GATHER = 2 };

typedef struct gw_voxel_params {
  int32_t grid_size;    /* g = ceil(2pi/(dq*r))          comparison.py:710 */
  double r_voxel_size;  /* r                                               */
  int32_t q_num;        /* length of the full q axis     comparison.py:721 */
  double q_min, q_max;  /* first / last value of the full axis             */
  double dq;            /* np.diff(qz)[0]                voxelgrids.py:496 */
  int32_t crop_lo, crop_hi; /* inclusive index range kept by
                               downselect_voxelgrid      voxelgrids.py:16  */
  double h_max;         /* max(fftshift(fftfreq(g,r))*2pi) voxelgrids.py:396 */
  int32_t fill_bkg;     /*                               voxelgrids.py:350 */
  double smooth;        /* sigma in r-voxels, 0 = off    voxelgrids.py:364 */
  int32_t mode;         /* GW_VOXEL_BATCHED | GW_VOXEL_PLAIN               */
  int32_t accum;        /* GW_ACCUM_FP64 | GW_ACCUM_KAHAN32                */
  int32_t average;      /* GW_STRUCTS_AVERAGE: one I(q) averaged over the
                           structures (old_modules/voxelgridmaker.py:56-61);
                           GW_STRUCTS_SUM: their sum; GW_STRUCTS_SEPARATE:
                           one I(q) per structure, concatenated (candidates
                           of a fit evaluated in one pass)                 */
  double f0_coef[9];    /* Cromer-Mann a1,b1,..,a4,b4,c  voxelgrids.py:849 */
  double f0_z;          /* Z of the f0 element; <= 0 skips the f0 factor   */
  int32_t batch_slices; /* slices per batch, 0 = automatic                 */
  int32_t deposit;      /* GW_DEPOSIT_NEAREST (the reference's np.add.at of
                           floor-divided indices, voxelgrids.py:328-341) |
                           GW_DEPOSIT_BILINEAR (each atom split over two
                           rows x two columns; differentiable in the
                           coordinates; no counterpart in the reference)    */
  int32_t fft_y, fft_z; /* chirp-z convolution lengths along y and z: 0 =
                           the smallest supported length >= L+N-1; else one
                           of 2^k, 3*2^k, 5*2^k in [64, 8192] and >= L+N-1 */
  int32_t transform_y, transform_z; /* kernel family of the row (y) and
                           column (z) chirp-z transforms.
                           GW_TRANSFORM_AUTO and GW_TRANSFORM_STOCKHAM: the
                           Stockham kernels (measured the faster family on
                           GB300); GW_TRANSFORM_FUSED: the fused kernel (two
                           shared-memory exchanges per convolution;
                           GW_ERR_ARG if the length has no fused shape)    */
  int32_t block_variant; /* block shape of the fused kernels (sequences per
                           block, register cap), 0 .. count-1 with the count
                           from gw_voxel_block_variants(); an autotuner
                           picks it by timing; 0 = the default shape       */
  int32_t real_grids;   /* 1: the caller states that every structure's
                           atom f values are real multiples of one complex
                           value (one element; real occupancies), so each
                           slice grid is that phase times a real grid: two
                           window rows share one row transform and only the
                           columns ky >= 0 are transformed (|F|^2 has the
                           symmetry F(-k) = conj F(k) of a real grid); the
                           bands are made symmetric.  Used in batched,
                           nearest-bin plans with the Stockham kernels (not
                           with GW_TRANSFORM_FUSED) when the window fits
                           half a transform buffer; no shells, no backward.
                           gw_voxel_info reports whether it runs.  0: the
                           general path.                                   */
  int32_t binning;      /* how |F|^2 pixels reach the voxel sums.
                           GW_BINNING_ATOMIC: float64 atomic adds as the
                           column transforms produce them (the sum's
                           rounding depends on arrival order);
                           GW_BINNING_GATHER: the column transforms store
                           every slice's pixels, then one pass per voxel
                           line adds its pixels in a fixed order
                           (compensated float32) and finalizes: no atomics,
                           bit-identical results run to run (batched plans
                           with float64 accumulation; GW_ERR_ARG
                           otherwise, or when the pixel store would exceed
                           the device budget); GW_BINNING_AUTO: gather for
                           one structure on real grids whose float64 sum
                           grid is larger than the L2 cache (the atomics
                           would go to DRAM), atomic otherwise.  Multi-q
                           shells always bin atomically.                   */
} gw_voxel_params;

typedef struct gw_structure {
  int64_t atom_begin, atom_count; /* slice of the atom arrays            */
  double x_bound, y_bound, z_bound; /* max-min per axis comparison.py:712 */
  double avg_f_re, avg_f_im;      /* avg_voxel_f      comparison.py:744   */
  double max_voxels;              /* sqrt(xb**2+yb**2)//r voxelgrids.py:344 */
} gw_structure;

typedef struct gw_phi {
  double cos_phi, sin_phi;   /* np.cos/np.sin(np.radians(phi))  utilities.py:305-312 */
  double right_qy, right_qx; /* slice h-axis end points       voxelgrids.py:396-399 */
  /* rectangular_collapse_lengths (voxelgrids.py:253-285) after the phi>90
   * fold: case 0 (phi'==0), 1 (phi'==90), 2 (general); swap = phi>90. */
  int32_t cl_case, cl_swap;
  double cos_t, sin_t, tan_t; /* of theta' = 90 - phi' (radians) */
  double cos_p, sin_p, tan_p; /* of phi' (radians)               */
} gw_phi;

typedef struct gw_voxel_plan gw_voxel_plan;

/* Build a plan for n_struct structures x n_phi rotations.  All tables that
 * depend only on sizes (CZT chirps, twiddles) are made here. */
int gw_voxel_plan_create(gw_ctx *ctx, const gw_voxel_params *p,
                         const gw_structure *structs, int32_t n_struct,
                         const gw_phi *phis, int32_t n_phi,
                         gw_voxel_plan **out);
int gw_voxel_plan_destroy(gw_voxel_plan *plan);
/* Atoms: xyz (n,3) float64, f (n,2) float32 complex scattering factor
 * (Z + f' + i f'', times any per-atom weight).  on_device: 0 host, 1 device
 * (device pointers are copied into the plan). */
int gw_voxel_set_atoms(gw_voxel_plan *plan, const double *xyz, const float *f,
                       int64_t n_atoms, int32_t on_device);
/* Multi-q atomic form factors (voxelgrids.py:650-707, aff_num_qs > 1).
 * Shell k holds the voxels with lower[k] < |q| <= upper[k], |q| taken from
 * q_axis (the full q axis, q_num values) as numpy's meshgrid sum does; f is
 * n_shells x n_atoms complex float32 (f0(q_k) + f' + i f'' per atom) and
 * avg_f n_shells x n_struct complex float64 (avg_voxel_f per shell).
 *   GW_SHELLS_PER_SHELL  one pass per shell, each voxel's I(q) from the
 *                        pass of its own shell (of both shells for a voxel
 *                        on a rounding boundary), voxels in no shell 0;
 *   GW_SHELLS_REFERENCE  what the reference returns: the last shell's pass
 *                        over every voxel, doubled inside the last shell
 *                        (voxelgrids.py:703-707 overwrite the grid each
 *                        shell and add the masked grid to itself).
 * Call after gw_voxel_set_atoms; n_shells = 0 clears the shells (the atoms
 * must then be set again: the passes overwrite the plan's copy of f).
 * Shells must increase, and shell k + 2 must start at or above the end of
 * shell k. */
int gw_voxel_set_shells(gw_voxel_plan *plan, int32_t n_shells, int32_t mode,
                        const double *q_axis, const double *lower,
                        const double *upper, const float *f,
                        const double *avg_f);
/* Enqueue the whole forward chain on the context stream (a CUDA graph
 * replay when gw_voxel_capture_graph succeeded). */
int gw_voxel_execute(gw_voxel_plan *plan);
int gw_voxel_capture_graph(gw_voxel_plan *plan);
/* Poll limit of the column kernel's bounded wait for its tile load
 * (default 4194304 polls, far beyond a load's latency).  When a wait runs
 * out the block records GW_ERR_TIMEOUT in the context's device error word
 * (reported by the next gw_ctx_synchronize or result call), waits again
 * with the default limit for the load in flight, and bins nothing; the
 * context stays usable.  0 makes every wait run out at once (a test hook
 * for that path).  Drops a captured graph.  No counterpart in the
 * reference (a bounded wait of this library's own). */
int gw_voxel_set_wait_limit(gw_voxel_plan *plan, uint32_t polls);
/* Number of block shapes of the fused chirp-z kernels (valid
 * gw_voxel_params.block_variant values are 0 .. count-1). */
int32_t gw_voxel_block_variants(void);
/* Results (synchronous).  iq: crop^3 float64, C order (qy,qx,qz); in
 * GW_STRUCTS_SEPARATE mode n_struct such grids back to back.
 * on_device: write to a device pointer instead of host memory. */
int gw_voxel_get_iq(gw_voxel_plan *plan, double *iq, int32_t on_device);
/* Device pointer to the float32 copy of I(q) the detector gathers from
 * (of structure `structure` in GW_STRUCTS_SEPARATE mode, else 0).  Each
 * grid starts 16-byte aligned. */
int gw_voxel_device_iq32(gw_voxel_plan *plan, int32_t structure,
                         const float **iq32);
/* Parity hooks: the cropped count and sum grids (float64, crop^3). */
int gw_voxel_get_counts(gw_voxel_plan *plan, double *counts);
int gw_voxel_get_sums(gw_voxel_plan *plan, double *sums);
/* Plan sizes, in this order: [crop, batch, Ly, Lz, Nc, Nr, My, Mz, y_lo,
 * z_lo, k0, kz0, n_slices, device_bytes, graph_kernels, col_tma (1 when
 * the column kernel loads its tiles by TMA), fused_y, fused_z (1 when the
 * fused chirp-z kernel runs along that axis), real (1 when the real-grid
 * path runs), gather (1 when the gather binning runs), heavy_lines (gather:
 * window lines summed by a whole block each), multi_rows (gather: window z
 * with more than one output row)].  Returns the number written (at most
 * n). */
int gw_voxel_info(gw_voxel_plan *plan, int64_t *info, int32_t n);
/* Deposit indices of one slice (after execute): y,z voxel index per atom of
 * that slice's structure, -1 where the reference's valid_mask drops it
 * (voxelgrids.py:328-335). */
int gw_voxel_debug_deposit(gw_voxel_plan *plan, int32_t slice, int32_t *y_idx,
                           int32_t *z_idx);
/* Parity hook: the deposited window of one slice before fill/smoothing,
 * complex64 (Lz, Ly) (row z_lo+zz, column y_lo+yy of the grid, cyclic):
 * np.add.at(grid[z, y], f) of voxelgrids.py:341 restricted to the window. */
int gw_voxel_debug_window(gw_voxel_plan *plan, int32_t slice, float *window);
/* The float32 I(q) the detector gathers from (crop^3 per structure, host). */
int gw_voxel_get_iq32(gw_voxel_plan *plan, float *iq32);
/* One-shot: plan, upload, execute, download, destroy (host buffers). */
int gw_voxelgrid(gw_ctx *ctx, const gw_voxel_params *p,
                 const gw_structure *structs, int32_t n_struct,
                 const gw_phi *phis, int32_t n_phi, const double *xyz,
                 const float *f, int64_t n_atoms, double *iq_out);

/* ---- detector stage ---------------------------------------------------- */
typedef struct gw_detector_params {
  int32_t n_h, n_v;         /* pixels (horizontal, vertical)             */
  int32_t iq_shape[3];      /* (ny, nx, nz) of the I(q) grid              */
  double qmin_x, qmin_y, qmin_z; /* np.min(qx), np.min(qy), np.min(qz)   */
  double dq;                /* np.diff(qz)[0]           detector.py:213   */
  int32_t mirror;           /* mirror_vertical_horizontal  comparison.py:857 */
  int32_t accum;            /* GW_ACCUM_FP64 | GW_ACCUM_KAHAN32           */
  int32_t exact;            /* 1: replay the float64 chain for every sample;
                               0: float32 fast path with exact replay of the
                               samples whose voxel it cannot decide        */
  int32_t no_plane;         /* 1: never use the plane gather (taken by the
                               fast path when every orientation keeps one
                               axis at a fixed index); same image either way */
  int32_t reserved[4];
} gw_detector_params;

typedef struct gw_detector_plan gw_detector_plan;

/* h_axis (n_h) and v_axis (n_v): make_detector's linspaces
 * (detector.py:24-25).  init_R: n_init 3x3 row-major matrices applied in
 * order to the plane (comparison.py:799-818).  Per orientation o,
 * n_rot[o] matrices (0..3, identity ones omitted) follow one another in
 * rot_R, and weights[o] = psi_w*phi_w*theta_w (detector.py:292). */
int gw_detector_plan_create(gw_ctx *ctx, const gw_detector_params *p,
                            const double *h_axis, const double *v_axis,
                            const double *init_R, int32_t n_init,
                            const int32_t *n_rot, const double *rot_R,
                            const double *weights, int32_t n_orient,
                            gw_detector_plan **out);
int gw_detector_plan_destroy(gw_detector_plan *plan);
/* I(q) to sample: float64 host or device array (converted to float32 on
 * the device), or a float32 device array used in place (gw_voxel_device_iq32). */
int gw_detector_set_iq(gw_detector_plan *plan, const double *iq,
                       int32_t on_device);
int gw_detector_set_iq32_device(gw_detector_plan *plan, const float *iq32);
int gw_detector_execute(gw_detector_plan *plan);
/* (n_v, n_h) float64 image after the epilogue (comparison.py:857-868). */
int gw_detector_get(gw_detector_plan *plan, double *out, int32_t on_device);
/* Device address of the plan's image (n_v, n_h) float64, valid until the
 * plan is destroyed and rewritten by every execute. */
int gw_detector_device_out(gw_detector_plan *plan, const double **out);
/* Flat (y*nx+x)*nz+z voxel index each pixel gathers for orientation o. */
int gw_detector_debug_indices(gw_detector_plan *plan, int32_t orient,
                              int64_t *flat_idx);
/* Allocation-free detector image; no counterpart in the reference.  For
 * callers that cannot allocate device memory when they need an image (their
 * memory budget is reserved up front, or a cudaMalloc/cudaFree stall or
 * failure mid-loop is not acceptable).  Every pointer is caller-owned device
 * memory: iq32 float32 (ny*nx*nz), h_axis/v_axis float64, init_R n_init
 * 3x3 matrices, n_rot int32 per orientation (0..3; the kernel reads counts
 * outside that range as the nearest of 0 and 3) with rot_R holding at least
 * the sum of the counts' matrices (9 doubles each; a shorter rot_R is read
 * past its end), weights float64 per orientation, out float64
 * (n_v, n_h).  Work is enqueued on `stream` (a cudaStream_t of the current
 * device) and not waited for.  The only scratch is a fixed 8 MiB float64
 * image inside the library, so images are limited to 1024 x 1024 pixels
 * (GW_ERR_ARG beyond).  The scratch is shared by all calls on a device:
 * calls that overlap on the GPU race, so serialise them.  The first call on
 * a device looks up the scratch address (cudaGetSymbolAddress); make that
 * first call before any stream capture. */
int gw_detector_noalloc(const gw_detector_params *p, const float *iq32,
                        const double *h_axis, const double *v_axis,
                        const double *init_R, int32_t n_init,
                        const int32_t *n_rot, const double *rot_R,
                        const double *weights, int32_t n_orient, double *out,
                        void *stream);
/* ---- adjoints (vector-Jacobian products) -------------------------------
 * No counterpart in the reference, which has no gradients; they give the
 * gradient of a scalar misfit of the detector image (the scale + flat
 * background least squares of tools/comparison.py:873-882 is one) with
 * respect to the inputs of the forward path.  Complex gradients are
 * dL/dRe + i dL/dIm.
 *
 * Detector: g_out is dL/d(image returned by gw_detector_get), (n_v, n_h)
 * float64; g_iq receives dL/dI(q) (ny*nx*nz float64).  The plan must have
 * been executed on the I(q) the gradient is taken at (the clamp of the
 * epilogue is evaluated on that image).  Synchronous. */
int gw_detector_backward(gw_detector_plan *plan, const double *g_out,
                         int32_t out_on_device, double *g_iq,
                         int32_t iq_on_device);
/* Voxel stage (batched mode, fill_bkg off): g_iq is dL/dI(q) on the
 * cropped cube (Qc^3 float64, host or device).  Every slice is recomputed
 * from the atoms set on the plan, one batch at a time (nothing per slice is
 * kept from the forward).  Outputs (host):
 *   g_f      n_atoms x 2: dL/d f of every atom's deposited scattering factor
 *            (input order), the constants of the structures held fixed;
 *   g_xyz    n_atoms x 3 or NULL: dL/d coordinates (GW_DEPOSIT_BILINEAR
 *            only), including the shift of every slice to its minimum
 *            rotated y and of the z axis to the minimum z;
 *   g_sigma  1 or NULL: dL/d smooth (sigma in voxels; plateau bounds and the
 *            kernel radius are piecewise constant and contribute nothing);
 *   g_c      n_struct x 2 or NULL: dL/d of each structure's background
 *            constant avg_voxel_f * max_voxels (smoothing on; else 0).
 * Synchronous. */
int gw_voxel_backward(gw_voxel_plan *plan, const double *g_iq,
                      int32_t iq_on_device, double *g_f, double *g_xyz,
                      double *g_sigma, double *g_c);
/* Plan-owned device buffer (Qc^3 float64) for dL/dI(q), so that the
 * detector adjoint can write it and gw_voxel_backward read it without a
 * host round trip.  Valid until the plan is destroyed. */
int gw_voxel_grad_buffer(gw_voxel_plan *plan, double **g_iq_dev);
/* One-shot with host buffers. */
int gw_detector(gw_ctx *ctx, const gw_detector_params *p, const double *iq,
                const double *h_axis, const double *v_axis,
                const double *init_R, int32_t n_init, const int32_t *n_rot,
                const double *rot_R, const double *weights, int32_t n_orient,
                double *out);

/* ---- slab construction (tools/comparison.py:595-671 slabmaker_fitting) -- */
/* A unit cell of n_cell atoms (cell_xyz, (n_cell, 3) float64 host) is
 * replicated along the cell vectors vecs = (a, b, c) (3x3 row-major, from
 * calc_real_space_abc; a_y = a_z = b_z = 0 as there), shifted to the origin,
 * cropped to the central size[0] x size[1] x size[2] box and shifted again,
 * bit for bit as the reference does it and in its atom order.  The result
 * stays on the device.  GW_ERR_ARG with the reference's message ("x_max
 * must be greater than x_size", ...) when the replicated slab is too small. */
typedef struct gw_slab gw_slab;
int gw_slab_create(gw_ctx *ctx, const double *cell_xyz, int32_t n_cell,
                   const double *vecs, const double *size, gw_slab **out);
int gw_slab_destroy(gw_slab *slab);
/* Number of atoms kept and their x/y/z extents (max - min per axis). */
int gw_slab_info(gw_slab *slab, int64_t *n, double *bounds);
/* Copy out the (n, 3) float64 coordinates and, if src is not NULL, the cell
 * atom (0..n_cell-1) of each atom; host or device destination. */
int gw_slab_get(gw_slab *slab, double *xyz, int32_t *src, int32_t on_device);
/* Device address of the coordinates (valid until gw_slab_destroy), for
 * gw_voxel_set_atoms(..., on_device = 1). */
int gw_slab_device_xyz(gw_slab *slab, const double **xyz);

/* ---- experimental comparison (tools/comparison.py:161-191 trim_sim_data,
 * :406-445 rebin_qmap_and_mask, :873-882 optimize_scale_offset) ---------- */
/* The experimental map (n_src values and mask values) is rebinned onto the
 * rows x cols trimmed window [v0, v0+rows) x [h0, h0+cols) of an n_v x n_h
 * simulated image by the sparse weights idx/w (3 per target pixel, row-major
 * over the window; idx[3i] < 0 marks a pixel outside the triangulation:
 * NaN).  The mask is thresholded (> 0).  Made once per experiment. */
typedef struct gw_compare gw_compare;
int gw_compare_create(gw_ctx *ctx, int32_t n_v, int32_t n_h, int32_t v0,
                      int32_t h0, int32_t rows, int32_t cols,
                      const int32_t *idx, const double *w,
                      const double *exp_values, const double *exp_mask,
                      int64_t n_src, gw_compare **out);
int gw_compare_destroy(gw_compare *cmp);
/* The rebinned map (rows x cols float64) and mask (uint8) (host). */
int gw_compare_target(gw_compare *cmp, double *target, uint8_t *mask);
/* Least-squares scale and offset of the trimmed simulated image onto the
 * target over the unmasked pixels; out = (scale, offset, misfit = sum of
 * squared residuals, number of pixels used).  sim is the whole n_v x n_h
 * image (host, or device with sim_on_device).  residual (host rows x cols,
 * or NULL) receives target - (scale sim + offset), 0 where masked. */
int gw_compare_eval(gw_compare *cmp, const double *sim, int32_t sim_on_device,
                    double *out, double *residual);

/* shift_peak (tools/comparison.py:566-592: linear_polar, add_pad, the zero
 * mask, polar_linear) on a rows x cols trimmed image, as fixed maps:
 *   polar[j] = sum_k p_w[4j+k] image[p_idx[4j+k]]       (n_t x n_r polar)
 *   z[t][c]  = polar[t][c] == 0 ? 0 : polar[t][col_src[c]]
 *   out[i]   = sum_k q_w[4i+k] z[q_idx[4i+k]]
 * indices flat (row-major), -1 = unused.  The maps come from the host
 * (giwaxsim_gb300.tools.comparison.shift_peak_maps). */
typedef struct gw_warp gw_warp;
int gw_warp_create(gw_ctx *ctx, int32_t rows, int32_t cols, int32_t n_t,
                   int32_t n_r, const int32_t *p_idx, const double *p_w,
                   const int32_t *col_src, const int32_t *q_idx,
                   const double *q_w, gw_warp **out);
int gw_warp_destroy(gw_warp *warp);
/* out = shift_peak(in), both rows x cols, host or device (flags). */
int gw_warp_apply(gw_warp *warp, const double *in, int32_t in_on_device,
                  double *out, int32_t out_on_device);
/* Apply `warp` (borrowed, same context and trimmed shape; NULL: none) to the
 * trimmed simulated image before every gw_compare_eval, as fit_slabsize.py
 * fullfit_model does (:36). */
int gw_compare_set_warp(gw_compare *cmp, gw_warp *warp);

/* ---- per-slice and helper entry points (device, synchronous) ---------- */
/* Gather I(q) at points (x,y,z) after applying n_R 3x3 rotations in order
 * (BLAS fused order), with the reference's floor division by dq and clip:
 * tools/detector.py:194-232 intersect_detector (n_R = 0, use_weight = 0) and
 * tools/detector.py:278-300 generate_detector_ints (the psi/phi/theta
 * matrices, weight = psi_w*phi_w*theta_w).  iq float64 (ny,nx,nz) host;
 * qmin = (min qx, min qy, min qz); out float64 (n) host. */
int gw_gather(gw_ctx *ctx, const double *iq, const int32_t *shape,
              const double *qmin, double dq, const double *x, const double *y,
              const double *z, int64_t n, const double *R, int32_t n_R,
              double weight, int32_t use_weight, double *out);
/* tools/voxelgrids.py:464-506 process_file2: bin one |F|^2 slice (nv,nh)
 * with per-column (qx,qy) and per-row qz into sum/count grids (q_num^3,
 * float64, host), added to what they hold. */
int gw_bin_slice(gw_ctx *ctx, const double *iq2d, int32_t nv, int32_t nh,
                 const double *hx, const double *hy, const double *vz,
                 int32_t q_num, double q_min, double q_max, double dq,
                 double *sum, double *count);
/* tools/detector.py:246-275 mirror_vertical_horizontal (float64, host). */
int gw_mirror(gw_ctx *ctx, const double *in, int32_t n_rows, int32_t n_cols,
              double *out);
/* tools/voxelgrids.py:828-857 add_f0_q_3d: iq (ny,nx,nz) times
 * ((sum_i a_i exp(-b_i q^2/16pi^2) + c)/Z)^2; coef = (a1,b1,...,a4,b4,c). */
int gw_f0_scale(gw_ctx *ctx, const double *iq, const int32_t *shape,
                const double *qx, const double *qy, const double *qz,
                const double *coef, double z, double *out);
/* tools/voxelgrids.py:238-309 rectangular_collapse_lengths at x_vals for the
 * slice scalars in ph (hor, ver before the phi > 90 swap). */
int gw_collapse_lengths(gw_ctx *ctx, const double *x_vals, int64_t n,
                        double hor, double ver, const gw_phi *ph, double *out);
/* Test hook for the conversion helpers hot kernels use instead of hardware
 * conversions: f32[i] = in[i] rounded to float (nearest even), f64[i] =
 * (double)(float)in[i], fl[i] = floor((float)in[i]) where fl_ok[i] = 1
 * (|x| < 2^21). */
int gw_debug_convert(gw_ctx *ctx, const double *in, int64_t n, float *f32,
                     double *f64, int32_t *fl, int32_t *fl_ok);

#ifdef __cplusplus
}
#endif
#endif /* GIWAXS_GB300_H */
