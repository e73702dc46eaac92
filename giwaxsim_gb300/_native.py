"""ctypes binding of libgiwaxs_gb300.so (the C ABI in include/giwaxs_gb300.h).

The library is required: importing works without it, but every call that
needs it raises NativeLibraryMissing naming the build command.  There is no
CPU fallback.  ctypes releases the GIL for the duration of each call.
"""
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgiwaxs_gb300.so")

GW_OK, GW_ERR_ARG, GW_ERR_OOM, GW_ERR_CUDA = 0, 1, 2, 3
GW_ERR_TIMEOUT, GW_ERR_BOUNDS, GW_ERR_STATE = 4, 5, 6
GW_VOXEL_BATCHED, GW_VOXEL_PLAIN = 0, 1
GW_ACCUM_FP64, GW_ACCUM_KAHAN32 = 0, 1
GW_DEPOSIT_NEAREST, GW_DEPOSIT_BILINEAR = 0, 1
GW_SHELLS_PER_SHELL, GW_SHELLS_REFERENCE = 1, 2
GW_TRANSFORM_AUTO, GW_TRANSFORM_STOCKHAM, GW_TRANSFORM_FUSED = 0, 1, 2
GW_BINNING_AUTO, GW_BINNING_ATOMIC, GW_BINNING_GATHER = 0, 1, 2

# every symbol include/giwaxs_gb300.h declares
EXPORTS = [
    "gw_version", "gw_status_string", "gw_last_error", "gw_ctx_create",
    "gw_ctx_destroy", "gw_ctx_synchronize", "gw_ctx_stream",
    "gw_ctx_launch_count", "gw_ctx_set_timing", "gw_ctx_kernel_times",
    "gw_kernel_category_name", "gw_rotate_points", "gw_collapse_base",
    "gw_voxel_plan_create", "gw_voxel_plan_destroy", "gw_voxel_set_atoms",
    "gw_voxel_set_shells", "gw_voxel_get_iq32", "gw_debug_convert",
    "gw_voxel_execute", "gw_voxel_capture_graph", "gw_voxel_get_iq",
    "gw_voxel_set_wait_limit", "gw_set_alloc_fault", "gw_voxel_block_variants",
    "gw_host_pin", "gw_host_unpin",
    "gw_voxel_device_iq32", "gw_voxel_get_counts", "gw_voxel_get_sums",
    "gw_voxel_info", "gw_voxel_debug_deposit", "gw_voxel_debug_window",
    "gw_voxelgrid",
    "gw_detector_plan_create", "gw_detector_plan_destroy",
    "gw_detector_set_iq", "gw_detector_set_iq32_device",
    "gw_detector_execute", "gw_detector_get", "gw_detector_debug_indices",
    "gw_detector_noalloc", "gw_detector", "gw_gather", "gw_bin_slice",
    "gw_mirror", "gw_f0_scale", "gw_collapse_lengths",
    "gw_detector_backward", "gw_voxel_backward", "gw_voxel_grad_buffer",
    "gw_ctx_device_name", "gw_ctx_mark", "gw_ctx_elapsed_ms",
    "gw_slab_create", "gw_slab_destroy", "gw_slab_info", "gw_slab_get",
    "gw_slab_device_xyz",
    "gw_compare_create", "gw_compare_destroy", "gw_compare_target",
    "gw_compare_eval", "gw_detector_device_out", "gw_warp_create",
    "gw_warp_destroy", "gw_warp_apply", "gw_compare_set_warp",
]


class NativeLibraryMissing(RuntimeError):
    pass


class GwError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (_STATUS.get(status, status), message))
        self.status = status


_STATUS = {1: "GW_ERR_ARG", 2: "GW_ERR_OOM", 3: "GW_ERR_CUDA",
           4: "GW_ERR_TIMEOUT", 5: "GW_ERR_BOUNDS", 6: "GW_ERR_STATE"}


class VoxelParams(ctypes.Structure):
    _fields_ = [("grid_size", ctypes.c_int32), ("r_voxel_size", ctypes.c_double),
                ("q_num", ctypes.c_int32), ("q_min", ctypes.c_double),
                ("q_max", ctypes.c_double), ("dq", ctypes.c_double),
                ("crop_lo", ctypes.c_int32), ("crop_hi", ctypes.c_int32),
                ("h_max", ctypes.c_double), ("fill_bkg", ctypes.c_int32),
                ("smooth", ctypes.c_double), ("mode", ctypes.c_int32),
                ("accum", ctypes.c_int32), ("average", ctypes.c_int32),
                ("f0_coef", ctypes.c_double * 9), ("f0_z", ctypes.c_double),
                ("batch_slices", ctypes.c_int32), ("deposit", ctypes.c_int32),
                ("fft_y", ctypes.c_int32), ("fft_z", ctypes.c_int32),
                ("transform_y", ctypes.c_int32), ("transform_z", ctypes.c_int32),
                ("block_variant", ctypes.c_int32), ("real_grids", ctypes.c_int32),
                ("binning", ctypes.c_int32)]


class Structure(ctypes.Structure):
    _fields_ = [("atom_begin", ctypes.c_int64), ("atom_count", ctypes.c_int64),
                ("x_bound", ctypes.c_double), ("y_bound", ctypes.c_double),
                ("z_bound", ctypes.c_double), ("avg_f_re", ctypes.c_double),
                ("avg_f_im", ctypes.c_double), ("max_voxels", ctypes.c_double)]


class Phi(ctypes.Structure):
    _fields_ = [("cos_phi", ctypes.c_double), ("sin_phi", ctypes.c_double),
                ("right_qy", ctypes.c_double), ("right_qx", ctypes.c_double),
                ("cl_case", ctypes.c_int32), ("cl_swap", ctypes.c_int32),
                ("cos_t", ctypes.c_double), ("sin_t", ctypes.c_double),
                ("tan_t", ctypes.c_double), ("cos_p", ctypes.c_double),
                ("sin_p", ctypes.c_double), ("tan_p", ctypes.c_double)]


class DetectorParams(ctypes.Structure):
    _fields_ = [("n_h", ctypes.c_int32), ("n_v", ctypes.c_int32),
                ("iq_shape", ctypes.c_int32 * 3), ("qmin_x", ctypes.c_double),
                ("qmin_y", ctypes.c_double), ("qmin_z", ctypes.c_double),
                ("dq", ctypes.c_double), ("mirror", ctypes.c_int32),
                ("accum", ctypes.c_int32), ("exact", ctypes.c_int32),
                ("no_plane", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


_lib = None
_lib_lock = threading.Lock()
P = ctypes.c_void_p


def _declare(lib):
    i32, i64, d = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    pp = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "gw_version": ([], ctypes.c_int),
        "gw_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "gw_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_size_t),
        "gw_ctx_create": ([ctypes.c_int, pp], ctypes.c_int),
        "gw_ctx_destroy": ([P], ctypes.c_int),
        "gw_ctx_synchronize": ([P], ctypes.c_int),
        "gw_ctx_stream": ([P, pp], ctypes.c_int),
        "gw_ctx_launch_count": ([P], i64),
        "gw_ctx_set_timing": ([P, i32], ctypes.c_int),
        "gw_ctx_kernel_times": ([P, P, P, i32], ctypes.c_int),
        "gw_kernel_category_name": ([i32], ctypes.c_char_p),
        "gw_rotate_points": ([P, P, i64, P], ctypes.c_int),
        "gw_collapse_base": ([P, P, i64, P], ctypes.c_int),
        "gw_voxel_plan_create": ([P, P, P, i32, P, i32, pp], ctypes.c_int),
        "gw_voxel_plan_destroy": ([P], ctypes.c_int),
        "gw_voxel_set_atoms": ([P, P, P, i64, i32], ctypes.c_int),
        "gw_voxel_set_shells": ([P, i32, i32, P, P, P, P, P], ctypes.c_int),
        "gw_voxel_get_iq32": ([P, P], ctypes.c_int),
        "gw_debug_convert": ([P, P, i64, P, P, P, P], ctypes.c_int),
        "gw_voxel_execute": ([P], ctypes.c_int),
        "gw_voxel_capture_graph": ([P], ctypes.c_int),
        "gw_voxel_set_wait_limit": ([P, ctypes.c_uint32], ctypes.c_int),
        "gw_set_alloc_fault": ([i64], ctypes.c_int),
        "gw_host_pin": ([P, ctypes.c_uint64], ctypes.c_int),
        "gw_host_unpin": ([P], ctypes.c_int),
        "gw_voxel_block_variants": ([], ctypes.c_int32),
        "gw_voxel_get_iq": ([P, P, i32], ctypes.c_int),
        "gw_voxel_device_iq32": ([P, ctypes.c_int32, pp], ctypes.c_int),
        "gw_voxel_get_counts": ([P, P], ctypes.c_int),
        "gw_voxel_get_sums": ([P, P], ctypes.c_int),
        "gw_voxel_info": ([P, P, i32], ctypes.c_int),
        "gw_voxel_debug_deposit": ([P, i32, P, P], ctypes.c_int),
        "gw_voxel_debug_window": ([P, i32, P], ctypes.c_int),
        "gw_voxelgrid": ([P, P, P, i32, P, i32, P, P, i64, P], ctypes.c_int),
        "gw_detector_plan_create": ([P, P, P, P, P, i32, P, P, P, i32, pp],
                                    ctypes.c_int),
        "gw_detector_plan_destroy": ([P], ctypes.c_int),
        "gw_detector_set_iq": ([P, P, i32], ctypes.c_int),
        "gw_detector_set_iq32_device": ([P, P], ctypes.c_int),
        "gw_detector_execute": ([P], ctypes.c_int),
        "gw_detector_get": ([P, P, i32], ctypes.c_int),
        "gw_detector_debug_indices": ([P, i32, P], ctypes.c_int),
        "gw_detector_noalloc": ([P, P, P, P, P, i32, P, P, P, i32, P, P],
                                ctypes.c_int),
        "gw_detector": ([P, P, P, P, P, P, i32, P, P, P, i32, P], ctypes.c_int),
        "gw_gather": ([P, P, P, P, d, P, P, P, i64, P, i32, d, i32, P],
                      ctypes.c_int),
        "gw_bin_slice": ([P, P, i32, i32, P, P, P, i32, d, d, d, P, P],
                         ctypes.c_int),
        "gw_mirror": ([P, P, i32, i32, P], ctypes.c_int),
        "gw_f0_scale": ([P, P, P, P, P, P, P, d, P], ctypes.c_int),
        "gw_collapse_lengths": ([P, P, i64, d, d, P, P], ctypes.c_int),
        "gw_detector_backward": ([P, P, i32, P, i32], ctypes.c_int),
        "gw_voxel_backward": ([P, P, i32, P, P, P, P], ctypes.c_int),
        "gw_voxel_grad_buffer": ([P, pp], ctypes.c_int),
        "gw_ctx_device_name": ([P, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
        "gw_ctx_mark": ([P, i32], ctypes.c_int),
        "gw_ctx_elapsed_ms": ([P, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
        "gw_slab_create": ([P, P, i32, P, P, pp], ctypes.c_int),
        "gw_slab_destroy": ([P], ctypes.c_int),
        "gw_slab_info": ([P, P, P], ctypes.c_int),
        "gw_slab_get": ([P, P, P, i32], ctypes.c_int),
        "gw_slab_device_xyz": ([P, pp], ctypes.c_int),
        "gw_compare_create": ([P, i32, i32, i32, i32, i32, i32, P, P, P, P, i64, pp],
                              ctypes.c_int),
        "gw_compare_destroy": ([P], ctypes.c_int),
        "gw_compare_target": ([P, P, P], ctypes.c_int),
        "gw_compare_eval": ([P, P, i32, P, P], ctypes.c_int),
        "gw_warp_create": ([P, i32, i32, i32, i32, P, P, P, P, P, pp], ctypes.c_int),
        "gw_warp_destroy": ([P], ctypes.c_int),
        "gw_warp_apply": ([P, P, i32, P, i32], ctypes.c_int),
        "gw_compare_set_warp": ([P, P], ctypes.c_int),
        "gw_detector_device_out": ([P, pp], ctypes.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """The loaded native library (raises NativeLibraryMissing if not built)."""
    global _lib
    if _lib is None:
        with _lib_lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise NativeLibraryMissing(
                        "giwaxsim_gb300 native library not found at %s; build "
                        "it with `python -m giwaxsim_gb300.build` (needs nvcc "
                        "13, targets sm_103a)" % LIB_PATH)
                lib_ = ctypes.CDLL(LIB_PATH)
                _declare(lib_)
                _lib = lib_
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(2048)
    lib().gw_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status):
    if status != GW_OK:
        raise GwError(status, last_error())
    return status


def ptr(a):
    """Host address of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """One gw_ctx: a CUDA stream on one device plus a device error word."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().gw_ctx_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def synchronize(self):
        check(lib().gw_ctx_synchronize(self.handle))

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().gw_ctx_stream(self.handle, ctypes.byref(s)))
        return s.value or 0

    def launch_count(self):
        return int(lib().gw_ctx_launch_count(self.handle))

    def device_name(self):
        buf = ctypes.create_string_buffer(256)
        check(lib().gw_ctx_device_name(self.handle, buf, 256))
        return buf.value.decode()

    def time_ms(self, fn, reps=1):
        """Device milliseconds per call of fn() (work on this context's
        stream), timed between two events on the stream."""
        check(lib().gw_ctx_mark(self.handle, 0))
        for _ in range(reps):
            fn()
        check(lib().gw_ctx_mark(self.handle, 1))
        ms = ctypes.c_float()
        check(lib().gw_ctx_elapsed_ms(self.handle, ctypes.byref(ms)))
        return ms.value / reps

    def set_timing(self, on):
        check(lib().gw_ctx_set_timing(self.handle, int(bool(on))))

    def kernel_times(self):
        """{category: (total_ms, launches)} since timing was switched on."""
        ms = np.zeros(32)
        n = np.zeros(32, dtype=np.int64)
        k = lib().gw_ctx_kernel_times(self.handle, ptr(ms), ptr(n), 32)
        if k < 0:
            check(k)
        return {lib().gw_kernel_category_name(i).decode(): (float(ms[i]), int(n[i]))
                for i in range(k) if n[i] > 0}

    def close(self):
        if self.handle:
            lib().gw_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_thread_contexts = threading.local()


def default_context(device=0):
    """The calling thread's context on `device`, made on first use.  Each
    thread has its own (own stream, own device error word): calls from
    several threads, as the reference's drivers make from a thread pool,
    run concurrently on the GPU and never land in each other's stream or
    graph capture.  A context passed explicitly is for one thread at a
    time.  A thread's context is destroyed when the thread ends and no
    plan holds it."""
    ctxs = getattr(_thread_contexts, "by_device", None)
    if ctxs is None:
        ctxs = _thread_contexts.by_device = {}
    c = ctxs.get(device)
    if c is None:
        c = ctxs[device] = Context(device)
    return c


def rotate_points(R, pts):
    """Host fused-chain rotation (np.dot(pts, R.T) as OpenBLAS evaluates it)."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.empty_like(pts)
    check(lib().gw_rotate_points(ptr(R), ptr(pts), len(pts), ptr(out)))
    return out


def collapse_base(ver, cos_t):
    ver = np.ascontiguousarray(ver, dtype=np.float64)
    cos_t = np.ascontiguousarray(cos_t, dtype=np.float64)
    out = np.empty_like(ver)
    check(lib().gw_collapse_base(ptr(ver), ptr(cos_t), len(ver), ptr(out)))
    return out


def set_alloc_fault(after):
    """Test hook: the (after+1)-th device allocation from now on and every
    later one fail with GW_ERR_OOM; after < 0 turns the injection off."""
    check(lib().gw_set_alloc_fault(int(after)))


def fused_variant_count():
    """Block shapes of the fused chirp-z kernels (block_variant 0 .. n-1)."""
    return int(lib().gw_voxel_block_variants())
