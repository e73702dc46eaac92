"""Host side of the forward path: reference-exact geometry and per-slice
scalars, and thin owners of the native voxel and detector plans.

Everything here is O(number of slices + orientations) host work on small
arrays; per-atom and per-pixel work is on the GPU (libgiwaxs_gb300.so).
The host computes, with numpy, exactly the scalars the reference computes
with numpy (its trig, pow and reductions), so that the device replays the
same float64 arithmetic per atom and per pixel:

  tools/comparison.py:704-744   grid size, q axis, automatic phis, checks,
                                bounds, f values, avg_voxel_f
  tools/voxelgrids.py:16-48     crop range (downselect_voxelgrid)
  tools/voxelgrids.py:253-285   rectangular_collapse_lengths branch scalars
  tools/voxelgrids.py:382-399   slice h-axis end points
  tools/comparison.py:790-841   detector set-up, weights, orientation order
  tools/detector.py:33-162      axis of each plane rotation from the
                                current plane's corners
"""
import atexit
import ctypes
import warnings

import numpy as np
from numpy.fft import fftfreq, fftshift

from . import _native as N
from .tools.ptable_dict import aff_dict, ptable


# ------------------------------------------------------------------ voxel
class VoxelGeometry:
    """Grid, q axis, automatic phis and crop of voxelgridmaker_fitting
    (comparison.py:704-731) and downselect_voxelgrid (voxelgrids.py:35-46)."""

    def __init__(self, r_voxel_size, q_voxel_size, max_q):
        max_q_diag = np.sqrt(2) * max_q
        if max_q_diag > 2 * np.pi / r_voxel_size:
            raise Exception("Max_q is non-physical for given voxel size")
        self.r_voxel_size = r_voxel_size
        self.q_voxel_size = q_voxel_size
        self.max_q = max_q
        self.grid_size = int(np.ceil(2 * np.pi / (q_voxel_size * r_voxel_size)))
        max_q_diag = max_q_diag + max_q_diag % q_voxel_size
        q_num = ((2 * max_q_diag / q_voxel_size) + 1).astype(int)
        if q_num % 2 == 0:
            q_num += 1
        self.q = np.linspace(-max_q_diag, max_q_diag, q_num)
        self.q_num = int(q_num)
        dphi = np.arctan(q_voxel_size / max_q_diag)
        phi_num = np.ceil(2 * np.pi / dphi).astype(int)
        self.auto_phis = np.linspace(0, 180 - (180 / phi_num), num=phi_num)
        # downselect_voxelgrid on the (identical) x, y and z axes
        voxel = np.abs(self.q[1] - self.q[0])
        keep = np.where(np.abs(self.q) < max_q + voxel)[0]
        self.crop_lo, self.crop_hi = int(keep[0]), int(keep[-1])
        self.q_crop = self.q[self.crop_lo:self.crop_hi + 1]
        self.dq = np.diff(self.q)[0]
        q_h = fftshift(fftfreq(self.grid_size, d=r_voxel_size) * 2 * np.pi)
        self.h_max = np.max(q_h)

    @classmethod
    def from_axes(cls, grid_size, r_voxel_size, q_axis):
        """Geometry of the reference's per-slice worker, which receives the
        grid size and the q axis instead of q_voxel_size and max_q
        (voxelgrids.py:311-315).  The crop is the whole axis."""
        g = cls.__new__(cls)
        g.r_voxel_size = r_voxel_size
        g.q_voxel_size = None
        g.max_q = None
        g.grid_size = int(grid_size)
        g.q = np.asarray(q_axis, dtype=np.float64)
        g.q_num = len(g.q)
        g.auto_phis = None
        g.crop_lo, g.crop_hi = 0, g.q_num - 1
        g.q_crop = g.q
        g.dq = np.diff(g.q)[0]
        q_h = fftshift(fftfreq(g.grid_size, d=r_voxel_size) * 2 * np.pi)
        g.h_max = np.max(q_h)
        return g

    def check_bounds(self, coords, ranges=None):
        b = coord_ranges(coords) if ranges is None else ranges
        if self.grid_size * self.r_voxel_size < np.min(b):
            raise Exception("Calculated real-space bounds smaller than "
                            "simulation. Please lower delta_q value")

    def phi_table(self, phis):
        """Per-slice scalars as numpy computes them in the reference (the
        last table made is kept for a call with the same phis; read-only)."""
        phis = np.asarray(phis, dtype=np.float64)
        global _PHI_TABLE_LAST
        key = (self.h_max, phis.tobytes())
        last = _PHI_TABLE_LAST  # one (key, table) tuple: threads see either whole
        if last is not None and last[0] == key:
            return last[1]
        t = self._phi_table(phis)
        t.flags.writeable = False
        _PHI_TABLE_LAST = (key, t)
        return t

    def _phi_table(self, phis):
        t = np.zeros(len(phis), dtype=_dtype_of(N.Phi))
        pr = np.radians(phis)
        t["cos_phi"] = np.cos(pr)
        t["sin_phi"] = np.sin(pr)
        t["right_qy"] = self.h_max * np.cos(np.deg2rad(-phis))
        t["right_qx"] = -self.h_max * np.sin(np.deg2rad(-phis))
        swap = phis > 90
        padj = np.where(swap, phis - 90, phis)
        theta = 90 - padj
        tr, pa = np.deg2rad(theta), np.deg2rad(padj)
        t["cl_case"] = np.where(padj == 0, 0, np.where(padj == 90, 1, 2))
        t["cl_swap"] = swap.astype(np.int32)
        t["cos_t"], t["sin_t"], t["tan_t"] = np.cos(tr), np.sin(tr), np.tan(tr)
        t["cos_p"], t["sin_p"], t["tan_p"] = np.cos(pa), np.sin(pa), np.tan(pa)
        return t


_DTYPES = {}
_PHI_TABLE_LAST = None  # ((h_max, phis bytes), table) of the last phi_table


def _dtype_of(ctype):
    """numpy dtype of a ctypes structure, made once per type."""
    d = _DTYPES.get(ctype)
    if d is None:
        d = _DTYPES[ctype] = np.dtype(ctype)
    return d


def element_kinds(elements):
    """Distinct element symbols and every atom's index into them.  Symbols
    of up to two characters (numpy's fixed-width strings) are compared as
    64-bit integers: no string sort, and one vector compare when all atoms
    are of one element."""
    a = np.asarray(elements)
    if a.ndim == 1 and len(a) and a.dtype.kind == "U" and a.dtype.itemsize <= 8:
        c = np.ascontiguousarray(a)
        key = c.view(np.uint64 if c.dtype.itemsize == 8 else np.uint32)
        if (key == key[0]).all():
            return [str(a[0])], np.zeros(len(a), np.intp)
        _, first, inv = np.unique(key, return_index=True, return_inverse=True)
        return [str(a[i]) for i in first], inv.reshape(-1)
    uniq, inv = np.unique(a, return_inverse=True)
    return [str(e) for e in uniq], inv.reshape(-1)


def element_f_values(elements, energy, f1f2=None):
    """f = Z + f' + i f'' per atom (comparison.py:735-739)."""
    from .tools.utilities import get_element_f1_f2_dict
    uniq, inv = element_kinds(elements)
    d = f1f2 if f1f2 is not None else get_element_f1_f2_dict(energy, uniq)
    vals = np.array([complex(d[e]) for e in uniq], dtype=complex)
    vals += np.array([ptable[e] for e in uniq])
    if len(vals) == 1:
        return np.full(len(inv), vals[0])
    return vals[inv]


def real_multiples(fv):
    """True when every f value is a real multiple of one complex value (to
    the float32 precision the device keeps them in) and their sum does not
    cancel: the slice grids are then that value's phase times real grids
    (gw_voxel_params.real_grids)."""
    f = np.asarray(fv, dtype=complex).ravel()
    if f.size == 0:
        return False
    if (f == f[0]).all():  # one value (one element, no weights): one pass
        return bool(f[0] != 0)
    ref = f[np.argmax(np.abs(f))]
    if ref == 0:
        return False
    cross = f.imag * ref.real - f.real * ref.imag  # Im(f conj(ref))
    if np.max(np.abs(cross)) > 1e-6 * abs(ref) * np.max(np.abs(f)):
        return False
    return bool(abs(np.sum(f)) > 1e-3 * np.sum(np.abs(f)))


def coord_ranges(coords):
    """max - min of x, y and z (comparison.py:712-717), from a transposed
    copy (contiguous reductions)."""
    t = np.ascontiguousarray(np.asarray(coords, dtype=np.float64).T)
    return [t[i].max() - t[i].min() for i in range(3)]


def structure_constants(coords, f_values, r_voxel_size, ranges=None):
    """x/y/z bounds, avg_voxel_f (comparison.py:712-744) and max_voxels
    (voxelgrids.py:344)."""
    xb, yb, zb = coord_ranges(coords) if ranges is None else ranges
    avg = (np.sum(f_values) / (xb * yb * zb)) * r_voxel_size ** 3
    max_voxels = np.sqrt(xb ** 2 + yb ** 2) // r_voxel_size
    return xb, yb, zb, complex(avg), float(max_voxels)


def f0_params(element):
    if element is None:
        return [0.0] * 9, 0.0
    return list(aff_dict[element]), float(ptable[element])


class HostPool:
    """Recycled host buffers for large results.  A fresh multi-hundred-MB
    numpy array costs the operating system a first-touch zeroing of every
    page several times longer than the device-to-host copy into it; a
    buffer whose previous result the caller has dropped (only the pool
    still references it) is handed out again instead.  Arrays given out are
    ordinary float64 arrays owned by the caller for as long as it keeps
    them; the pool keeps at most `per_shape` buffers per shape and
    `max_bytes` in all.  Kept buffers are page-locked (gw_host_pin) when
    `pin` is on, so that the result copies into them run at the link's
    speed rather than through the driver's staging buffers; clear()
    releases them (at exit too)."""

    def __init__(self, min_bytes=64 << 20, per_shape=2, max_bytes=4 << 30,
                 pin=True):
        import sys
        import threading
        self._refs = sys.getrefcount
        self._lock = threading.Lock()
        self.min_bytes, self.per_shape, self.max_bytes = min_bytes, per_shape, max_bytes
        self.pin = pin
        self._bufs = {}
        self._pinned = []

    def _pin(self, b):
        """Page-lock b (kept by the pool until clear()); a refusal leaves it
        pageable."""
        try:
            ok = N.lib().gw_host_pin(ctypes.c_void_p(b.ctypes.data), b.nbytes) == N.GW_OK
        except N.NativeLibraryMissing:
            ok = False
        if ok:
            # the address only: a reference here would keep the buffer
            # from ever being handed out again (see empty())
            self._pinned.append(b.ctypes.data)

    def empty(self, shape, dtype=np.float64):
        shape, dtype = tuple(int(v) for v in shape), np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        if nbytes < self.min_bytes:
            return np.empty(shape, dtype)
        key = (shape, dtype.str)
        with self._lock:
            bufs = self._bufs.setdefault(key, [])
            for b in bufs:
                # referenced by the list, the loop variable and getrefcount's
                # argument only: no result array uses it any more
                if self._refs(b) <= 3:
                    return b.view()
            held = sum(x.nbytes for v in self._bufs.values() for x in v)
            b = np.empty(shape, dtype)
            if len(bufs) < self.per_shape and held + nbytes <= self.max_bytes:
                bufs.append(b)
                if self.pin:
                    self._pin(b)
            return b.view()

    def clear(self):
        """Drop the kept buffers (arrays handed out stay valid), releasing
        their page locks first."""
        with self._lock:
            for ptr in self._pinned:
                N.lib().gw_host_unpin(ctypes.c_void_p(ptr))
            self._pinned.clear()
            self._bufs.clear()


HOST_POOL = HostPool()
atexit.register(HOST_POOL.clear)  # page locks released before the driver goes


class VoxelPlan:
    """Owner of a gw_voxel_plan for one geometry, a list of structures and
    a list of phis.  structures: list of (coords (N,3), f_values (N,)
    complex, weights (N,) or None).  real: None runs the real-grid path
    (gw_voxel_params.real_grids) when every structure's weighted f values
    are real multiples of one complex value in a batched, nearest-bin plan
    without a fused kernel asked for; False keeps the general path (needed
    for set_shells and backward); True asks for it and refuses f values
    that do not allow it.  binning: "auto" (gather where it applies),
    "atomic" or "gather" (gw_voxel_params.binning)."""

    def __init__(self, geom, structures, phis=None, fill_bkg=False, smooth=0,
                 mode="batched", accum="fp64", average=True, f0_element="C",
                 batch_slices=0, constants=None, deposit="nearest", fft_y=0,
                 fft_z=0, tune=False, ctx=None, create=True, ranges=None,
                 transform="auto", block_variant=0, real=None, binning="auto"):
        self.geom = geom
        self.handle = None
        self.reused = False          # handed out again by PlanCache
        self.graph_captured = False  # the library drops the graph when the
        self._atoms_n = None         # atom count or the shells change
        self.ctx = ctx or N.default_context()
        self.tuned = None
        if tune and mode == "batched":
            from . import autotune

            def make(**choice):
                return VoxelPlan(geom, structures, phis=phis, fill_bkg=fill_bkg,
                                 smooth=smooth, mode=mode, accum=accum,
                                 average=average, f0_element=f0_element,
                                 constants=constants, deposit=deposit,
                                 real=real, ctx=self.ctx, **choice)

            self.tuned = autotune.tune(make, len(structures), fill_bkg, smooth,
                                       deposit, ctx=self.ctx)
            fft_y, fft_z = self.tuned["fft_y"], self.tuned["fft_z"]
            batch_slices = self.tuned["batch_slices"]
            transform = self.tuned["transform"]
            block_variant = self.tuned["block_variant"]
            binning = self.tuned.get("binning", binning)
        self.phis = geom.auto_phis if phis is None else np.asarray(phis, np.float64)
        if len(self.phis) < 1:
            raise ValueError("at least one phi is required")
        r = geom.r_voxel_size
        st = np.zeros(len(structures), dtype=_dtype_of(N.Structure))
        xyz, fs = [], []
        all_real = True
        begin = 0
        for i, (coords, fv, w) in enumerate(structures):
            coords = np.ascontiguousarray(coords, dtype=np.float64)
            if coords.ndim != 2 or coords.shape[1] != 3 or len(coords) == 0:
                raise ValueError("coords must be a non-empty (N, 3) array")
            fv = np.asarray(fv, dtype=complex)
            if w is not None:
                fv = fv * np.asarray(w, dtype=np.float64)
            all_real = all_real and real_multiples(fv)
            if constants is not None:
                # the per-slice worker receives the driver's constants
                xb, yb, zb, avg = constants[i]
                avg = complex(avg)
                mv = float(np.sqrt(xb ** 2 + yb ** 2) // r)
            else:
                # ranges: per-structure coord_ranges the caller already has
                rg = coord_ranges(coords) if ranges is None else ranges[i]
                geom.check_bounds(coords, rg)
                xb, yb, zb, avg, mv = structure_constants(coords, fv, r, rg)
            # real grids take the phase of avg (a finite, nonzero value)
            all_real = all_real and bool(np.isfinite(avg) and avg != 0)
            st[i] = (begin, len(coords), xb, yb, zb, avg.real, avg.imag, mv)
            begin += len(coords)
            xyz.append(coords)
            fs.append(fv.astype(np.complex64))
        self.structs = st
        # the plan's own copy of the coordinates; the f values are already
        # a fresh array for one structure
        self.xyz = np.ascontiguousarray(np.concatenate(xyz))
        self.f = (fs[0] if len(fs) == 1 else np.concatenate(fs)).view(np.float32)
        self.phi_tab = geom.phi_table(self.phis)
        p = N.VoxelParams()
        p.grid_size = geom.grid_size
        p.r_voxel_size = r
        p.q_num = geom.q_num
        p.q_min, p.q_max = geom.q[0], geom.q[-1]
        p.dq = geom.dq
        p.crop_lo, p.crop_hi = geom.crop_lo, geom.crop_hi
        p.h_max = geom.h_max
        p.fill_bkg = int(bool(fill_bkg))
        p.smooth = float(smooth) if smooth else 0.0
        p.mode = {"batched": N.GW_VOXEL_BATCHED, "plain": N.GW_VOXEL_PLAIN}[mode]
        p.accum = {"fp64": N.GW_ACCUM_FP64, "kahan32": N.GW_ACCUM_KAHAN32}[accum]
        # True/False: average/sum over structures; "separate": one I(q) each
        p.average = 2 if average == "separate" else int(bool(average))
        self.n_out = len(structures) if average == "separate" else 1
        coef, z = f0_params(f0_element)
        for i in range(9):
            p.f0_coef[i] = coef[i]
        p.f0_z = z
        p.batch_slices = int(batch_slices)
        p.deposit = {"nearest": N.GW_DEPOSIT_NEAREST,
                     "bilinear": N.GW_DEPOSIT_BILINEAR}[deposit]
        p.fft_y, p.fft_z = int(fft_y), int(fft_z)
        # one kernel family for both axes, or (rows, columns)
        ty, tz = (transform, transform) if isinstance(transform, str) else transform
        fam = {"auto": N.GW_TRANSFORM_AUTO, "stockham": N.GW_TRANSFORM_STOCKHAM,
               "fused": N.GW_TRANSFORM_FUSED}
        p.transform_y, p.transform_z = fam[ty], fam[tz]
        p.block_variant = int(block_variant)
        # real grids (every structure's f values real multiples of one
        # value): None decides from the f values, False keeps the general
        # path (the adjoint and multi-q shells need it)
        if real is None:
            real = (all_real and mode == "batched" and deposit == "nearest"
                    and "fused" not in (ty, tz))
        elif real and not all_real:
            raise ValueError("real=True needs every structure's f values to be "
                             "real multiples of one complex value, with a finite, "
                             "nonzero average voxel f")
        p.real_grids = int(bool(real))
        p.binning = {"auto": N.GW_BINNING_AUTO, "atomic": N.GW_BINNING_ATOMIC,
                     "gather": N.GW_BINNING_GATHER}[binning]
        self.params = p
        self.Qc = geom.crop_hi - geom.crop_lo + 1
        if create:
            self.create()

    def create(self):
        """Make the native plan (VoxelPlan(..., create=False) leaves it to
        this call)."""
        h = ctypes.c_void_p()
        N.check(N.lib().gw_voxel_plan_create(
            self.ctx.handle, ctypes.byref(self.params), N.ptr(self.structs),
            len(self.structs), N.ptr(self.phi_tab), len(self.phi_tab),
            ctypes.byref(h)))
        self.handle = h

    def key(self):
        """Everything gw_voxel_plan_create receives: two plans with equal
        keys are the same plan (the atoms themselves come with set_atoms).
        The context enters by identity: a plan keeps its context object
        alive, so a context made after another was closed never matches."""
        return (id(self.ctx), bytes(self.params),
                self.structs.tobytes(), self.phi_tab.tobytes(), self.n_out)

    def set_atoms(self, xyz=None, f=None, on_device=False):
        if xyz is None:
            xyz, f = self.xyz, self.f
        elif not on_device and getattr(getattr(self, "params", None), "real_grids", 0):
            self._check_real(f)
        n = len(self.xyz) if on_device else len(xyz)
        if n != self._atoms_n:
            self.graph_captured = False
            self._atoms_n = None
        if on_device:
            N.check(N.lib().gw_voxel_set_atoms(self.handle, ctypes.c_void_p(xyz),
                                               ctypes.c_void_p(f), n, 1))
        else:
            N.check(N.lib().gw_voxel_set_atoms(self.handle, N.ptr(xyz), N.ptr(f),
                                               n, 0))
        self._atoms_n = n

    def _check_real(self, f):
        """A real-grid plan takes each structure's grid as the phase of its
        average voxel f times a real grid: atoms whose f values are not
        real multiples of that phase would give wrong intensities, so they
        are refused (make the plan with real=False for them)."""
        fc = np.asarray(f)
        fc = (np.ascontiguousarray(fc).view(np.complex64) if fc.dtype == np.float32
              else fc.astype(complex)).ravel()
        for s in self.structs:
            b, n = int(s["atom_begin"]), int(s["atom_count"])
            part = fc[b:b + n].astype(complex)
            avg = complex(s["avg_f_re"], s["avg_f_im"])
            cross = part.imag * avg.real - part.real * avg.imag
            if len(part) != n or np.max(np.abs(cross), initial=0.0) > (
                    1e-6 * abs(avg) * np.max(np.abs(part), initial=0.0)):
                raise ValueError("set_atoms: f values that are not real multiples "
                                 "of the structure's average f, on a real-grid plan")

    def set_shells(self, q_axis, lower, upper, f_shells, avg_shells,
                   mode="per_shell"):
        """Multi-q form factors (voxelgrids.py:650-707): shell k (lower[k] <
        |q| <= upper[k]) takes its I(q) from a pass with the per-atom f
        values f_shells[k] (n_atoms complex, in the plan's atom order) and
        the per-structure avg_voxel_f avg_shells[k].  mode "per_shell" or
        "reference" (the reference's own output, see gw_voxel_set_shells).
        Call after set_atoms; set_shells(None) clears them (set the atoms
        again afterwards)."""
        self.graph_captured = False
        if q_axis is None:
            N.check(N.lib().gw_voxel_set_shells(self.handle, 0, 0, None, None,
                                                None, None, None))
            return
        lower = np.ascontiguousarray(lower, dtype=np.float64)
        upper = np.ascontiguousarray(upper, dtype=np.float64)
        K = len(lower)
        f = np.ascontiguousarray(np.asarray(f_shells, dtype=np.complex64)
                                 .reshape(K, len(self.xyz)))
        avg = np.ascontiguousarray(np.asarray(avg_shells, dtype=np.complex128)
                                   .reshape(K, len(self.structs)))
        q = np.ascontiguousarray(q_axis, dtype=np.float64)
        if len(q) != self.params.q_num or len(upper) != K:
            raise ValueError("q_axis must be the full q axis and lower/upper "
                             "one value per shell")
        m = {"per_shell": N.GW_SHELLS_PER_SHELL,
             "reference": N.GW_SHELLS_REFERENCE}[mode]
        N.check(N.lib().gw_voxel_set_shells(self.handle, K, m, N.ptr(q),
                                            N.ptr(lower), N.ptr(upper),
                                            N.ptr(f), N.ptr(avg)))

    def execute(self):
        N.check(N.lib().gw_voxel_execute(self.handle))

    def capture_graph(self):
        N.check(N.lib().gw_voxel_capture_graph(self.handle))
        self.graph_captured = True

    def set_wait_limit(self, polls):
        """Poll limit of the column kernel's bounded tile-load wait (0 makes
        every wait run out: a test hook for the timeout path).  Drops a
        captured graph."""
        N.check(N.lib().gw_voxel_set_wait_limit(self.handle, int(polls)))
        self.graph_captured = False

    def iq(self, out=None):
        """I(q) (Qc, Qc, Qc); (n_struct, Qc, Qc, Qc) for separate structures.
        Without `out`, a fresh array (large ones from the recycled host
        buffers of HostPool)."""
        shape = (self.Qc,) * 3 if self.n_out == 1 else (self.n_out,) + (self.Qc,) * 3
        out = HOST_POOL.empty(shape) if out is None else out
        N.check(N.lib().gw_voxel_get_iq(self.handle, N.ptr(out), 0))
        return out

    def iq32(self):
        """The float32 I(q) the detector gathers from (host copy)."""
        shape = (self.Qc,) * 3 if self.n_out == 1 else (self.n_out,) + (self.Qc,) * 3
        out = np.empty(shape, dtype=np.float32)
        N.check(N.lib().gw_voxel_get_iq32(self.handle, N.ptr(out)))
        return out

    def iq_to_device(self, dev_ptr):
        N.check(N.lib().gw_voxel_get_iq(self.handle, ctypes.c_void_p(dev_ptr), 1))

    def device_iq32(self, structure=0):
        """Device address of the float32 I(q) (of one structure when they
        are separate)."""
        p = ctypes.c_void_p()
        N.check(N.lib().gw_voxel_device_iq32(self.handle, int(structure),
                                             ctypes.byref(p)))
        return p.value

    def counts(self):
        out = np.empty((self.Qc,) * 3)
        N.check(N.lib().gw_voxel_get_counts(self.handle, N.ptr(out)))
        return out

    def sums(self):
        out = np.empty((self.Qc,) * 3)
        N.check(N.lib().gw_voxel_get_sums(self.handle, N.ptr(out)))
        return out

    def info(self):
        v = np.zeros(24, dtype=np.int64)
        n = N.lib().gw_voxel_info(self.handle, N.ptr(v), 24)
        keys = ["crop", "batch", "Ly", "Lz", "Nc", "Nr", "My", "Mz", "y_lo",
                "z_lo", "k0", "kz0", "n_slices", "device_bytes",
                "graph_kernels", "col_tma", "fused_y", "fused_z", "real",
                "gather", "heavy_lines", "multi_rows"]
        return dict(zip(keys, (int(x) for x in v[:n])))

    def debug_deposit(self, slice_index):
        t = int(slice_index) // len(self.phis)
        n = int(self.structs[t]["atom_count"])
        y = np.empty(n, np.int32)
        z = np.empty(n, np.int32)
        N.check(N.lib().gw_voxel_debug_deposit(self.handle, int(slice_index),
                                               N.ptr(y), N.ptr(z)))
        return y, z

    def grad_buffer(self):
        """Device address of the plan's dL/dI(q) buffer (Qc^3 float64)."""
        p = ctypes.c_void_p()
        N.check(N.lib().gw_voxel_grad_buffer(self.handle, ctypes.byref(p)))
        return p.value

    def backward(self, g_iq, iq_on_device=False, want_xyz=False):
        """Vector-Jacobian product of the voxel stage (gw_voxel_backward):
        g_iq is dL/dI(q) on the cropped cube (host array, or a device
        pointer with iq_on_device).  Returns dict(g_f (N,) complex: dL/d of
        every atom's deposited f with the structure constants held fixed,
        g_xyz (N,3) or None, g_sigma float, g_c (n_struct,) complex: dL/d of
        each structure's background constant avg_voxel_f * max_voxels)."""
        n = len(self.xyz)
        g_f = np.empty(2 * n)
        g_xyz = np.empty((n, 3)) if want_xyz else None
        g_sigma = np.zeros(1)
        g_c = np.zeros(2 * len(self.structs))
        if iq_on_device:
            src, flag = ctypes.c_void_p(g_iq), 1
        else:
            g_iq = np.ascontiguousarray(g_iq, dtype=np.float64)
            if g_iq.shape != (self.Qc,) * 3:
                raise ValueError("g_iq must have shape %s" % ((self.Qc,) * 3,))
            src, flag = N.ptr(g_iq), 0
        N.check(N.lib().gw_voxel_backward(self.handle, src, flag, N.ptr(g_f),
                                          N.ptr(g_xyz), N.ptr(g_sigma),
                                          N.ptr(g_c)))
        return dict(g_f=g_f.view(complex), g_xyz=g_xyz, g_sigma=float(g_sigma[0]),
                    g_c=g_c.view(complex))

    def debug_window(self, slice_index):
        """Deposited (Lz, Ly) complex window of one slice and its origin
        (z_lo, y_lo) in grid coordinates (cyclic)."""
        info = self.info()
        out = np.zeros((info["Lz"], info["Ly"]), dtype=np.complex64)
        N.check(N.lib().gw_voxel_debug_window(self.handle, int(slice_index),
                                              N.ptr(out.view(np.float32))))
        return out, info["z_lo"], info["y_lo"]

    def close(self):
        if getattr(self, "handle", None):
            N.lib().gw_voxel_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlanCache:
    """Voxel plans kept after a call for the next call with the same plan
    inputs (geometry, options, phis, structure constants and atom count),
    as FFT libraries keep plans: such a call skips the plan's table set-up
    and allocations; the atoms are uploaded and every slice is computed
    again.  A plan is checked out for the duration of a call (concurrent
    callers never share one), returned afterwards, and the least recently
    returned plans beyond `size` are destroyed.  size 0 disables keeping;
    clear() destroys every kept plan (their device memory is released)."""

    def __init__(self, size=1):
        import collections
        import threading
        self.size = size
        self._lock = threading.Lock()
        self._plans = collections.OrderedDict()

    def checkout(self, geom, structures, **kw):
        spec = VoxelPlan(geom, structures, create=False, **kw)
        key = spec.key()
        with self._lock:
            plan = self._plans.pop(key, None)
        if plan is None:
            spec.create()
            return spec
        plan.xyz, plan.f = spec.xyz, spec.f
        plan.reused = True
        return plan

    def give_back(self, plan, ok=True):
        """Return a checked-out plan; ok False (the call failed) destroys it."""
        if not ok or self.size <= 0 or not plan.handle:
            plan.close()
            return
        drop = []
        with self._lock:
            key = plan.key()
            old = self._plans.pop(key, None)
            if old is not None and old is not plan:
                drop.append(old)
            self._plans[key] = plan
            while len(self._plans) > self.size:
                drop.append(self._plans.popitem(last=False)[1])
        for p in drop:
            p.close()

    def clear(self):
        with self._lock:
            plans = list(self._plans.values())
            self._plans.clear()
        for p in plans:
            p.close()


PLAN_CACHE = PlanCache()
atexit.register(PLAN_CACHE.clear)  # kept plans go before the interpreter tears down


# ------------------------------------------------------------------ slab
class Slab:
    """Owner of a gw_slab: a unit cell tiled and cropped on the device
    (comparison.py:595-671).  cell_xyz (n_cell, 3); vecs the cell vectors
    a, b, c (calc_real_space_abc); size (x, y, z)."""

    def __init__(self, cell_xyz, vecs, size, ctx=None):
        self.ctx = ctx or N.default_context()
        cell = np.ascontiguousarray(cell_xyz, dtype=np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(np.asarray(vecs, dtype=np.float64).reshape(3, 3))
        sz = np.ascontiguousarray(np.asarray(size, dtype=np.float64).reshape(3))
        h = ctypes.c_void_p()
        st = N.lib().gw_slab_create(self.ctx.handle, N.ptr(cell), len(cell),
                                    N.ptr(v), N.ptr(sz), ctypes.byref(h))
        if st != 0:
            msg = N.last_error()
            if "must be greater than" in msg:
                raise AssertionError(msg.split(": ", 1)[-1])
            N.check(st)
        self.handle = h
        n = ctypes.c_int64()
        b = np.zeros(3)
        N.check(N.lib().gw_slab_info(self.handle, ctypes.byref(n), N.ptr(b)))
        self.n = int(n.value)
        self.bounds = b

    def coords(self):
        """(n, 3) float64 coordinates and (n,) cell-atom indices (host)."""
        xyz = np.empty((self.n, 3))
        src = np.empty(self.n, dtype=np.int32)
        N.check(N.lib().gw_slab_get(self.handle, N.ptr(xyz), N.ptr(src), 0))
        return xyz, src

    def device_xyz(self):
        p = ctypes.c_void_p()
        N.check(N.lib().gw_slab_device_xyz(self.handle, ctypes.byref(p)))
        return p.value

    def close(self):
        if getattr(self, "handle", None):
            N.lib().gw_slab_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ detector
def rotation_matrix(u, theta):
    """Rodrigues rotation (utilities.py:222-245), same expression trees."""
    ux, uy, uz = u[0], u[1], u[2]
    R = np.zeros((3, 3))
    R[0, 0] = np.cos(theta) + ux ** 2 * (1 - np.cos(theta))
    R[0, 1] = ux * uy * (1 - np.cos(theta)) - uz * np.sin(theta)
    R[0, 2] = ux * uz * (1 - np.cos(theta)) + uy * np.sin(theta)
    R[1, 0] = uy * ux * (1 - np.cos(theta)) + uz * np.sin(theta)
    R[1, 1] = np.cos(theta) + uy ** 2 * (1 - np.cos(theta))
    R[1, 2] = uy * uz * (1 - np.cos(theta)) - ux * np.sin(theta)
    R[2, 0] = uz * ux * (1 - np.cos(theta)) - uy * np.sin(theta)
    R[2, 1] = uz * uy * (1 - np.cos(theta)) + ux * np.sin(theta)
    R[2, 2] = np.cos(theta) + uz ** 2 * (1 - np.cos(theta))
    return R


class PlaneCorners:
    """The three plane corners [0,0], [0,-1], [-1,0] the reference derives
    rotation axes from (detector.py:58-60, 104-105, 146-147), carried through
    the same fused-chain rotations as the full plane."""

    def __init__(self, h, v):
        self.pts = np.array([[0.0, h[0], v[0]], [0.0, h[-1], v[0]],
                             [0.0, h[0], v[-1]]])

    @classmethod
    def from_grids(cls, x, y, z):
        c = cls.__new__(cls)
        c.pts = np.array([[x[0, 0], y[0, 0], z[0, 0]],
                          [x[0, -1], y[0, -1], z[0, -1]],
                          [x[-1, 0], y[-1, 0], z[-1, 0]]], dtype=np.float64)
        return c

    def matrix(self, kind, angle):
        p1, p2, p3 = self.pts
        if kind == "psi":
            axis = np.cross(p2 - p1, p3 - p1)
        elif kind == "theta":
            axis = p2 - p1
        elif kind == "phi":
            axis = p3 - p1
        else:
            raise ValueError(kind)
        axis /= np.linalg.norm(axis)
        return rotation_matrix(axis, np.radians(angle))

    def rotate(self, R):
        out = PlaneCorners.__new__(PlaneCorners)
        out.pts = N.rotate_points(R, self.pts)
        return out


_IDENTITY = np.eye(3)


class DetectorPlan:
    """Owner of a gw_detector_plan (comparison.py:790-870)."""

    def __init__(self, iq_shape, qx, qy, qz, num_pixels, max_q,
                 angle_init_vals, angle_init_axs, psis, psi_weights, phis,
                 phi_weights, thetas, theta_weights, mirror=True,
                 accum="fp64", exact=False, plane=True, ctx=None):
        self.ctx = ctx or N.default_context()
        nh = nv = int(num_pixels)
        h = np.linspace(-max_q, max_q, nh)
        v = np.linspace(-max_q, max_q, nv)
        self.det_h, self.det_v = h, v
        corners = PlaneCorners(h, v)
        init = []
        for val, ax in zip(angle_init_vals, angle_init_axs):
            if ax in ("psi", "phi", "theta"):
                R = corners.matrix(ax, val)
                corners = corners.rotate(R)
                init.append(R)
        psis, phis, thetas = (np.atleast_1d(np.asarray(a)) for a in
                              (psis, phis, thetas))
        n_rot, mats, weights = [], [], []
        for ps, pw in zip(psis, psi_weights):
            for ph, hw in zip(phis, phi_weights):
                for th, tw in zip(thetas, theta_weights):
                    c = corners
                    k = 0
                    for kind, ang in (("psi", ps), ("phi", ph), ("theta", th)):
                        R = c.matrix(kind, ang)
                        c = c.rotate(R)
                        if not np.array_equal(R, _IDENTITY):
                            mats.append(R)
                            k += 1
                    n_rot.append(k)
                    weights.append(pw * hw * tw)
        if not weights:
            raise ValueError("no detector orientation")
        self.n_orient = len(weights)
        self.iq_shape = tuple(int(s) for s in iq_shape)
        p = N.DetectorParams()
        p.n_h, p.n_v = nh, nv
        for i in range(3):
            p.iq_shape[i] = self.iq_shape[i]
        p.qmin_x, p.qmin_y, p.qmin_z = np.min(qx), np.min(qy), np.min(qz)
        p.dq = np.diff(qz)[0]
        p.mirror = int(bool(mirror))
        p.accum = {"fp64": N.GW_ACCUM_FP64, "kahan32": N.GW_ACCUM_KAHAN32}[accum]
        p.exact = int(bool(exact))
        p.no_plane = int(not plane)
        self.params = p
        self._h = np.ascontiguousarray(h)
        self._v = np.ascontiguousarray(v)
        self._init = np.ascontiguousarray(np.array(init).reshape(-1, 9)) if init else None
        self._nrot = np.ascontiguousarray(np.array(n_rot, dtype=np.int32))
        self._mats = (np.ascontiguousarray(np.array(mats).reshape(-1, 9))
                      if mats else None)
        self._w = np.ascontiguousarray(np.array(weights, dtype=np.float64))
        hdl = ctypes.c_void_p()
        N.check(N.lib().gw_detector_plan_create(
            self.ctx.handle, ctypes.byref(p), N.ptr(self._h), N.ptr(self._v),
            N.ptr(self._init), len(init), N.ptr(self._nrot), N.ptr(self._mats),
            N.ptr(self._w), self.n_orient, ctypes.byref(hdl)))
        self.handle = hdl

    def set_iq(self, iq):
        iq = np.ascontiguousarray(iq, dtype=np.float64)
        if iq.shape != self.iq_shape:
            raise ValueError("iq shape %s != plan shape %s" % (iq.shape, self.iq_shape))
        N.check(N.lib().gw_detector_set_iq(self.handle, N.ptr(iq), 0))

    def set_iq_device32(self, dev_ptr):
        N.check(N.lib().gw_detector_set_iq32_device(self.handle,
                                                    ctypes.c_void_p(dev_ptr)))

    def execute(self):
        N.check(N.lib().gw_detector_execute(self.handle))

    def result(self):
        out = np.empty((self.params.n_v, self.params.n_h))
        N.check(N.lib().gw_detector_get(self.handle, N.ptr(out), 0))
        return out

    def device_result(self):
        """Device address of the image the last execute wrote."""
        p = ctypes.c_void_p()
        N.check(N.lib().gw_detector_device_out(self.handle, ctypes.byref(p)))
        return p.value

    def backward(self, g_image, g_iq_device=None):
        """dL/dI(q) from dL/d(image of result()) (gw_detector_backward).
        Written to the device buffer g_iq_device when given, else returned
        as a host array of the plan's I(q) shape."""
        g = np.ascontiguousarray(g_image, dtype=np.float64)
        if g.shape != (self.params.n_v, self.params.n_h):
            raise ValueError("g_image must have the detector's shape")
        if g_iq_device is not None:
            N.check(N.lib().gw_detector_backward(self.handle, N.ptr(g), 0,
                                                 ctypes.c_void_p(g_iq_device), 1))
            return None
        out = np.empty(self.iq_shape)
        N.check(N.lib().gw_detector_backward(self.handle, N.ptr(g), 0,
                                             N.ptr(out), 0))
        return out

    def debug_indices(self, orient):
        out = np.empty(self.params.n_v * self.params.n_h, dtype=np.int64)
        N.check(N.lib().gw_detector_debug_indices(self.handle, int(orient),
                                                  N.ptr(out)))
        return out

    def close(self):
        if getattr(self, "handle", None):
            N.lib().gw_detector_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
