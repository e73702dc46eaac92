"""Autotuner for the batched voxel plan.

Three plan choices trade work against efficiency and are picked by timing
them on the plan's own inputs (graph replays, device events):

  fft_y, fft_z   chirp-z convolution length per axis: the smallest supported
                 length >= L+N-1 (2^k, 3*2^k or 5*2^k) and the next two
                 larger ones (a power of two may run faster per point than a
                 mixed-radix length that is a little shorter);
  batch_slices   slices per batch: the L2-sized default, half and double.

Results are cached per device and plan shape in a JSON file
($GIWAXSIM_GB300_TUNE_CACHE, default ~/.cache/giwaxsim_gb300/tune.json), so a
shape is tuned once.  tune() returns the keyword arguments for VoxelPlan.
"""
import itertools
import json
import os
import threading

from . import _native as N

# the transform lengths the library instantiates (kFftSizes in gw_fft.cuh)
FFT_SIZES = (64, 128, 256, 384, 512, 640, 768, 1024, 1280, 1536, 2048, 2560,
             3072, 4096, 5120, 6144, 8192)

_lock = threading.Lock()


def cache_path():
    return os.environ.get("GIWAXSIM_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache",
                                       "giwaxsim_gb300", "tune.json"))


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(cache):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = "%s.%d" % (path, os.getpid())
        with open(tmp, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only costs re-tuning


def length_candidates(need, count=2):
    """The `count` smallest supported lengths >= need."""
    return [m for m in FFT_SIZES if m >= need][:count]


def shape_key(ctx, info, n_structures, fill_bkg, smooth, deposit):
    return "|".join(str(x) for x in (
        ctx.device_name(), info["Ly"], info["Nc"], info["Lz"], info["Nr"],
        info["n_slices"], n_structures, int(bool(fill_bkg)),
        int(bool(smooth)), deposit))


def tune(make_plan, n_structures, fill_bkg=False, smooth=0,
         deposit="nearest", ctx=None, reps=3, use_cache=True, log=None):
    """Best {fft_y, fft_z, batch_slices} for the plan make_plan(**choice)
    builds (make_plan must accept those three keywords; 0 = automatic).
    Every candidate plan gets its atoms, one warm-up, a captured graph and
    `reps` timed replays."""
    ctx = ctx or N.default_context()
    base = make_plan(fft_y=0, fft_z=0, batch_slices=0)
    try:
        info = base.info()
    finally:
        base.close()
    key = shape_key(ctx, info, n_structures, fill_bkg, smooth, deposit)
    if use_cache:
        with _lock:
            hit = _load().get(key)
        if hit:
            return dict(hit["choice"])
    ys = length_candidates(info["Ly"] + info["Nc"] - 1)
    zs = length_candidates(info["Lz"] + info["Nr"] - 1)
    S = info["batch"]
    batches = sorted({S, max(1, S // 2), min(info["n_slices"], 2 * S, 4096)})
    results = []
    for fy, fz, b in itertools.product(ys, zs, batches):
        choice = dict(fft_y=fy, fft_z=fz, batch_slices=b)
        plan = make_plan(**choice)
        try:
            plan.set_atoms()
            plan.execute()
            ctx.synchronize()
            plan.capture_graph()
            plan.execute()
            ms = ctx.time_ms(plan.execute, reps)
        finally:
            plan.close()
        results.append((ms, choice))
        if log:
            log("tune %s: %.4f ms" % (choice, ms))
    ms, best = min(results, key=lambda r: r[0])
    if use_cache:
        with _lock:
            cache = _load()
            cache[key] = {"choice": best, "ms": ms,
                          "default_ms": next(m for m, c in results
                                             if c == dict(fft_y=ys[0], fft_z=zs[0],
                                                          batch_slices=S)),
                          "candidates": len(results)}
            _store(cache)
    return dict(best)
