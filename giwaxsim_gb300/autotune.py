"""Autotuner for the batched voxel plan.

Plan choices that trade work against efficiency, picked by timing them on
the plan's own inputs (graph replays, device events):

  fft_y, fft_z     chirp-z convolution length per axis: the smallest
                   supported length >= L+N-1 (2^k, 3*2^k or 5*2^k) and the
                   next larger one (a power of two may run faster per point
                   than a mixed-radix length that is a little shorter);
  transform        kernel family per axis: the fused chirp-z kernel (two
                   shared-memory exchanges per convolution, where the length
                   has a fused shape) or the Stockham kernels;
  binning          float64 atomic adds or the gather binning (the pixels
                   stored, each voxel summed in a fixed order);
  batch_slices     slices per batch: the L2-sized default, half and double;
  block_variant    block shape of the fused kernels: sequences per block and
                   register cap (occupancy against register spills).

The search is staged (row length, column length, the kernel families of
both axes together, batch, block shape), each stage keeping the best of
the previous ones: the two transform kernels are separate launches whose
times add, but a fused kernel on either axis changes the whole plan (no
real-grid path, atomic binning), so the families are timed as pairs.  Results are cached per device and
plan shape in a JSON file ($GIWAXSIM_GB300_TUNE_CACHE, default
~/.cache/giwaxsim_gb300/tune.json), so a shape is tuned once.  tune()
returns the keyword arguments for VoxelPlan.
"""
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
        "v5", ctx.device_name(), info["Ly"], info["Nc"], info["Lz"], info["Nr"],
        info.get("real", 0),
        info["n_slices"], n_structures, int(bool(fill_bkg)),
        int(bool(smooth)), deposit))


def _as_kwargs(choice):
    out = dict(choice)
    out["transform"] = tuple(out["transform"])
    return out


def tune(make_plan, n_structures, fill_bkg=False, smooth=0,
         deposit="nearest", ctx=None, reps=3, use_cache=True, log=None):
    """Best {fft_y, fft_z, batch_slices, transform, block_variant,
    binning} for the plan make_plan(**choice) builds (make_plan must accept
    those keywords; 0 / "auto" = the defaults).  Every candidate plan gets
    its atoms, one
    warm-up, a captured graph and `reps` timed replays; a candidate the
    library refuses (a fused family for a length without a fused shape) is
    skipped."""
    ctx = ctx or N.default_context()
    default = dict(fft_y=0, fft_z=0, batch_slices=0,
                   transform=("auto", "auto"), block_variant=0, binning="auto")
    base = make_plan(**_as_kwargs(default))
    try:
        info = base.info()
    finally:
        base.close()
    key = shape_key(ctx, info, n_structures, fill_bkg, smooth, deposit)
    if use_cache:
        with _lock:
            hit = _load().get(key)
        if hit:
            return _as_kwargs(hit["choice"])

    timed = {}

    def time_choice(choice):
        k = json.dumps(choice, sort_keys=True)
        if k in timed:
            return timed[k]
        try:
            plan = make_plan(**_as_kwargs(choice))
        except N.GwError as e:
            if e.status != N.GW_ERR_ARG:
                raise
            timed[k] = None
            return None
        try:
            plan.set_atoms()
            plan.execute()
            ctx.synchronize()
            plan.capture_graph()
            plan.execute()
            ms = ctx.time_ms(plan.execute, reps)
        finally:
            plan.close()
        timed[k] = ms
        if log:
            log("tune %s: %.4f ms" % (choice, ms))
        return ms

    def best_of(cands):
        res = [(time_choice(c), c) for c in cands]
        res = [r for r in res if r[0] is not None]
        return min(res, key=lambda r: r[0])

    best = dict(default, fft_y=info["My"], fft_z=info["Mz"],
                batch_slices=info["batch"])
    default_ms = time_choice(best)
    # transform lengths, rows then columns, with the default kernels
    ys = length_candidates(info["Ly"] + info["Nc"] - 1)
    _, best = best_of([dict(best, fft_y=m) for m in ys])
    zs = length_candidates(info["Lz"] + info["Nr"] - 1)
    _, best = best_of([dict(best, fft_z=m) for m in zs])
    # kernel families of both axes together: a fused kernel on either axis
    # takes the plan off the real-grid path and off gather binning, so the
    # axes are not independent
    _, best = best_of([dict(best, transform=[fy, fz])
                       for fy in ("auto", "fused") for fz in ("auto", "fused")])
    # binning: atomic float64 adds or gather (refused where it does not
    # apply); auto is one of the two
    _, best = best_of([dict(best, binning=b) for b in ("atomic", "gather")])
    # slices per batch
    S = info["batch"]
    batches = sorted({S, max(1, S // 2), min(info["n_slices"], 2 * S, 4096)})
    _, best = best_of([dict(best, batch_slices=b) for b in batches])
    # block shape of the fused kernels
    if "fused" in best["transform"]:
        _, best = best_of([dict(best, block_variant=v)
                           for v in range(N.fused_variant_count())])
    ms = time_choice(best)
    if use_cache:
        with _lock:
            cache = _load()
            cache[key] = {"choice": best, "ms": ms, "default_ms": default_ms,
                          "candidates": len(timed)}
            _store(cache)
    return _as_kwargs(best)
