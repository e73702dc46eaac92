"""Benchmark of the GIWAXS forward path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload si-100A]

A step is one full voxel stage over every phi slice of the workload (all
slices -> cropped I(q) with counts, average and f0).  Headline metric:
slices/s.  The same JSON line also carries the seconds per detector image
(voxel stage + detector, batched and plain), the roofline of the dominant
kernel, the CPU baseline (the float64 numpy oracle on the host cores), the
SM clocks sampled during the timed region, and e2e (the public drop-in API
voxelgridmaker_fitting on host numpy arrays, copies included).

Multi-GPU: the path has no exchange step; each rank runs an independent
replica of the workload (weak scaling), rank 0 prints.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "slices/s & s/detector image: batched vs plain on 1 GB300 at <=1e-5 rel err vs FP64"
L2_BYTES = 129 * 1024 * 1024

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per slice of the
# two transform kernels, keyed by (workload, kernel, fft_y, fft_z, real
# grids), from one ncu --set full capture of a launch of that kernel on the
# same workload and plan shape (complex grids and atomic binning: a 51-slice
# launch; real grids and gather binning: a 102-slice launch); a launch's
# traffic is this times its slices (both kernels move per-slice data only).
NCU_TRAFFIC = {("si-100A", "row_czt", 1280, 1024, 0): (1.48 + 38.03) * 1e6 / 51,
               ("si-100A", "col_czt_bin", 1280, 1024, 0): (148.42 + 28.70) * 1e6 / 51,
               ("si-100A", "row_czt", 1280, 1024, 1): (1.76 + 42.04) * 1e6 / 102,
               ("si-100A", "col_czt_bin", 1280, 1024, 1): (83.23 + 15.57) * 1e6 / 102}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="si-100A")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the five-workload batched/plain table")
    ap.add_argument("--no-tune", action="store_true",
                    help="use the default transform lengths and batch size")
    ap.add_argument("--no-grad", action="store_true",
                    help="skip the forward+backward timing")
    ap.add_argument("--phis", type=int, default=0,
                    help="use this many slices instead of the workload's")
    ap.add_argument("--profile", action="store_true",
                    help="one eager voxel pass and one detector pass, no "
                         "timing (for ncu)")
    ap.add_argument("--transform", default="auto",
                    choices=["auto", "stockham", "fused"],
                    help="chirp-z kernel family of --profile's plan")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
            except (ValueError, IndexError):
                continue
            for k, n in enumerate(names):
                if len(s) > 3 + k and s[3 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        # one process per GPU over NCCL; gloo where no GPU is present (the
        # host-side logic is exercised that way)
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ workload
def load_workload(name, n_phi=0):
    from giwaxsim_gb300 import forward as F
    from giwaxsim_gb300 import workloads as W
    w = W.WORKLOADS[name]
    structs = W.structures(name)
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = W.phis_linspace(n_phi or w["n_phi"])
    items = [(xyz, F.element_f_values(el, w["energy"]), wt)
             for xyz, el, wt in structs]
    return w, structs, geom, phis, items


def detector_args(w, geom):
    init_vals, init_axs = w["init"]
    a, b, n = w["psis"]
    psis = np.linspace(a, b, n)
    one = np.array([0.0])
    return dict(num_pixels=w["num_pixels"], max_q=w["max_q"],
                angle_init_vals=init_vals, angle_init_axs=init_axs, psis=psis,
                psi_weights=np.ones_like(psis) / len(psis), phis=one,
                phi_weights=one + 1.0, thetas=one, theta_weights=one + 1.0)


# ------------------------------------------------------------------ gb300 arm
def run_gb300(args, world, rank, local, pg):
    from giwaxsim_gb300 import _native as N
    from giwaxsim_gb300 import forward as F
    from giwaxsim_gb300.tools import comparison

    w, structs, geom, phis, items = load_workload(args.workload, args.phis)
    ctx = N.Context(local)
    n_slices = len(items) * len(phis)
    if args.profile:
        run_profile(args, w, geom, phis, items, ctx)
        return
    plan = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                       smooth=w["smooth"], tune=not args.no_tune, ctx=ctx)
    plan.set_atoms()
    plan.execute()
    ctx.synchronize()
    plan.capture_graph()
    info = plan.info()
    # L2 flush buffer (written between timed iterations, outside the events)
    flush = None
    try:
        import torch
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32,
                            device="cuda:%d" % local)
    except Exception:
        flush = None

    stream = ctx.stream()
    import torch
    ts = torch.cuda.ExternalStream(stream, device="cuda:%d" % local)

    def do_flush():
        if flush is not None:
            with torch.cuda.stream(ts):
                flush.fill_(1.0)

    for _ in range(args.warmup):
        plan.execute()
    ctx.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launch_count()
    evs = []
    for _ in range(args.steps):
        do_flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ts)
        plan.execute()
        e1.record(ts)
        evs.append((e0, e1))
    ctx.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    t_ms = sum(a.elapsed_time(b) for a, b in evs)
    t_ms = max_over_ranks(pg, t_ms)
    barrier(pg)
    ms_per_step = t_ms / args.steps
    value = world * n_slices * args.steps / (t_ms / 1e3)

    # detector (batched) on the device-resident float32 I(q)
    dargs = detector_args(w, geom)
    q = geom.q_crop
    det = F.DetectorPlan((plan.Qc,) * 3, q, q, q, dargs["num_pixels"],
                         dargs["max_q"], dargs["angle_init_vals"],
                         dargs["angle_init_axs"], dargs["psis"],
                         dargs["psi_weights"], dargs["phis"],
                         dargs["phi_weights"], dargs["thetas"],
                         dargs["theta_weights"], mirror=True, ctx=ctx)
    det.set_iq_device32(plan.device_iq32())
    for _ in range(2):
        det.execute()
    ctx.synchronize()
    d0 = torch.cuda.Event(enable_timing=True)
    d1 = torch.cuda.Event(enable_timing=True)
    d0.record(ts)
    nd = max(1, args.steps)
    for _ in range(nd):
        det.execute()
    d1.record(ts)
    torch.cuda.synchronize()
    det_ms = d0.elapsed_time(d1) / nd

    # per-kernel device times (eager, instrumented replica of the same work)
    eager = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                        smooth=w["smooth"], **plan_choice(plan), ctx=ctx)
    eager.set_atoms()
    eager.execute()
    ctx.synchronize()
    ctx.set_timing(True)
    eager.execute()
    det.execute()
    kt = ctx.kernel_times()
    ctx.set_timing(False)
    eager.close()

    # plain per-rotation path: one slice per launch sequence, full grid,
    # timed over every slice of the workload
    plain = None
    if not args.no_plain:
        plain_ms = plain_path_ms(geom, w, items, phis, ctx, ts)
        plain = n_slices / (plain_ms / 1e3)

    # e2e through the public API with host arrays
    e2e = None
    if len(items) == 1:
        xyz, el, wt = structs[0]
        t_e = []
        # two untimed calls first: the host result buffers the API recycles
        # (forward.HOST_POOL) and the plan it keeps for calls with the same
        # plan inputs (forward.PLAN_CACHE) exist from then on; every timed
        # call uploads the atoms, computes all slices and copies I(q) out
        for k in range(2 + max(3, min(args.steps, 5))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            iq, qx, qy, qz = comparison.voxelgridmaker_fitting(
                xyz, el, w["r"], w["dq"], w["max_q"], w["energy"],
                fill_bkg=w["fill_bkg"], smooth=w["smooth"], phis=phis,
                weights=wt, ctx=ctx)
            t_e.append(time.perf_counter() - t0)
        te = float(np.mean(t_e[2:]))
        # where the e2e time goes: the same steps as the call, each timed,
        # averaged over as many calls; "plan_s" is the plan inputs and the
        # kept plan's lookup (forward.PLAN_CACHE), "fresh_plan_s" what a
        # plan made from scratch costs
        ph = {k: [] for k in ("inputs_s", "plan_s", "upload_execute_s",
                              "d2h_s", "give_back_s")}
        for k in range(len(t_e) - 2):
            out = None
            t0 = time.perf_counter()
            g2 = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
            c2 = np.asarray(xyz, dtype=np.float64)
            rg = F.coord_ranges(c2)
            g2.check_bounds(c2, rg)
            fv = F.element_f_values(el, w["energy"])
            t1 = time.perf_counter()
            pl = F.PLAN_CACHE.checkout(g2, [(c2, fv, wt)], phis=phis,
                                       fill_bkg=w["fill_bkg"],
                                       smooth=w["smooth"], ctx=ctx,
                                       ranges=[rg])
            t2 = time.perf_counter()
            pl.set_atoms()
            pl.execute()
            ctx.synchronize()
            t3 = time.perf_counter()
            out = pl.iq()  # the result array as the API returns it (HostPool)
            t4 = time.perf_counter()
            F.PLAN_CACHE.give_back(pl)
            t5 = time.perf_counter()
            for key, v in zip(ph, (t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4)):
                ph[key].append(v)
            del out
        ph = {k: float(np.mean(v)) for k, v in ph.items()}
        t0 = time.perf_counter()
        pl = F.VoxelPlan(geom, [(xyz, F.element_f_values(el, w["energy"]), wt)],
                         phis=phis, fill_bkg=w["fill_bkg"], smooth=w["smooth"],
                         ctx=ctx)
        ph["fresh_plan_s"] = time.perf_counter() - t0
        pl.close()
        F.PLAN_CACHE.clear()
        e2e = {"value": world * n_slices / te, "unit": "slices/s",
               "h2d_bytes_per_step": int(xyz.size * 8 + len(xyz) * 8),
               "d2h_bytes_per_step": int(iq.size * 8),
               "s_per_step": te, "s_per_call": [round(v, 6) for v in t_e],
               "phases": ph}

    # rooflines: the dominant kernel (`roofline`) and every stage kernel
    # (`rooflines`: row and column transforms with the binning, finalize,
    # detector), from the eager per-kernel event times
    peak, peak_kind = measured_peaks()

    # voxels with a count (the finalize reads their sums only)
    cnt = plan.counts()
    counted = (int(np.count_nonzero(cnt)), int(cnt.sum()))

    def kernel_roof(name):
        ms_tot, nl = kt[name]
        avg_ms = ms_tot / max(nl, 1)
        # slices per launch of the batched kernels: the batches' average
        spl = n_slices / nl if name in ("row_czt", "col_czt_bin") else None
        algo = algorithmic_bytes(name, info, w, spl, dargs, plan.Qc, counted)
        if not algo:
            return None
        achieved = algo / (avg_ms / 1e3) / 1e9
        tkey = (args.workload, name, info["My"], info["Mz"], info.get("real", 0))
        traffic = NCU_TRAFFIC[tkey] * spl if tkey in NCU_TRAFFIC else None
        r = {"kernel": name, "bound": "hbm", "achieved": achieved,
             "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
             "frac": achieved / peak, "traffic": traffic,
             "traffic_source": "ncu capture of one launch, scaled by slices "
                               "per launch" if traffic else None,
             "avg_launch_ms": avg_ms, "launches": nl,
             "slices_per_launch": spl, "algorithmic_bytes_per_launch": algo}
        if name in ("row_czt", "col_czt_bin"):
            # the transforms' own limiter: shared-memory passes
            r["shared"] = shared_roof(name, info, spl, avg_ms)
        return r

    rooflines = {k: kernel_roof(k) for k in ("row_czt", "col_czt_bin",
                                             "finalize", "detector") if k in kt}
    top = max(kt.items(), key=lambda kv: kv[1][0])[0] if kt else None
    roof = rooflines.get(top) if top else None
    kernel_share = {k: {"ms": round(v[0], 4), "launches": v[1]}
                    for k, v in kt.items()}

    # the five workloads: seconds per detector image, batched vs plain
    table = None
    if not args.no_workloads:
        table = {}
        for name in WORKLOAD_NAMES:
            table[name] = workload_summary(name, ctx, ts, do_flush,
                                           tune=not args.no_tune)
    grad = None if args.no_grad else grad_timing(ctx)

    # CPU baseline and accuracy: one pass of the float64 oracle over every
    # slice (timed), then its detector image; the GPU's I(q), counts and
    # image are compared with them outside every timed region
    cpu = accuracy = None
    if rank == 0 and not args.no_cpu_baseline and len(items) == 1:
        ref = oracle_voxel(w, geom, phis, items)
        cpu = {"value": ref["slices"] / ref["seconds"], "unit": "slices/s",
               "cores": ref["cores"], "threads": ref["threads"], "kind": "port",
               "sample": "all %d slices of %s, one pass (float64 numpy oracle, "
                         "%d threads), %.1f s" % (ref["slices"], args.workload,
                                                  ref["threads"], ref["seconds"])}
        t0 = time.perf_counter()
        dref = oracle_detector(ref["iq"], ref["q"], dargs, ref["threads"])
        t_det = time.perf_counter() - t0
        accuracy = {
            "reference": "float64 numpy oracle, all %d slices, %d px x %d "
                         "orientations" % (n_slices, dargs["num_pixels"],
                                           int(det.n_orient)),
            "iq": compare(plan.iq(), ref["iq"]),
            "counts_bit_exact": bool(np.array_equal(plan.counts(), ref["count"])),
            "detector": compare(det.result(), dref),
            "oracle_detector_s": round(t_det, 2)}
        accuracy["meets_1e-5"] = (accuracy["iq"]["rel_l2"] <= 1e-5 and
                                  accuracy["detector"]["rel_l2"] <= 1e-5 and
                                  accuracy["counts_bit_exact"])
        del ref, dref

    out = {
        "metric": METRIC, "value": value, "unit": "slices/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 accum)",
        "data": "synthetic (seeded structure generator, f = Z)",
        "config": {"workload": args.workload, "atoms": int(len(plan.xyz)),
                   "grid_size": geom.grid_size, "crop": plan.Qc,
                   "slices_per_step": n_slices,
                   "detector_px": w["num_pixels"],
                   "orientations": int(det.n_orient),
                   "l2": "flushed between timed iterations (2x L2 write)",
                   "plan": info, "tuned": plan.tuned and dict(
                       plan.tuned, transform=list(plan.tuned["transform"]))},
        "s_per_detector_image": {
            "batched": ms_per_step / 1e3 / len(items) + det_ms / 1e3,
            "detector_only_s": det_ms / 1e3,
            "plain": (n_slices / plain / len(items) + det_ms / 1e3) if plain else None},
        "plain_slices_per_s": plain,
        # seconds per detector image, plain over batched (the detector
        # the same on both); the voxel stage alone in slices_batched_vs_plain
        "batched_vs_plain": ((n_slices / plain / len(items) + det_ms / 1e3)
                             / (ms_per_step / 1e3 / len(items) + det_ms / 1e3))
                            if plain else None,
        "slices_batched_vs_plain": (value / world / plain) if plain else None,
        "gpu_launches": int(launches),
        "e2e": e2e, "roofline": roof, "rooflines": rooflines,
        "kernel_ms": kernel_share,
        "cpu_baseline": cpu, "accuracy": accuracy, "clocks": clk,
        "workloads": table, "gradient": grad,
    }
    if rank == 0:
        print(json.dumps(out))
    for p_ in (det, plan):
        p_.close()


WORKLOAD_NAMES = ("graphite-50A", "si-100A", "graphite-64", "si-60A-occ",
                  "lamellar-200A")


def fft_passes(m):
    """Stockham passes of a length-m transform (radix-16 passes, then the
    power-of-two remainder, then the odd factor 3 or 5)."""
    odd = m
    while odd % 2 == 0:
        odd //= 2
    l2 = (m // odd).bit_length() - 1
    return l2 // 4 + (1 if l2 % 4 else 0) + (1 if odd > 1 else 0)


def shared_roof(name, info, spl, avg_ms):
    """Shared-memory traffic of a transform kernel's Stockham passes (one
    read and one write of every point per pass, forward and inverse) per
    launch, against the nominal shared bandwidth."""
    m = info["My"] if name == "row_czt" else info["Mz"]
    # real grids: two window rows per row transform, columns ky >= 0 only
    rows = info["Lz"] / 2 if info.get("real") else info["Lz"]
    units = spl * (rows if name == "row_czt" else f1_columns(info))
    sb = units * 2 * fft_passes(m) * m * 16
    speak = 152 * 128 * 2070e6 / 1e12
    return {"achieved": sb / (avg_ms / 1e3) / 1e12, "peak": speak,
            "unit": "TB/s", "frac": sb / (avg_ms / 1e3) / 1e12 / speak,
            "peak_kind": "nominal: 152 SMs x 128 B/clk x 2070 MHz",
            "bytes_per_launch": sb}


def _event_ms(ts, fn, reps, flush=None):
    import torch
    tot = 0.0
    for _ in range(reps):
        if flush:
            flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ts)
        fn()
        e1.record(ts)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    return tot / reps


def plan_choice(plan):
    """The tuned choices of a plan (lengths, batch, kernel family per axis,
    block shape, binning) as VoxelPlan keywords, for a replica of it."""
    p = plan.params
    fam = {0: "auto", 1: "stockham", 2: "fused"}
    binning = {0: "auto", 1: "atomic", 2: "gather"}
    return dict(fft_y=p.fft_y, fft_z=p.fft_z, batch_slices=p.batch_slices,
                transform=(fam[p.transform_y], fam[p.transform_z]),
                block_variant=p.block_variant, binning=binning[p.binning])


def plain_path_ms(geom, w, items, phis, ctx, ts, reps=2):
    """Device time of the plain per-rotation path (one slice per launch
    sequence, full grid and transform, binning into the whole cube) over
    every slice of every structure, ms (mean of `reps` executions)."""
    from giwaxsim_gb300 import forward as F
    pp = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                     smooth=w["smooth"], mode="plain", ctx=ctx)
    pp.set_atoms()
    pp.execute()
    ctx.synchronize()
    t = _event_ms(ts, pp.execute, reps)
    pp.close()
    return t


def workload_summary(name, ctx, ts, flush, reps=3, tune=True):
    """Seconds per detector image of one workload: batched (graph replay of
    the voxel stage over all slices + detector) and plain (the per-rotation
    path over all slices + detector)."""
    from giwaxsim_gb300 import forward as F
    w, structs, geom, phis, items = load_workload(name)
    n_slices = len(items) * len(phis)
    plan = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                       smooth=w["smooth"], tune=tune, ctx=ctx)
    plan.set_atoms()
    plan.execute()
    ctx.synchronize()
    plan.capture_graph()
    plan.execute()
    ctx.synchronize()
    vox_ms = _event_ms(ts, plan.execute, reps, flush)
    dargs = detector_args(w, geom)
    q = geom.q_crop
    det = F.DetectorPlan((plan.Qc,) * 3, q, q, q, dargs["num_pixels"],
                         dargs["max_q"], dargs["angle_init_vals"],
                         dargs["angle_init_axs"], dargs["psis"],
                         dargs["psi_weights"], dargs["phis"],
                         dargs["phi_weights"], dargs["thetas"],
                         dargs["theta_weights"], mirror=True, ctx=ctx)
    det.set_iq_device32(plan.device_iq32())
    det.execute()
    ctx.synchronize()
    det_ms = _event_ms(ts, det.execute, reps)
    info = plan.info()
    det_ref = det.result() if len(items) > 1 else None
    det.close()
    # the Kahan-compensated float32 accumulation beside float64 (the
    # multi-structure workload compares them): time and normwise difference
    kahan = None
    if len(items) > 1:
        dk = F.DetectorPlan((plan.Qc,) * 3, q, q, q, dargs["num_pixels"],
                            dargs["max_q"], dargs["angle_init_vals"],
                            dargs["angle_init_axs"], dargs["psis"],
                            dargs["psi_weights"], dargs["phis"],
                            dargs["phi_weights"], dargs["thetas"],
                            dargs["theta_weights"], mirror=True,
                            accum="kahan32", ctx=ctx)
        dk.set_iq_device32(plan.device_iq32())
        dk.execute()
        ctx.synchronize()
        dk_ms = _event_ms(ts, dk.execute, reps)
        dimg = dk.result()
        dk.close()
        ref = plan.iq()
        pk = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                         smooth=w["smooth"], accum="kahan32",
                         **plan_choice(plan), ctx=ctx)
        pk.set_atoms()
        pk.execute()
        ctx.synchronize()
        pk.capture_graph()
        pk.execute()
        ctx.synchronize()
        k_ms = _event_ms(ts, pk.execute, reps, flush)
        ik = pk.iq()
        kahan = {"voxel_ms": round(k_ms, 4),
                 "rel_l2_vs_fp64": float(np.linalg.norm(ik - ref) / np.linalg.norm(ref)),
                 "detector_ms": round(dk_ms, 4),
                 "detector_rel_l2_vs_fp64":
                     float(np.linalg.norm(dimg - det_ref) / np.linalg.norm(det_ref))}
        del ik, ref
        pk.close()
    plan.close()
    # plain: the per-rotation path over every slice of every structure
    plain_ms = plain_path_ms(geom, w, items, phis, ctx, ts)
    batched = (vox_ms + det_ms) / 1e3
    plain = (plain_ms + det_ms) / 1e3
    return {"slices": n_slices, "atoms": int(sum(len(x[0]) for x in items)),
            "grid": geom.grid_size, "crop": info["crop"],
            "fft_y": info["My"], "fft_z": info["Mz"], "batch": info["batch"],
            "tuned": plan.tuned is not None,
            "voxel_ms": round(vox_ms, 4), "detector_ms": round(det_ms, 4),
            "slices_per_s": n_slices / (vox_ms / 1e3),
            "s_per_image_batched": batched, "s_per_image_plain": plain,
            "plain_ms": round(plain_ms, 4),
            "plain_sample_slices": n_slices, "batched_vs_plain": plain / batched,
            "kahan32": kahan}


def grad_timing(ctx, steps=3):
    """Forward + backward of the scale/offset misfit on si-60A-occ
    (bilinear deposit, checkpoint interval 16): wall seconds per step."""
    import torch
    from giwaxsim_gb300 import workloads as W
    from giwaxsim_gb300.autograd import (DetectorModel, detector_image,
                                         scale_offset_misfit)
    w = W.WORKLOADS["si-60A-occ"]
    (xyz, el, hidden), = W.structures("si-60A-occ")
    model = DetectorModel(el, w["energy"], w["r"], w["dq"], w["max_q"],
                          w["num_pixels"], psis=np.linspace(*w["psis"]),
                          phis=W.phis_linspace(w["n_phi"]), deposit="bilinear",
                          checkpoint_every=16, ctx=ctx)
    target = torch.from_numpy(model.forward(xyz, hidden, 1.5)[0])
    X = torch.tensor(xyz, requires_grad=True)
    fw, bw = [], []
    for k in range(steps + 1):
        occ = torch.ones(len(xyz), dtype=torch.float64, requires_grad=True)
        sig = torch.tensor(1.2, dtype=torch.float64, requires_grad=True)
        t0 = time.perf_counter()
        loss, _, _ = scale_offset_misfit(detector_image(model, occ, sig, X),
                                         target)
        t1 = time.perf_counter()
        loss.backward()
        t2 = time.perf_counter()
        if k:
            fw.append(t1 - t0)
            bw.append(t2 - t1)
    model.close()
    f, b = float(np.mean(fw)), float(np.mean(bw))
    return {"workload": "si-60A-occ", "deposit": "bilinear",
            "checkpoint_every": 16, "atoms": int(len(xyz)),
            "parameters": int(4 * len(xyz) + 1), "forward_s": f,
            "backward_s": b, "step_s": f + b,
            "backward_over_forward": b / f}


def run_profile(args, w, geom, phis, items, ctx):
    """One eager pass of the voxel stage and one detector image."""
    from giwaxsim_gb300 import forward as F
    plan = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                       smooth=w["smooth"], transform=args.transform, ctx=ctx)
    plan.set_atoms()
    plan.execute()
    ctx.synchronize()
    dargs = detector_args(w, geom)
    q = geom.q_crop
    det = F.DetectorPlan((plan.Qc,) * 3, q, q, q, dargs["num_pixels"],
                         dargs["max_q"], dargs["angle_init_vals"],
                         dargs["angle_init_axs"], dargs["psis"],
                         dargs["psi_weights"], dargs["phis"],
                         dargs["phi_weights"], dargs["thetas"],
                         dargs["theta_weights"], mirror=True, ctx=ctx)
    det.set_iq_device32(plan.device_iq32())
    det.execute()
    ctx.synchronize()
    print(json.dumps({"profile": args.workload, "slices": len(phis) * len(items),
                      "plan": plan.info(), "orientations": det.n_orient}))
    det.close()
    plan.close()


def f1_columns(info):
    """Columns of the row stage's output F1: the band's Nc, or with real
    grids the columns ky >= 0 (from m_zero = -k0 on)."""
    return info["Nc"] + info["k0"] if info.get("real") else info["Nc"]


def algorithmic_bytes(name, info, w, S, dargs, Qc, counted=(None, None)):
    """Bytes a launch of `name` must move at minimum (its inputs read once,
    outputs written once), per the plan's sizes; S = slices per launch.
    The row stage's input is the window grid (complex; real with real
    grids), its output F1; the column stage reads F1 and read-modify-writes
    a float64 sum of every band pixel."""
    nf = f1_columns(info)
    if name == "row_czt":
        return S * info["Lz"] * (info["Ly"] * (4 if info.get("real") else 8) + nf * 8)
    if name == "col_czt_bin":
        if info.get("gather"):
            # F1 read + every pixel stored once (float32) for the gather
            return S * (info["Lz"] * nf * 8 + info["Nr"] * nf * 4)
        # F1 read + float64 read-modify-write of every band pixel
        return S * (info["Lz"] * nf * 8 + info["Nr"] * info["Nc"] * 16)
    if name == "detector":
        npx = dargs["num_pixels"] ** 2
        return len(dargs["psis"]) * npx * 4 + npx * 8
    nonzero, binned = counted
    if name == "finalize" and info.get("gather"):
        # every binned pixel read once (float32), the float32 I(q) of every
        # voxel written (the line and z tables are a few MB)
        return (Qc ** 3 if binned is None else binned) * 4 + Qc ** 3 * 4
    if name == "finalize":
        # the float64 sum of every voxel with a count, the float32 I(q) of
        # every voxel (the count factor tables are a few KB)
        return (Qc ** 3 if nonzero is None else nonzero) * 8 + Qc ** 3 * 4
    return None


# ------------------------------------------------------------------ CPU
def oracle_voxel(w, geom, phis, items, workers=None):
    """The float64 numpy oracle over every slice of a single-structure
    workload, threaded over slices like the reference's ThreadPoolExecutor
    (comparison.py:759-763).  Returns the cropped I(q) with the f0 factor,
    the count grid and the wall time of the whole pass."""
    from oracle import giwaxs_oracle as O
    xyz, fv, wt = items[0]
    fvw = fv if wt is None else fv * wt
    cores = os.cpu_count() or 1
    workers = workers or min(32, cores + 4)
    t0 = time.perf_counter()
    out = O.voxelgrid_crop_threaded(xyz, fvw, w["r"], w["dq"], w["max_q"],
                                    phis, w["fill_bkg"], w["smooth"], workers)
    out.update(seconds=time.perf_counter() - t0, threads=workers, cores=cores,
               slices=len(phis))
    return out


def oracle_detector(iq, qc, dargs, workers):
    """The oracle's detector image (comparison.py:790-870) of a float64
    I(q), its orientations summed on `workers` threads."""
    from oracle import giwaxs_oracle as O
    return O.detector_threaded(iq, qc, qc, qc, dargs["num_pixels"],
                               dargs["max_q"], dargs["angle_init_vals"],
                               dargs["angle_init_axs"], dargs["psis"],
                               dargs["psi_weights"], dargs["phis"],
                               dargs["phi_weights"], dargs["thetas"],
                               dargs["theta_weights"], True, workers)[0]


def compare(gpu, ref):
    """Per-output error of a GPU result against the float64 oracle:
    normwise relative L2, max |diff| / max |ref|, and the p50/p99 of the
    elementwise relative error over the nonzero reference values."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    d = np.abs(gpu - ref)
    nz = ref != 0
    rel = d[nz] / np.abs(ref[nz])
    return {"rel_l2": float(np.linalg.norm(gpu - ref) / np.linalg.norm(ref)),
            "max_abs_over_max": float(d.max() / np.abs(ref).max()),
            "p50_rel": float(np.percentile(rel, 50)),
            "p99_rel": float(np.percentile(rel, 99)),
            "zero_where_ref_zero": bool(np.all(gpu[~nz] == 0))}


def run_reference(args, world, rank, local, pg):
    """The reference arm: the float64 numpy oracle (the reference's path
    restated) on the host cores, every step the whole workload (all slices
    of the voxel stage), threaded like the reference."""
    if rank != 0:
        return
    w, structs, geom, phis, items = load_workload(args.workload, args.phis)
    for _ in range(args.warmup):
        oracle_voxel(w, geom, phis, items)
    secs = []
    for _ in range(args.steps):
        r = oracle_voxel(w, geom, phis, items)
        secs.append(r["seconds"])
    n = len(phis) * len(items)
    t = float(np.sum(secs))
    value = n * args.steps / t
    cb = {"value": value, "unit": "slices/s", "cores": r["cores"],
          "threads": r["threads"], "kind": "port",
          "sample": "%d full steps of %d slices of %s (float64 numpy oracle, "
                    "%d threads), %.1f s timed" % (args.steps, n,
                                                    args.workload,
                                                    r["threads"], t)}
    out = {"metric": METRIC, "impl": "reference", "value": value,
           "unit": "slices/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded structure generator, f = Z)",
           "config": {"workload": args.workload, "slices_per_step": n},
           "cpu_baseline": cb,
           "e2e": {"value": value, "unit": "slices/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    # synthetic workloads: f = Z for every atom (f' = f'' = 0), as stated
    # in the line's "data"; xraydb is not installed on the GPU machine
    from giwaxsim_gb300.tools import utilities
    utilities.use_zero_f1f2()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, local, pg)
    else:
        run_gb300(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
