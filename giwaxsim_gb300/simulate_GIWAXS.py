"""Config-file driver with the reference's interface (simulate_GIWAXS.py).

    python -m giwaxsim_gb300.simulate_GIWAXS --config cfg.txt

Keys and defaults are the reference's (simulate_GIWAXS.py:19-82, README.md
41-94), including its quirks: `smooth` is parsed with int(), `num_pixels`
defaults to max_q/q_voxel_size, a zero slab size falls back to a, b, c.
Additional optional keys (defaults reproduce the reference):

  phi_slices      number of phi slices instead of the automatic count
  average_inputs  True: with input_folder, average I(q) over all files
                  before the detector (legacy voxelgridmaker behaviour)
  accum           fp64 | kahan32
  mode            batched | plain

Outputs per structure: det_h.npy, det_v.npy, det_sum.npy, config.txt (and
PNG previews when matplotlib is installed).  The experimental-image
comparison branch (img_path) needs fabio and is not provided.
"""
import argparse
import glob
import json
import os
import time

import numpy as np

from .tools.comparison import (detectormaker_fitting, slabmaker_fitting,
                               voxelgridmaker_average, voxelgridmaker_fitting)
from .tools.utilities import (load_pdb_cell_params, parse_config_file,
                              save_config_to_txt, str_to_bool)
from .workloads import phis_linspace


def _save_pngs(folder, det_sum, det_h, det_v):
    try:
        import matplotlib
        matplotlib.use("Agg")
        import matplotlib.pyplot as plt
    except ImportError:
        return
    img = det_sum.copy()
    img[img <= 0] = 1e-6
    for name, norm in (("lin", matplotlib.colors.Normalize(
            vmin=np.percentile(img, 1), vmax=np.percentile(img, 99.5))),
                       ("log", matplotlib.colors.LogNorm(
            vmin=np.percentile(img, 50), vmax=np.percentile(img, 99.95)))):
        fig, ax = plt.subplots(figsize=(10, 5))
        cax = ax.imshow(img, norm=norm, cmap="turbo", origin="lower",
                        extent=(np.min(det_v), np.max(det_v), np.min(det_h),
                                np.max(det_h)))
        fig.colorbar(cax, ax=ax, shrink=0.82, aspect=20, pad=0.02)
        ax.set_xlabel("q_xy (1/A)")
        ax.set_ylabel("q_z (1/A)")
        plt.tight_layout()
        plt.savefig(f"{folder}/det_sum_{name}.png", dpi=300)
        plt.close("all")


def main(config):
    input_folder = config.get("input_folder", None)
    input_path = config.get("input_filepath", None)
    filetype = config.get("filetype", None)
    x_size = float(config.get("x_size", 0))
    y_size = float(config.get("y_size", 0))
    z_size = float(config.get("z_size", 0))
    a = float(config.get("a", 0))
    b = float(config.get("b", 0))
    c = float(config.get("c", 0))
    alpha = float(config.get("alpha", 0))
    beta = float(config.get("beta", 0))
    gamma = float(config.get("gamma", 0))
    r_voxel_size = float(config.get("r_voxel_size", 0.3))
    q_voxel_size = float(config.get("q_voxel_size", 0.04))
    max_q = float(config.get("max_q", 2.5))
    energy = float(config.get("energy", 10000))
    fill_bkg = str_to_bool(config.get("fill_bkg", "False"))
    smooth = int(config.get("smooth", 0))
    num_pixels = int(config.get("num_pixels", max_q / q_voxel_size))
    init_vals = tuple(float(config.get(f"angle_init_val{i}", 0)) for i in (1, 2, 3))
    init_axs = tuple(config.get(f"angle_init_ax{i}", "None") for i in (1, 2, 3))
    psis = np.linspace(float(config.get("psi_start")), float(config.get("psi_end")),
                       int(config.get("psi_num")))
    phis = np.linspace(float(config.get("phi_start")), float(config.get("phi_end")),
                       int(config.get("phi_num")))
    thetas = np.linspace(float(config.get("theta_start")),
                         float(config.get("theta_end")),
                         int(config.get("theta_num")))
    psi_w = config.get("psi_weights_path", None)
    phi_w = config.get("phi_weights_path", None)
    theta_w = config.get("theta_weights_path", None)
    mirror = str_to_bool(config.get("mirror", "False"))
    img_path = config.get("img_path", None)
    phi_slices = int(config.get("phi_slices", 0))
    average_inputs = str_to_bool(config.get("average_inputs", "False"))
    accum = config.get("accum", "fp64")
    mode = config.get("mode", "batched")
    save_folder = config.get("save_folder", os.getcwd())
    write_metrics = str_to_bool(config.get("metrics", "True"))
    os.makedirs(save_folder, exist_ok=True)
    # wall time of every stage, written to save_folder/metrics.json (the
    # device-side ranges of the same stages are NVTX ranges named
    # "giwaxsim: ...", for timeline profilers)
    metrics = {"stages": [], "device": None}
    t_run = time.perf_counter()

    def stage(name, t0, **info):
        metrics["stages"].append(dict(name=name, seconds=time.perf_counter() - t0, **info))
    if img_path:
        raise NotImplementedError(
            "the experimental-image comparison (img_path) is not provided")

    if input_folder:
        if not filetype:
            raise Exception("filetype must be specified")
        input_paths = glob.glob(f"{input_folder}/*{filetype}")
    elif input_path:
        input_paths = [input_path]
    else:
        raise Exception("Either input_folder or input_path must be specified")
    gen_names = [os.path.splitext(os.path.basename(p))[0] for p in input_paths]
    slice_phis = phis_linspace(phi_slices) if phi_slices else None

    slabs = []
    t0 = time.perf_counter()
    for path in input_paths:
        if path.lower().endswith(".xyz"):
            cell = (a, b, c, alpha, beta, gamma)
        elif path.lower().endswith(".pdb"):
            cell = load_pdb_cell_params(path)
        else:
            raise Exception("Files must be a .pdb or .xyz file")
        if x_size == 0 or y_size == 0 or z_size == 0:
            x_size, y_size, z_size = a, b, c
            print("at least one slab size was not defined. Defaulting x,y,z "
                  "slab dimensions to a, b, c")
        if any(v == 0 for v in cell):
            raise Exception("at least one unit cell parameter a, b, c, alpha, "
                            "beta, gamma not defined")
        slabs.append(slabmaker_fitting(path, x_size, y_size, z_size, *cell))
    stage("slabs", t0, atoms=[len(s[0]) for s in slabs])

    def detector_and_save(iq, qx, qy, qz, name):
        t0 = time.perf_counter()
        det_sum, det_h, det_v = detectormaker_fitting(
            iq, qx, qy, qz, num_pixels, max_q, init_vals, init_axs, psis, psi_w,
            phis, phi_w, thetas, theta_w, mirror=mirror, accum=accum)
        stage("detector", t0, input=name, pixels=int(num_pixels),
              orientations=int(len(psis) * len(phis) * len(thetas)))
        t0 = time.perf_counter()
        folder = f"{save_folder}/{name}"
        os.makedirs(folder, exist_ok=True)
        if mirror:
            kh = np.where(det_h >= 0)[0]
            kv = np.where(det_v >= 0)[0]
            det_h, det_v = det_h[kh], det_v[kv]
            det_sum = det_sum[np.ix_(kv, kh)]
        np.save(f"{folder}/det_h.npy", det_h)
        np.save(f"{folder}/det_v.npy", det_v)
        np.save(f"{folder}/det_sum.npy", det_sum)
        _save_pngs(folder, det_sum, det_h, det_v)
        save_config_to_txt(config, f"{folder}/config.txt")
        stage("save", t0, input=name)
        return det_sum, det_h, det_v

    def finish(results):
        if write_metrics:
            from . import _native
            try:
                metrics["device"] = _native.default_context().device_name()
            except Exception:  # no device: the metrics still record the host
                pass
            metrics["total_seconds"] = time.perf_counter() - t_run
            with open(f"{save_folder}/metrics.json", "w") as fh:
                json.dump(metrics, fh, indent=1)
        return results

    results = {}
    if average_inputs and len(slabs) > 1:
        t0 = time.perf_counter()
        iq, qx, qy, qz = voxelgridmaker_average(
            slabs, r_voxel_size, q_voxel_size, max_q, energy, fill_bkg=fill_bkg,
            smooth=smooth, phis=slice_phis, accum=accum)
        stage("voxel", t0, input="average", structures=len(slabs))
        results["average"] = detector_and_save(iq, qx, qy, qz, "average")
        return finish(results)
    for (coords, elements), name in zip(slabs, gen_names):
        t0 = time.perf_counter()
        iq, qx, qy, qz = voxelgridmaker_fitting(
            coords, elements, r_voxel_size, q_voxel_size, max_q, energy,
            fill_bkg=fill_bkg, smooth=smooth, phis=slice_phis, mode=mode,
            accum=accum)
        stage("voxel", t0, input=name, atoms=len(coords), crop=int(iq.shape[0]))
        results[name] = detector_and_save(iq, qx, qy, qz, name)
    return finish(results)


if __name__ == "__main__":
    start = time.time()
    parser = argparse.ArgumentParser(description="Process a configuration file.")
    parser.add_argument("--config", type=str, required=True,
                        help="Path to the configuration file")
    args = parser.parse_args()
    main(parse_config_file(args.config))
    print(f"\nTotal Time: {time.time() - start}")
