"""Seeded synthetic structures and run settings for the five benchmark
workloads of the GIWAXS forward path.

No dataset ships with the reference for these workloads, so structures are
built here from their crystallographic descriptions with
numpy.random.default_rng(seed):

  graphite-50A   hexagonal graphite (a=2.46 A, c=6.70 A, 4 C per cell) in a
                 50 A cube; r=0.3 A, dq=0.03 1/A, max_q=3, 180 phi slices;
                 500 px detector, psi 0..180 step 2.
  si-100A        diamond Si (a=5.431 A, 8 per cell), 100 A cube, 0.08 A
                 Gaussian displacements; r=0.25, dq=0.02, max_q=4, smooth=2,
                 fill_bkg; 360 slices; 1000 px, init psi=90, psi 0..90.
  graphite-64    64 graphite slabs with edges U(30,120) A per axis, 5 %
                 vacancies, 0.1 A displacements; r=0.3, dq=0.03, max_q=3,
                 smooth=1; 180 slices each, I(q) averaged; 1024 px, psi
                 0..180 step 1.
  si-60A-occ     Si 60 A cube with site occupancies U(0.8,1); r=0.3,
                 dq=0.04095 (g=512), max_q=3, smooth=1.5; 180 slices;
                 512 px, psi 0..90.
  lamellar-200A  polymer-like lamellar slab in a 200 A cube (C backbones along
                 x every 1.4 A, pi-stacked 3.7 A along y, lamellae 20 A along
                 z, 0.3 A chain disorder, 8-atom C side chains plus one S and
                 one F on every 4th backbone atom); r=0.2, dq=0.015,
                 max_q=2.5, smooth=2, fill_bkg; 720 slices; 2048 px, psi
                 0..180 step 1.
"""
import numpy as np

GRAPHITE_CELL = np.array([[2.46, 0.0, 0.0],
                          [-1.23, 2.46 * np.sqrt(3) / 2, 0.0],
                          [0.0, 0.0, 6.70]])
GRAPHITE_BASIS = np.array([[0, 0, 0.25], [0, 0, 0.75],
                           [1 / 3, 2 / 3, 0.25], [2 / 3, 1 / 3, 0.75]])
SI_A = 5.431
SI_CELL = np.eye(3) * SI_A
_FCC = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
SI_BASIS = np.concatenate([_FCC, _FCC + 0.25])


def lattice_box(cell, basis, size):
    """All lattice sites (cell rows are the lattice vectors) whose Cartesian
    position lies in [0,X) x [0,Y) x [0,Z)."""
    size = np.asarray(size, dtype=np.float64)
    corners = np.array([[i, j, k] for i in (0, 1) for j in (0, 1)
                        for k in (0, 1)], dtype=np.float64) * size
    frac = corners @ np.linalg.inv(cell)
    lo = np.floor(frac.min(0)).astype(int) - 1
    hi = np.ceil(frac.max(0)).astype(int) + 1
    ii, jj, kk = np.meshgrid(np.arange(lo[0], hi[0]), np.arange(lo[1], hi[1]),
                             np.arange(lo[2], hi[2]), indexing="ij")
    cells = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1).astype(np.float64)
    frac_all = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    xyz = frac_all @ cell
    keep = np.all((xyz >= 0) & (xyz < size), axis=1)
    return xyz[keep]


def graphite_slab(size, rng=None, disp_sigma=0.0, vacancy=0.0):
    xyz = lattice_box(GRAPHITE_CELL, GRAPHITE_BASIS, size)
    return _perturb(xyz, rng, disp_sigma, vacancy), "C"


def silicon_slab(size, rng=None, disp_sigma=0.0, vacancy=0.0):
    xyz = lattice_box(SI_CELL, SI_BASIS, size)
    return _perturb(xyz, rng, disp_sigma, vacancy), "Si"


def _perturb(xyz, rng, disp_sigma, vacancy):
    if rng is not None and vacancy > 0:
        xyz = xyz[rng.random(len(xyz)) >= vacancy]
    if rng is not None and disp_sigma > 0:
        xyz = xyz + rng.normal(0.0, disp_sigma, xyz.shape)
    return xyz


def lamellar_slab(size=200.0, rng=None):
    """Lamellar polymer-like slab: backbones along x, pi-stacking along y,
    lamellae along z; side chains of 8 C (random walk, 1.5 A steps) plus one
    S and one F on every 4th backbone atom.  Returns (coords, elements)."""
    rng = rng or np.random.default_rng(4)
    bx = np.arange(0.0, size, 1.4)
    xyz, el = [], []
    for z0 in np.arange(2.0, size - 2.0, 20.0):
        for y0 in np.arange(1.0, size - 1.0, 3.7):
            off = rng.normal(0.0, 0.3, 3)
            tilt = rng.normal(0.0, 0.3 / size, 2)
            bb = np.stack([bx + off[0], y0 + off[1] + tilt[0] * bx,
                           z0 + off[2] + tilt[1] * bx], 1)
            xyz.append(bb)
            el += ["C"] * len(bb)
            anchors = bb[::4]
            steps = rng.normal(size=(len(anchors), 8, 3))
            steps *= 1.5 / np.linalg.norm(steps, axis=2, keepdims=True)
            side = anchors[:, None, :] + np.cumsum(steps, axis=1)
            xyz.append(side.reshape(-1, 3))
            el += ["C"] * (8 * len(anchors))
            tip = side[:, -1, :]
            xyz.append(tip + np.array([0.0, 0.0, 1.8]))
            el += ["S"] * len(anchors)
            xyz.append(tip + np.array([0.0, 0.0, -1.4]))
            el += ["F"] * len(anchors)
    xyz = np.concatenate(xyz)
    el = np.array(el)
    keep = np.all((xyz >= 0) & (xyz < size), axis=1)
    return xyz[keep], el[keep]


def phis_linspace(n):
    """n slices over [0, 180) degrees."""
    return np.linspace(0.0, 180.0 - 180.0 / n, n)


WORKLOADS = {
    "graphite-50A": dict(r=0.3, dq=0.03, max_q=3.0, energy=10000.0,
                         fill_bkg=False, smooth=0, n_phi=180, seed=0,
                         num_pixels=500, init=((0, 0, 0), ("None",) * 3),
                         psis=(0.0, 180.0, 91)),
    "si-100A": dict(r=0.25, dq=0.02, max_q=4.0, energy=12000.0, fill_bkg=True,
                    smooth=2, n_phi=360, seed=1, num_pixels=1000,
                    init=((90, 0, 0), ("psi", "None", "None")),
                    psis=(0.0, 90.0, 91)),
    "graphite-64": dict(r=0.3, dq=0.03, max_q=3.0, energy=10000.0,
                        fill_bkg=False, smooth=1, n_phi=180, seed=2,
                        num_pixels=1024, init=((0, 0, 0), ("None",) * 3),
                        psis=(0.0, 180.0, 181)),
    "si-60A-occ": dict(r=0.3, dq=0.04095, max_q=3.0, energy=11000.0,
                       fill_bkg=False, smooth=1.5, n_phi=180, seed=3,
                       num_pixels=512, init=((0, 0, 0), ("None",) * 3),
                       psis=(0.0, 90.0, 91)),
    "lamellar-200A": dict(r=0.2, dq=0.015, max_q=2.5, energy=10000.0,
                          fill_bkg=True, smooth=2, n_phi=720, seed=4,
                          num_pixels=2048, init=((0, 0, 0), ("None",) * 3),
                          psis=(0.0, 180.0, 181)),
}


def structures(name):
    """List of (coords (N,3) float64, elements (N,) str, weights (N,) or None)
    for a named workload."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w["seed"])
    if name == "graphite-50A":
        xyz, e = graphite_slab((50, 50, 50))
        return [(xyz, np.full(len(xyz), e), None)]
    if name == "si-100A":
        xyz, e = silicon_slab((100, 100, 100), rng, disp_sigma=0.08)
        return [(xyz, np.full(len(xyz), e), None)]
    if name == "graphite-64":
        out = []
        for _ in range(64):
            size = rng.uniform(30, 120, 3)
            xyz, e = graphite_slab(size, rng, disp_sigma=0.1, vacancy=0.05)
            out.append((xyz, np.full(len(xyz), e), None))
        return out
    if name == "si-60A-occ":
        xyz, e = silicon_slab((60, 60, 60))
        occ = rng.uniform(0.8, 1.0, len(xyz))
        return [(xyz, np.full(len(xyz), e), occ)]
    if name == "lamellar-200A":
        xyz, el = lamellar_slab(200.0, rng)
        return [(xyz, el, None)]
    raise KeyError(name)
