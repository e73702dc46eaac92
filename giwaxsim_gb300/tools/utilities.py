"""Host utilities of the forward path, with the reference's names and
behaviour (tools/utilities.py of the reference):

  str_to_bool            utilities.py:10-41
  parse_config_file      utilities.py:43-50
  save_config_to_txt     utilities.py:52-55
  load_xyz / load_pdb    utilities.py:97-162
  load_pdb_cell_params   utilities.py:165-196
  write_xyz              utilities.py:199-220
  rotation_matrix        utilities.py:222-245
  calc_real_space_abc    utilities.py:276-301
  rotate_coords_z        utilities.py:303-317
  get_element_f0_dict    utilities.py:319-340 (kept with the reference's
                         q instead of q**2 in the exponent)
  get_element_f1_f2_dict utilities.py:342-366
"""
import os
import re
import warnings
from collections import Counter

import numpy as np

from .ptable_dict import aff_dict, ptable  # noqa: F401  (re-exported)

_TRUE = {"true", "t", "yes", "y", "1", "on"}
_FALSE = {"false", "f", "no", "n", "0", "off"}


def str_to_bool(input_value, default=False):
    s = str(input_value).strip().lower()
    if s in _TRUE:
        return True
    if s in _FALSE:
        return False
    if default is not None:
        return default
    raise ValueError(f"Invalid input for boolean conversion: {input_value}")


def parse_config_file(file_path):
    """key=value lines -> dict of strings (split on the first '=')."""
    config = {}
    with open(file_path, "r") as fh:
        for line in fh:
            if "=" in line:
                key, value = line.strip().split("=", 1)
                config[key] = value
    return config


def save_config_to_txt(config, save_path):
    with open(save_path, "w") as fh:
        for key, value in config.items():
            fh.write(f"{key}={value}\n")


def strip_numbers(element):
    m = re.match(r"([a-zA-Z]+)", element)
    return m.group(1) if m else element


def load_xyz(xyz_path):
    """Symbols and coordinates from an .xyz file; rows with fewer than four
    fields or unparsable numbers are skipped with a message."""
    symbols, coords = [], []
    with open(xyz_path, "r") as fh:
        lines = fh.readlines()
    for line in lines[2:]:
        parts = line.split()
        if len(parts) < 4:
            print(f"Skipping line due to insufficient parts: {line.strip()}")
            continue
        try:
            xyz = [float(v) for v in parts[1:4]]
        except ValueError as e:
            print(f"Skipping line due to error: {line.strip()} ({e})")
            continue
        symbols.append(strip_numbers(parts[0]))
        coords.append(xyz)
    return np.array(coords), np.array(symbols)


def load_pdb(pdb_path):
    """ATOM/HETATM records: element from columns 77-78, x/y/z from 31-54."""
    coords, elements = [], []
    with open(pdb_path, "r") as fh:
        for line in fh:
            if line.startswith("ATOM") or line.startswith("HETATM"):
                elements.append(line[76:78].strip())
                coords.append([float(line[30:38]), float(line[38:46]),
                               float(line[46:54])])
    return np.array(coords), np.array(elements)


def load_pdb_cell_params(pdb_path):
    with open(pdb_path, "r") as fh:
        for line in fh:
            if line.startswith("CRYST1"):
                return (float(line[6:15]), float(line[15:24]),
                        float(line[24:33]), float(line[33:40]),
                        float(line[40:47]), float(line[47:54]))
    raise ValueError("No CRYST1 line found in the PDB file.")


def most_common_element(input_path):
    if input_path[-3:] == "xyz":
        _, elements = load_xyz(input_path)
    elif input_path[-3:] == "pdb":
        _, elements = load_pdb(input_path)
    else:
        raise Exception("files must be a .pdb or .xyz file")
    return Counter(elements).most_common(1)[0][0]


def write_xyz(output_path, coords, elements):
    if len(coords) != len(elements):
        raise ValueError("Length of coordinates and elements must be the same.")
    with open(output_path, "w") as fh:
        fh.write(f"{len(elements)}\n")
        fh.write("XYZ file generated by write_xyz function\n")
        for el, (x, y, z) in zip(elements, coords):
            fh.write(f"{el} {x:.8f} {y:.8f} {z:.8f}\n")


def rotation_matrix(u, theta):
    """Rotation by theta (radians) about the unit vector u (Rodrigues)."""
    from ..forward import rotation_matrix as _rm
    return _rm(u, theta)


def calc_real_space_abc(a_mag, b_mag, c_mag, alpha_deg, beta_deg, gamma_deg):
    """Cartesian lattice vectors, a along x and b in the x-y plane."""
    al, be, ga = np.deg2rad(alpha_deg), np.deg2rad(beta_deg), np.deg2rad(gamma_deg)
    V = a_mag * b_mag * c_mag * np.sqrt(
        1 - np.cos(al) ** 2 - np.cos(be) ** 2 - np.cos(ga) ** 2
        + 2 * np.cos(al) * np.cos(be) * np.cos(ga))
    a = np.array([a_mag, 0, 0])
    b = np.array([b_mag * np.cos(ga), b_mag * np.sin(ga), 0])
    c = np.array([c_mag * np.cos(be),
                  c_mag * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga),
                  V / (a_mag * b_mag * np.sin(ga))])
    return a, b, c


def rotate_coords_z(coords, phi):
    """coords @ Rz(phi).T, evaluated in the fused order OpenBLAS uses."""
    from .. import _native
    pr = np.radians(phi)
    R = np.array([[np.cos(pr), -np.sin(pr), 0],
                  [np.sin(pr), np.cos(pr), 0],
                  [0, 0, 1]])
    return _native.rotate_points(R, np.asarray(coords, dtype=np.float64))


def get_element_f0_dict(q_val, elements):
    """f0 per element at q_val (utilities.py:318-340): the Cromer-Mann sum
    with the exponent -b q / (16 pi^2), q and not q^2, as the reference
    writes it (its multi-q shells call this)."""
    out = {}
    for el in set(elements):
        a = aff_dict[el]
        s = 16 * np.pi ** 2
        out[el] = (a[0] * np.exp(-a[1] * q_val / s) + a[2] * np.exp(-a[3] * q_val / s)
                   + a[4] * np.exp(-a[5] * q_val / s) + a[6] * np.exp(-a[7] * q_val / s)
                   + a[8])
    return out


_warned_xraydb = False

# f' = f'' = 0 (f = Z) when xraydb is missing: off unless the caller opts in
# (use_zero_f1f2(), or GIWAXSIM_F1F2=zero in the environment)
_ZERO_F1F2 = [os.environ.get("GIWAXSIM_F1F2", "").lower() == "zero"]

_XRAYDB = []


def use_zero_f1f2(on=True):
    """Opt in (or out) to f' = f'' = 0 when xraydb is not installed.  The
    reference imports xraydb at module level (tools/utilities.py:3) and
    cannot run without it; by default this drop-in refuses as well rather
    than change the intensities silently.  Callers that pass their own
    f' + i f'' table (the f1f2= keyword of the drivers) need neither."""
    _ZERO_F1F2[0] = bool(on)


def _xraydb():
    """The xraydb module or None, looked up once (a failed import is not
    cached by Python and costs a path search on every call)."""
    if not _XRAYDB:
        try:
            import xraydb
        except ImportError:
            xraydb = None
        _XRAYDB.append(xraydb)
    return _XRAYDB[0]


def get_element_f1_f2_dict(energy, elements):
    """f' + i f'' per element at `energy` eV from xraydb's Chantler tables
    (utilities.py:342-366).  Without xraydb: ImportError, unless the caller
    opted in to f' = f'' = 0 with use_zero_f1f2() (then a warning is issued
    once and the scattering factor is Z)."""
    global _warned_xraydb
    xraydb = _xraydb()
    if xraydb is None:
        if not _ZERO_F1F2[0]:
            raise ImportError(
                "xraydb is not installed: the f', f'' lookup needs it "
                "(tools/utilities.py:342-366).  Install xraydb, pass an "
                "f' + i f'' table (f1f2=...), or opt in to f' = f'' = 0 with "
                "giwaxsim_gb300.tools.utilities.use_zero_f1f2() or "
                "GIWAXSIM_F1F2=zero")
        if not _warned_xraydb:
            warnings.warn("xraydb is not installed: using f' = f'' = 0 "
                          "(opted in)")
            _warned_xraydb = True
        return {el: 0j for el in set(np.asarray(elements).tolist())}
    out = {}
    for el in set(np.asarray(elements).tolist()):
        try:
            out[el] = xraydb.f1_chantler(el, energy) + 1j * xraydb.f2_chantler(el, energy)
        except KeyError:
            print(f"Data for element '{el}' at energy {energy} eV not found.")
        except Exception as e:
            print(f"An error occurred for element '{el}': {e}")
    return out


def create_shared_array(shape, name=None):
    """float64 shared-memory block for `shape` (utilities.py:378-398); the
    name is always a fresh 29-character uuid (macOS limit), as there."""
    import uuid
    from multiprocessing import shared_memory
    size = int(np.prod(shape)) * np.dtype(np.float64).itemsize
    name = uuid.uuid4().hex[:29]
    try:
        return shared_memory.SharedMemory(create=True, size=size, name=name)
    except FileExistsError:
        shared_memory.SharedMemory(name=name).unlink()
        return shared_memory.SharedMemory(create=True, size=size, name=name)
