"""Trajectory ingest: GROMACS .gro trajectories into the reference's npz
trajectory layout, and the monoclinic coordinate transform.

Replaces load_traj.py's readers for .gro and .trr files -- ``process_gro_mdtraj``
(load_traj.py:91-110, which reads through mdtraj: coordinates nm -> Angstrom
x10, unitcell lengths x10, then ``np.savez_compressed(out, dims, coords,
name, mass, typ=name)``) and ``load_gro`` (load_traj.py:11-20, atom names) --
and the transform of main_gromacs.py:204-207.  The parsing is native
(``msf_gro_*`` and ``msf_trr_*`` in libmsf, one host thread per group of
frames); mdtraj is not needed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import c_p, call

# masses of the element guessed from an atom name (leading digits dropped,
# the two-letter ions NA and CL, else the first letter); 0 when unknown
MASSES = {"H": 1.008, "C": 12.011, "N": 14.007, "O": 15.999, "P": 30.974, "S": 32.06,
          "NA": 22.990, "CL": 35.45}


def scan_gro(path):
    """(n_atoms, n_frames) of a .gro trajectory."""
    na, nf = C.c_int64(), C.c_int64()
    call("msf_gro_scan", str(path).encode(), C.byref(na), C.byref(nf))
    return int(na.value), int(nf.value)


def read_gro(path, threads=0):
    """coords (T, N, 3) float32 Angstrom, dims (T, 3) float32 Angstrom (box
    vector lengths) and the atom names (N,) of a .gro trajectory."""
    n, t = scan_gro(path)
    xyz = np.empty((t, n, 3), np.float32)
    box = np.empty((t, 3), np.float64)
    names = np.zeros((max(n, 1), 8), np.uint8)
    call("msf_gro_read", str(path).encode(), n, t, c_p(xyz.ctypes.data), c_p(box.ctypes.data),
         c_p(names.ctypes.data), int(threads))
    nm = names.view("S8")[:n, 0].astype(str)
    return xyz, box.astype(np.float32), nm


def load_gro(path):
    """Atom names of the first frame, load_traj.py:11-20."""
    return list(read_gro(path)[2])


def guess_mass(name):
    s = name.lstrip("0123456789").upper()
    if s[:2] in ("NA", "CL"):
        return MASSES[s[:2]]
    return MASSES.get(s[:1], 0.0)


def process_gro(gro_path, output_filename, threads=0):
    """load_traj.process_gro_mdtraj for a .gro trajectory: writes
    output_filename(.npz) with dims, coords, name, mass and typ (= name, as
    the reference saves it, load_traj.py:110)."""
    coords, dims, name = read_gro(gro_path, threads)
    mass = np.array([guess_mass(s) for s in name])
    np.savez_compressed(output_filename, dims=dims, coords=coords, name=name, mass=mass, typ=name)


def scan_trr(path):
    """(n_atoms, n_frames) of a .trr trajectory."""
    na, nf = C.c_int64(), C.c_int64()
    call("msf_trr_scan", str(path).encode(), C.byref(na), C.byref(nf))
    return int(na.value), int(nf.value)


def read_trr(path, threads=0):
    """coords (T, N, 3) float32 Angstrom and dims (T, 3) float32 Angstrom
    (box vector lengths) of a .trr trajectory."""
    n, t = scan_trr(path)
    xyz = np.empty((t, n, 3), np.float32)
    box = np.empty((t, 3), np.float64)
    call("msf_trr_read", str(path).encode(), n, t, c_p(xyz.ctypes.data), c_p(box.ctypes.data), int(threads))
    return xyz, box.astype(np.float32)


def process_gro_trr(topology_filename, trajectory_filename, output_filename, threads=0):
    """load_traj.process_gro_mdtraj(top, traj, out) for the reference CLI's
    pair (main_gromacs.py:95-101): atom names from the .gro topology,
    coordinates and box lengths from the .trr (or a .gro) trajectory."""
    names = read_gro(topology_filename, threads)[2]
    if str(trajectory_filename).endswith(".gro"):
        coords, dims, _ = read_gro(trajectory_filename, threads)
    else:
        coords, dims = read_trr(trajectory_filename, threads)
    if coords.shape[1] != len(names):
        raise ValueError("topology and trajectory have different atom counts")
    mass = np.array([guess_mass(s) for s in names])
    np.savez_compressed(output_filename, dims=dims, coords=coords, name=names, mass=mass, typ=names)


def monoclinic(T, theta):
    """main_gromacs.py:204-207, in place: y /= sin(theta), then
    x -= y * cos(theta)."""
    T[..., 1] = T[..., 1] / np.sin(theta)
    T[..., 0] = T[..., 0] - T[..., 1] * np.cos(theta)
    return T


def write_gro(path, coords_angstrom, dims_angstrom, names, title="mdsf", decimals=3, box9=None):
    """Writes a .gro trajectory (coordinates and box in nm = Angstrom / 10,
    fixed columns with `decimals` decimals); box9 (T, 9) nm gives triclinic
    box lines instead of the three lengths."""
    coords = np.asarray(coords_angstrom, np.float64) / 10.0
    dims = np.asarray(dims_angstrom, np.float64) / 10.0
    if coords.ndim == 2:
        coords = coords[None]
        dims = dims[None]
    w = decimals + 5
    fmt = "%%%d.%df" % (w, decimals)
    with open(path, "w") as f:
        for t in range(coords.shape[0]):
            f.write("%s, t= %d\n%5d\n" % (title, t, coords.shape[1]))
            for i in range(coords.shape[1]):
                nm = str(names[i])[:5]
                f.write("%5d%-5s%5s%5d" % ((i // 3 + 1) % 100000, "SYS", nm, (i + 1) % 100000))
                f.write("".join(fmt % c for c in coords[t, i]) + "\n")
            if box9 is not None:
                f.write(" ".join("%10.5f" % v for v in box9[t]) + "\n")
            else:
                f.write(" ".join("%10.5f" % v for v in dims[t]) + "\n")
