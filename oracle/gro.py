"""Oracle: GROMACS .gro trajectory ingest.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

* :func:`load_gro` restates ``load_traj.load_gro`` (load_traj.py:11-20)
  line for line in meaning: the atom names are columns 11-15, stripped, of
  every line from the third to the second last of the file.
* :func:`read_gro` restates what ``load_traj.process_gro_mdtraj``
  (load_traj.py:91-110) takes from its trajectory reader for a .gro file:
  positions in nm as float32, times 10 (float32) to Angstrom, and the
  lengths of the three box vectors, float32, times 10.  The reader the
  reference calls is mdtraj's (``md.load``; requirements.txt names it with
  no version), which is not installed here; its .gro parsing is restated
  from the published file format: fixed columns, coordinate fields of equal
  width w = the distance between the first two decimal points from column
  21, a box line of 3 numbers (v1x v2y v3z) or 9 (then v1y v1z v2x v2z v3x
  v3y).  The float32 norm of each box vector is this restatement's choice
  (mdtraj's intermediate type could not be checked): box lengths are pinned
  only to within one float32 ulp.
* :func:`write_gro` writes test trajectories in that format.

Pure-Python loops: meant for files of up to ~10^5 atom lines.
"""
from __future__ import annotations

import numpy as np

F10 = np.float32(10.0)


def load_gro(path):
    """load_traj.py:11-20."""
    with open(path) as f:
        lines = f.readlines()
    return [ln[10:15].strip() for ln in lines[2:-1]]


def _width(line):
    d1 = line.index(".", 20)
    d2 = line.index(".", d1 + 1)
    return d2 - d1


def _box_lengths(line):
    v = [float(t) for t in line.split()]
    if len(v) not in (3, 9):
        raise ValueError("box line must hold 3 or 9 numbers")
    vec = np.zeros((3, 3), np.float32)
    vec[0, 0], vec[1, 1], vec[2, 2] = v[0], v[1], v[2]
    if len(v) == 9:
        vec[0, 1], vec[0, 2], vec[1, 0], vec[1, 2], vec[2, 0], vec[2, 1] = v[3:9]
    out = np.zeros(3, np.float32)
    for a in range(3):
        s2 = vec[a, 0] * vec[a, 0] + vec[a, 1] * vec[a, 1] + vec[a, 2] * vec[a, 2]
        out[a] = np.sqrt(np.float32(s2)) * F10
    return out


def read_gro(path):
    """(coords (T, N, 3) float32 Angstrom, dims (T, 3) float32 Angstrom,
    names (N,) of the first frame)."""
    with open(path) as f:
        lines = f.read().splitlines()
    while lines and not lines[-1].strip():
        lines.pop()
    coords, dims, names = [], [], None
    l = 0
    w = None
    while l < len(lines):
        n = int(lines[l + 1].split()[0])
        atoms = lines[l + 2:l + 2 + n]
        if len(atoms) != n or l + 2 + n >= len(lines):
            raise ValueError("truncated frame")
        if w is None and n:
            w = _width(atoms[0])
        xyz = np.zeros((n, 3), np.float32)
        for i, ln in enumerate(atoms):
            for c in range(3):
                xyz[i, c] = np.float32(float(ln[20 + c * w:20 + (c + 1) * w])) * F10
        if names is None:
            names = [ln[10:15].strip() for ln in atoms]
        coords.append(xyz)
        dims.append(_box_lengths(lines[l + 2 + n]))
        l += n + 3
    if coords and any(c.shape != coords[0].shape for c in coords):
        raise ValueError("atom count changes between frames")
    return np.stack(coords), np.stack(dims), names


def write_gro(path, coords_nm, box_nm, names, decimals=3, title="test", velocities=None):
    """coords_nm (T, N, 3), box_nm (T, 3) or (T, 9), names (N,)."""
    coords_nm = np.asarray(coords_nm, np.float64)
    box_nm = np.asarray(box_nm, np.float64)
    w = decimals + 5
    with open(path, "w") as f:
        for t in range(coords_nm.shape[0]):
            f.write("%s t= %d\n%5d\n" % (title, t, coords_nm.shape[1]))
            for i in range(coords_nm.shape[1]):
                f.write("%5d%-5s%5s%5d" % ((i // 3 + 1) % 100000, "SOL", str(names[i])[:5],
                                          (i + 1) % 100000))
                f.write("".join("%*.*f" % (w, decimals, c) for c in coords_nm[t, i]))
                if velocities is not None:
                    f.write("".join("%*.*f" % (w + 1, decimals + 1, c) for c in velocities[t, i]))
                f.write("\n")
            f.write(" ".join("%10.5f" % b for b in box_nm[t]) + "\n")
