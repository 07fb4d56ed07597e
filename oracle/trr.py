"""Oracle: GROMACS .trr trajectory frames (XDR, big-endian).

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

The reference reads .trr trajectories through mdtraj (``md.load(traj,
top=gro)`` in ``load_traj.process_gro_mdtraj``, load_traj.py:91-110, the
pair main_gromacs.py:95-101 passes); neither mdtraj nor a .trr fixture is
available here, so this module restates the published frame layout (parity
is pinned to that restatement, not to mdtraj):

    int magic 1993; int len("GMX_trn_file") + 1; XDR string (uint length,
    bytes padded to 4); 13 ints ir_size e_size box_size vir_size pres_size
    top_size sym_size x_size v_size f_size natoms step nre; reals t lambda;
    box[9] vir[9] pres[9] x[natoms*3] v[...] f[...] (each when its size > 0),
    a real being 4 or 8 bytes.

Positions as the reference's pipeline sees them: float32 nm * 10 in
float32; box lengths the float32 norm of each box vector * 10.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = 1993
VERSION = b"GMX_trn_file"
F10 = np.float32(10.0)


def write_trr(path, coords_nm, box_nm, double=False, velocities=None, forces=None, with_box=True):
    """coords_nm (T, N, 3), box_nm (T, 3, 3) box vectors (rows) in nm."""
    coords_nm = np.asarray(coords_nm, np.float64)
    T, N, _ = coords_nm.shape
    fmt = ">d" if double else ">f"
    prec = 8 if double else 4
    with open(path, "wb") as f:
        for t in range(T):
            box_size = 9 * prec if with_box else 0
            vs = 3 * N * prec if velocities is not None else 0
            fs = 3 * N * prec if forces is not None else 0
            f.write(struct.pack(">ii", MAGIC, len(VERSION) + 1))
            f.write(struct.pack(">I", len(VERSION)) + VERSION + b"\0" * ((-len(VERSION)) % 4))
            f.write(struct.pack(">13i", 0, 0, box_size, 0, 0, 0, 0, 3 * N * prec, vs, fs, N, t * 10, 0))
            f.write(struct.pack(fmt, 0.5 * t) + struct.pack(fmt, 0.0))
            if with_box:
                f.write(np.asarray(box_nm[t], np.float64).reshape(9).astype(fmt).tobytes())
            f.write(coords_nm[t].astype(fmt).tobytes())
            if velocities is not None:
                f.write(np.asarray(velocities[t]).astype(fmt).tobytes())
            if forces is not None:
                f.write(np.asarray(forces[t]).astype(fmt).tobytes())


def read_trr(path):
    """(coords (T, N, 3) float32 Angstrom, dims (T, 3) float32 Angstrom)."""
    data = open(path, "rb").read()
    pos = 0
    coords, dims = [], []
    while pos < len(data):
        magic, _slen = struct.unpack_from(">ii", data, pos)
        if magic != MAGIC:
            raise ValueError("not a trr frame")
        pos += 8
        (xl,) = struct.unpack_from(">I", data, pos)
        pos += 4 + xl + ((-xl) % 4)
        h = struct.unpack_from(">13i", data, pos)
        pos += 52
        box_size, vir, pres, xs, vs, fs, natoms = h[2], h[3], h[4], h[7], h[8], h[9], h[10]
        prec = box_size // 9 if box_size else xs // (3 * natoms)
        fmt = ">f8" if prec == 8 else ">f4"
        pos += 2 * prec
        box = None
        if box_size:
            box = np.frombuffer(data, fmt, 9, pos).astype(np.float32).reshape(3, 3)
            pos += box_size
        pos += vir + pres
        x = np.frombuffer(data, fmt, 3 * natoms, pos).astype(np.float32).reshape(natoms, 3)
        pos += xs + vs + fs
        coords.append(x * F10)
        if box is None:
            dims.append(np.zeros(3, np.float32))
        else:
            out = np.zeros(3, np.float32)
            for a in range(3):
                s2 = box[a, 0] * box[a, 0] + box[a, 1] * box[a, 1] + box[a, 2] * box[a, 2]
                out[a] = np.sqrt(np.float32(s2)) * F10
            dims.append(out)
    return np.stack(coords), np.stack(dims)
