"""Seeded synthetic systems with the shapes of the benchmark workloads.

No trajectory files ship with the reference (its test trajectory is missing),
so the workloads are generated from ``numpy.random.default_rng(seed)``:

* :func:`water_box`   -- rigid waters (O 8 e, H 1 e, O-H 0.09572 nm,
  H-O-H 104.52 deg), O uniform, orientation uniform, in a cubic box.
* :func:`columnar`    -- hexagonally packed columns along z made of shells of
  radius 1.0-1.8 nm, types C:O:N:H = 40:10:5:45 (6/8/7/1 e), 10% uniform
  background, Gaussian thermal noise per frame.
* :func:`uniform_system` -- uniform atoms with weights from {1, 6, 7, 8}.
* :func:`smooth_sizes` -- the 2^a 3^b 5^c grid sizes in a range.
* :func:`ewald_q_set` -- q vectors on the three Ewald-sphere slices of
  plot2d.py:236-255 plus a |q| shell (the differentiable workload).

Positions are wrapped into [0, L) (``np.mod``, then clamped below L in the
output precision).
"""
from __future__ import annotations

import numpy as np

ELECTRONS = {"C": 6, "O": 8, "N": 7, "H": 1}


def _clamp_below(x, L, dtype):
    x = np.mod(x, L).astype(dtype)
    top = np.nextafter(np.asarray(L, dtype=dtype), np.asarray(0, dtype=dtype))
    # largest value of `dtype` strictly below L (in FP64 comparison)
    top = np.where(top.astype(np.float64) < L, top, np.nextafter(top, np.asarray(0, dtype=dtype)))
    return np.minimum(x, top.astype(dtype))


def random_rotations(rng, n):
    """Uniform random rotation matrices (n, 3, 3) from unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def water_box(n_waters=1500, L=2.5, frames=10, seed=1, dtype=np.float64):
    """(positions (T, 3n, 3), box (3,), weights (3n,) int32): O, H, H per molecule."""
    rng = np.random.default_rng(seed)
    d = 0.09572
    half = np.deg2rad(104.52) / 2
    local = np.array([[0.0, 0.0, 0.0],
                      [d * np.sin(half), d * np.cos(half), 0.0],
                      [-d * np.sin(half), d * np.cos(half), 0.0]])
    box = np.array([L, L, L])
    pos = np.empty((frames, 3 * n_waters, 3), dtype=dtype)
    for t in range(frames):
        o = rng.uniform(0.0, L, size=(n_waters, 3))
        R = random_rotations(rng, n_waters)
        mol = o[:, None, :] + np.einsum("nij,kj->nki", R, local)
        pos[t] = _clamp_below(mol.reshape(-1, 3), box, dtype)
    w = np.tile(np.array([8, 1, 1], np.int32), n_waters)
    return pos, box, w


def columnar(n_atoms=200_000, box=(16.0, 13.856, 8.0), n_cols=(4, 4), lattice=4.0, frames=100,
             noise=0.1, background=0.1, seed=2, dtype=np.float32):
    """(positions (T, N, 3), box (3,), weights (N,) int32) of the columnar system."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, np.float64)
    n_bg = int(round(background * n_atoms))
    n_sh = n_atoms - n_bg
    cols = np.array([[(i + 0.5 * (j % 2)) * lattice, j * lattice * np.sqrt(3) / 2]
                     for j in range(n_cols[1]) for i in range(n_cols[0])])
    c = rng.integers(0, len(cols), n_sh)
    r = rng.uniform(1.0, 1.8, n_sh)
    phi = rng.uniform(0, 2 * np.pi, n_sh)
    shell = np.stack([cols[c, 0] + r * np.cos(phi), cols[c, 1] + r * np.sin(phi),
                      rng.uniform(0, box[2], n_sh)], -1)
    bg = rng.uniform(0, 1, (n_bg, 3)) * box
    base = np.concatenate([shell, bg])
    types = rng.choice(np.array(["C", "O", "N", "H"]), size=n_atoms, p=[0.40, 0.10, 0.05, 0.45])
    w = np.where(types == "C", 6, np.where(types == "O", 8, np.where(types == "N", 7, 1))).astype(np.int32)
    pos = np.empty((frames, n_atoms, 3), dtype=dtype)
    for t in range(frames):
        pos[t] = _clamp_below(base + rng.normal(0.0, noise, base.shape), box, dtype)
    return pos, box, w


def columnar_frames(base_seed, n_atoms, box, frames, dtype=np.float32, **kw):
    return columnar(n_atoms=n_atoms, box=box, frames=frames, seed=base_seed, dtype=dtype, **kw)


def uniform_system(n_atoms, box, frames=1, seed=3, dtype=np.float32):
    rng = np.random.default_rng(seed)
    box = np.asarray(box, np.float64)
    pos = _clamp_below(rng.uniform(0, 1, (frames, n_atoms, 3)) * box, box, dtype)
    w = rng.choice(np.array([1, 6, 7, 8], np.int32), n_atoms)
    return pos, box, w


def smooth_sizes(lo=48, hi=256):
    out = []
    for n in range(lo, hi + 1):
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return out


def pack_float4(pos, w):
    """(T, N, 3) float32 + (N,) -> (T, N, 4) float32 with the weight in .w."""
    pos = np.asarray(pos, np.float32)
    out = np.empty(pos.shape[:-1] + (4,), np.float32)
    out[..., :3] = pos
    out[..., 3] = np.asarray(w, np.float32)
    return out


def ewald_q_set(m=65_536, wavelength=0.154, extent=15.0, shell=(5.0, 15.0), seed=6):
    """(m, 3) float32 q vectors (nm^-1): three Ewald-sphere slices and a shell.

    Each slice is an n x n grid of in-plane points (a, b) in [-extent,
    extent]^2 lifted onto the sphere of radius K = 2 pi / wavelength as
    plot2d.py:236-255 does (theta = atan(sqrt(a^2 + b^2) / K), in-plane
    coordinates times cos(theta), the third K (1 - cos(theta)); xy, xz, yz
    planes), n = the largest power of two with 3 n^2 <= 3m/4; the rest are
    uniform directions with |q| uniform in ``shell``."""
    rng = np.random.default_rng(seed)
    K = 2.0 * np.pi / wavelength
    n = 1
    while 3 * (2 * n) ** 2 <= 3 * m // 4:
        n *= 2
    ax = np.linspace(-extent, extent, n)
    a, b = np.meshgrid(ax, ax, indexing="ij")
    c = np.cos(np.arctan(np.sqrt(a * a + b * b) / K))
    h = K * (1.0 - c)
    slices = [np.stack([a * c, b * c, h], -1), np.stack([a * c, h, b * c], -1), np.stack([h, a * c, b * c], -1)]
    q = [s.reshape(-1, 3) for s in slices]
    rest = m - 3 * n * n
    d = rng.standard_normal((rest, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q.append(d * rng.uniform(shell[0], shell[1], (rest, 1)))
    return np.concatenate(q).astype(np.float32)


def direct_system(n_atoms=20_000, L=6.0, seed=0, sigma=0.05):
    """(r (N,3) float32 in a cubic box, f (N,) float32 from {1,6,7,8},
    r_target = r + N(0, sigma) float32): the differentiable workload."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.0, L, (n_atoms, 3)).astype(np.float32)
    f = rng.choice(np.array([1, 6, 7, 8], np.float32), n_atoms)
    rt = (r + rng.normal(0.0, sigma, r.shape)).astype(np.float32)
    return r, f, rt
