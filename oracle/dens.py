"""Oracle: numpy restatement of the reference's ``dens.compute_sf`` (Gaussian mode).

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.  Every function cites
the reference lines (``dens.py`` of joeyelk/MD-Structure-Factor) it restates.
The per-atom loop is a pure-Python loop, as in the reference, so this module
is meant for small systems (a few thousand atom-frames).
"""
from __future__ import annotations

import math

import numpy as np

PRECISION = 1.0e-24          # dens.py:18
BUFFSIZE = 1_000_000         # dens.py:206


def load_radii(filename):
    """Type table: name -> (electrons, sigma in Angstrom).  dens.py:23-35.

    Each line is ``Nel name sigma_pm``; later duplicates of a name win and the
    sigma is divided by 100 (pm -> Angstrom).
    """
    out = {}
    with open(filename) as f:
        for line in f.readlines():
            fields = line.strip().split()
            out[fields[1]] = (float(fields[0]), float(fields[2]) / 100.0)
    return out


def grid_dims(L, Sres, better_resolution=True):
    """Spatial grid from a resolution, dens.py:181-189.

    ``int(L/Sres)`` per axis, bumped by one when the spacing is coarser than
    ``Sres``, then forced even.
    """
    L = np.asarray(L, dtype=np.float64)
    n = (L / Sres).astype(int)
    if better_resolution:
        for i in range(3):
            if L[i] / n[i] > Sres:
                n[i] += 1
    for i in range(3):
        n[i] += n[i] % 2
    return n


def rescale(coords, dims):
    """Scale each frame to the mean box, IN PLACE, dens.py:46-62."""
    avgdims = np.average(dims, axis=0)
    a = avgdims / dims
    for it in range(coords.shape[0]):
        for i in range(3):
            coords[it, :, i] *= a[it, i]
    return coords, avgdims


def wrap(r, L):
    """Periodic wrap, IN PLACE, dens.py:204-221.

    ``r<L ? r : r-L`` then ``r>0 ? r : r+L`` (so 0 maps to L).  For systems of
    ``BUFFSIZE`` atoms or more the reference's buffered branch only touches
    atoms ``[0, n_frames)`` of every frame (dens.py:214-221); that is
    reproduced here.
    """
    zv = np.zeros(3)
    if r.shape[1] < BUFFSIZE:
        for it in range(r.shape[0]):
            r[it, ...] = np.where(r[it, ...] < L, r[it, ...], r[it, ...] - L)
            r[it, ...] = np.where(r[it, ...] > zv, r[it, ...], r[it, ...] + L)
    else:
        m = min(r.shape[0], r.shape[1])
        for it in range(r.shape[0]):
            r[it, :m, :] = np.where(r[it, :m, :] < L, r[it, :m, :], r[it, :m, :] - L)
            r[it, :m, :] = np.where(r[it, :m, :] > zv, r[it, :m, :], r[it, :m, :] + L)
    return r


def borders(rad, dr, types):
    """Half-width of each type's footprint in grid steps, dens.py:38-43.

    Returns ``(bdict, Nborder)`` where ``bdict[t]`` is the float per-axis
    width ``sigma*sqrt(ln(Nel/1e-24))/dr`` and ``Nborder = int(max)`` over all
    types and axes (dens.py:223-231).
    """
    bdict = {}
    for a in types:
        bdict[a] = rad[a][1] * np.sqrt(np.log(rad[a][0] / PRECISION)) / dr
    Nborder = int(max(max(v) for v in bdict.values()))
    return bdict, Nborder


def padded_coords(N, Nborder, dr):
    """Per-axis coordinates of the padded grid, dens.py:244-256."""
    return [(np.arange(N[i] + 2 * Nborder) - Nborder) * dr[i] for i in range(3)]


def deposit_frame(r_t, typ, rad, bdict, Nborder, N, dr, ucell, d0=None):
    """Gaussian splat of one frame into the padded grid, dens.py:283-308."""
    shape = tuple(int(N[i]) + 2 * Nborder for i in range(3))
    if d0 is None:
        d0 = np.zeros(shape)
    gx, gy, gz = padded_coords(N, Nborder, dr)
    for im in range(r_t.shape[0]):
        ir = (r_t[im, :] / dr).astype(int)
        Ax, Ay, Az = bdict[typ[im]].astype(int)
        ix0, ix1 = ir[0] - Ax + Nborder, ir[0] + Ax + Nborder
        iy0, iy1 = ir[1] - Ay + Nborder, ir[1] + Ay + Nborder
        iz0, iz1 = ir[2] - Az + Nborder, ir[2] + Az + Nborder
        g = np.zeros((ix1 - ix0, iy1 - iy0, iz1 - iz0, 3))
        g[..., 0] = gx[ix0:ix1, None, None]
        g[..., 1] = gy[None, iy0:iy1, None]
        g[..., 2] = gz[None, None, iz0:iz1]
        buf = r_t[im, :] - g
        buf2 = np.einsum('ml,ijkm', ucell, buf)
        distSQ = buf2[..., 0] ** 2 + buf2[..., 1] ** 2 + buf2[..., 2] ** 2
        sig = rad[typ[im]][1]
        Nel = rad[typ[im]][0]
        d0[ix0:ix1, iy0:iy1, iz0:iz1] += (Nel / np.power(sig, 3.)) * np.exp(-distSQ / (2 * np.power(sig, 2.)))
    return d0


def fold_tcl(d0, N, Nborder):
    """Fold the padding back onto the periodic cell, dens.py:86-108, 258-263.

    Faces (6) and edges (12) land on their periodic images.  The 8 corner
    blocks take their z destination from the *y* side (the reference indexes
    ``des[2][id2]`` where ``des[2][id3]`` is meant, dens.py:107), so 4 of them
    land on the wrong z corner; that quirk is reproduced.
    """
    B = Nborder
    des = [[0, B, int(N[i]) - B, int(N[i])] for i in range(3)]
    ori = [[0, B, B + int(N[i]), 2 * B + int(N[i])] for i in range(3)]
    d1 = np.copy(d0[ori[0][1]:ori[0][2], ori[1][1]:ori[1][2], ori[2][1]:ori[2][2]])
    for io1 in (0, 2):
        id1 = 2 - io1
        d1[:, :, des[2][id1]:des[2][id1 + 1]] += d0[ori[0][1]:ori[0][2], ori[1][1]:ori[1][2], ori[2][io1]:ori[2][io1 + 1]]
        d1[:, des[1][id1]:des[1][id1 + 1], :] += d0[ori[0][1]:ori[0][2], ori[1][io1]:ori[1][io1 + 1], ori[2][1]:ori[2][2]]
        d1[des[0][id1]:des[0][id1 + 1], :, :] += d0[ori[0][io1]:ori[0][io1 + 1], ori[1][1]:ori[1][2], ori[2][1]:ori[2][2]]
        for io2 in (0, 2):
            id2 = 2 - io2
            d1[:, des[1][id1]:des[1][id1 + 1], des[2][id2]:des[2][id2 + 1]] += \
                d0[ori[0][1]:ori[0][2], ori[1][io1]:ori[1][io1 + 1], ori[2][io2]:ori[2][io2 + 1]]
            d1[des[0][id1]:des[0][id1 + 1], :, des[2][id2]:des[2][id2 + 1]] += \
                d0[ori[0][io1]:ori[0][io1 + 1], ori[1][1]:ori[1][2], ori[2][io2]:ori[2][io2 + 1]]
            d1[des[0][id1]:des[0][id1 + 1], des[1][id2]:des[1][id2 + 1], :] += \
                d0[ori[0][io1]:ori[0][io1 + 1], ori[1][io2]:ori[1][io2 + 1], ori[2][1]:ori[2][2]]
            for io3 in (0, 2):
                # corner quirk: z destination indexed by id2, not id3 (dens.py:107)
                d1[des[0][id1]:des[0][id1 + 1], des[1][id2]:des[1][id2 + 1], des[2][id2]:des[2][id2 + 1]] += \
                    d0[ori[0][io1]:ori[0][io1 + 1], ori[1][io2]:ori[1][io2 + 1], ori[2][io3]:ori[2][io3 + 1]]
    return d1


def power(d1):
    """Unnormalised forward R2C FFT and |F|^2, dens.py:313-316."""
    dfft = np.fft.rfftn(d1)
    dmag = dfft.conjugate()
    return np.real(np.multiply(dmag, dfft, out=dmag))


def get_dplot(dmag):
    """Half spectrum -> centred plottable array, dens.py:142-163.

    fftshift in x and y, Hermitian mirror in z, the z-Nyquist plane dropped,
    the DC voxel replaced by the mean of its +x, +y, +z neighbours and one
    voxel trimmed from every face.
    """
    n0, n1, nh = dmag.shape
    dplot = np.zeros([n0, n1, nh * 2 - 1])
    ix1, ix2 = n0 // 2, n0
    iy1, iy2 = n1 // 2, n1
    iz1, iz2 = nh - 1, nh * 2 - 2
    dplot[ix1:ix2, iy1:iy2, iz1:iz2] = dmag[0:ix1, 0:iy1, 0:iz1]
    dplot[0:ix1, iy1:iy2, iz1:iz2] = dmag[ix1:ix2, 0:iy1, 0:iz1]
    dplot[ix1:ix2, 0:iy1, iz1:iz2] = dmag[0:ix1, iy1:iy2, 0:iz1]
    dplot[0:ix1, 0:iy1, iz1:iz2] = dmag[ix1:ix2, iy1:iy2, 0:iz1]
    dplot[1:ix2 - 1, 1:iy2 - 1, :iz1] = dplot[:1:-1, :1:-1, iz2:iz1:-1]
    c0, c1, c2 = dplot.shape[0] // 2, dplot.shape[1] // 2, dplot.shape[2] // 2
    dplot[c0, c1, c2] = 1.0 / 3.0 * (dplot[c0 + 1, c1, c2] + dplot[c0, c1 + 1, c2] + dplot[c0, c1, c2 + 1])
    return dplot[1:-1, 1:-1, 1:-1]


def kgrid(shape, L):
    """q coordinates of the half spectrum, dens.py:325-334 (channel 3 stays 0).

    Negative frequencies carry the reference's half-bin offset
    ``-(i+0.5)*2*pi/L``.
    """
    kg = np.zeros((shape[0], shape[1], shape[2], 4))
    for ix in range(int(kg.shape[0] / 2)):
        kg[ix, :, :, 0] = ix * 2.0 * math.pi / L[0]
        kg[kg.shape[0] - 1 - ix, :, :, 0] = -(ix + 0.5) * 2.0 * math.pi / L[0]
    for iy in range(int(kg.shape[1] / 2)):
        kg[:, iy, :, 1] = iy * 2.0 * math.pi / L[1]
        kg[:, kg.shape[1] - 1 - iy, :, 1] = -(iy + 0.5) * 2.0 * math.pi / L[1]
    for iz in range(kg.shape[2]):
        kg[:, :, iz, 2] = iz * 2.0 * math.pi / L[2]
    return kg


def plot_axes(shape, L):
    """Axis coordinates of ``kgridplt`` for a half spectrum of ``shape``, dens.py:336-342."""
    n = (shape[0] - 2, shape[1] - 2, shape[2] * 2 - 3)
    return [np.array([(ix - n[a] / 2) * 2.0 * math.pi / L[a] for ix in range(n[a])]) for a in range(3)]


def kgridplt(sfplt, L):
    """Centred q grid with S in channel 3, dens.py:336-344."""
    shp = sfplt.shape
    kp = np.zeros((shp[0], shp[1], shp[2], 4))
    ax = plot_axes((shp[0] + 2, shp[1] + 2, (shp[2] + 3) // 2), L)
    kp[..., 0] = ax[0][:, None, None]
    kp[..., 1] = ax[1][None, :, None]
    kp[..., 2] = ax[2][None, None, :]
    kp[..., 3] = sfplt
    return kp


def compute_sf(r, L, typ, rad, ucell, Sres):
    """Full restatement of ``dens.compute_sf`` (dens.py:166-346), returning the
    npz arrays as a dict instead of writing them.  ``r`` and ``L`` are
    modified in place as in the reference.
    """
    r, Lm = rescale(r, L)
    N = grid_dims(Lm, Sres)
    dr = np.divide(Lm, N)
    wrap(r, Lm)
    bdict, Nb = borders(rad, dr, set(typ))
    sf = np.zeros([int(N[0]), int(N[1]), int(N[2] / 2) + 1])
    for it in range(r.shape[0]):
        d0 = deposit_frame(r[it], typ, rad, bdict, Nb, N, dr, ucell)
        d1 = fold_tcl(d0, N, Nb)
        sf += power(d1)
    sfplt = get_dplot(sf)
    return dict(sf=sf, sfplt=sfplt, L=Lm, N=N, kgrid=kgrid(sf.shape, Lm), kgridplt=kgridplt(sfplt, Lm))
