"""Drop-in replacement for the reference's ``dens`` module (dens.py).

``compute_sf(r, L, typ, out_filename, rad, ucell, Sres)`` has the reference's
signature, side effects and output file (dens.py:166-346): ``r`` is rescaled
to the mean box and wrapped into the cell in place, the grid is derived from
``Sres``, and ``out_filename``(.npz) receives ``sf`` (the undivided sum over
frames of |rfftn(density)|^2), ``sfplt``, ``L``, ``N``, ``kgrid`` and
``kgridplt`` with the reference's shapes, dtypes and quirks.  The per-frame
work -- density deposit, padding fold, FFT, |F|^2 and the frame sum -- runs
in libmsf on the GPU:

* ``mode="gauss"`` (default): the reference's Gaussian splat (dens.py:283-311)
  in FP64, folded with remap_grid_tcl's map (dens.py:86-108).
* ``mode="hist"``: each atom's electron count binned with numpy.histogramdd
  semantics (bit-exact int32 grid), the plain method.

Module globals mirror the reference's knobs (dens.py:10-20).
Host-side steps (rescale, wrap, grid sizing, borders, the kgrid tables and
the npz writer) are restated from the reference lines cited on each function.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import api
from ._lib import call
from .api import _ptr, to_device
from .plan import get_plan, stream_ptr

USE_BETTER_RESOLUTION = True   # dens.py:10
PRINT_DETAILS = False          # dens.py:11 (the reference prints banners; off here)
RANDOM_NOISE = 0               # dens.py:12
theta = np.pi / 3              # dens.py:16 (set by main_gromacs.py:87, unused by compute_sf)
PRECISION = 1.0e-24            # dens.py:18
BUFFSIZE = 1_000_000           # dens.py:206
FRAMES_PER_LAUNCH = 8          # Gaussian grids deposited before one batched FFT call


def load_radii(filename):
    """Type table name -> (electrons, sigma in Angstrom), dens.py:23-35."""
    out = {}
    with open(filename) as f:
        for line in f.readlines():
            fields = line.strip().split()
            out[fields[1]] = (float(fields[0]), float(fields[2]) / 100.0)
    return out


def get_borders(ad, dr, keys):
    """Per-type footprint half-width in grid steps, dens.py:38-43."""
    return {a: ad[a][1] * np.sqrt(np.log(ad[a][0] / PRECISION)) / dr for a in keys}


def rescale(coords, dims):
    """Scale frames to the mean box in place, dens.py:46-62."""
    avgdims = np.average(dims, axis=0)
    a = avgdims / dims
    for it in range(coords.shape[0]):
        for i in range(3):
            coords[it, :, i] *= a[it, i]
    return coords, avgdims


def grid_dims(L, Sres):
    """Grid from the resolution, dens.py:181-189."""
    n = (np.asarray(L, np.float64) / Sres).astype(int)
    if USE_BETTER_RESOLUTION:
        for i in range(3):
            if L[i] / n[i] > Sres:
                n[i] += 1
    for i in range(3):
        n[i] += n[i] % 2
    return n


def wrap_positions(r, L):
    """Periodic wrap in place, dens.py:204-221 (including the buffered
    branch for >= BUFFSIZE atoms, which only reaches atoms [0, n_frames))."""
    zv = np.zeros(3)
    m = r.shape[1] if r.shape[1] < BUFFSIZE else min(r.shape[0], r.shape[1])
    for it in range(r.shape[0]):
        v = r[it, :m, :]
        v[...] = np.where(v < L, v, v - L)
        v[...] = np.where(v > zv, v, v + L)
    return r


def kgrid(shape, L):
    """q coordinates of the half spectrum, dens.py:325-334."""
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


def kgridplt(sfplt, L):
    """Centred q grid with S in channel 3, dens.py:336-344."""
    shp = sfplt.shape
    kp = np.zeros((shp[0], shp[1], shp[2], 4))
    ax = api.plot_axes((shp[0] + 2, shp[1] + 2, (shp[2] + 3) // 2), L)
    kp[..., 0] = ax[0][:, None, None]
    kp[..., 1] = ax[1][None, :, None]
    kp[..., 2] = ax[2][None, None, :]
    kp[..., 3] = sfplt
    return kp


def get_dplot(dmag):
    """dens.py:142-163 on the GPU; numpy in, numpy out (torch in, torch out)."""
    if isinstance(dmag, torch.Tensor):
        return api.get_dplot(dmag)
    t = api.get_dplot(to_device(np.asarray(dmag, np.float64), torch.device("cuda", torch.cuda.current_device())))
    return t.cpu().numpy()


def _ptr_np(a):
    from ._lib import c_p
    return c_p(a.ctypes.data)


def _type_table(rad, typ, dr):
    """Unique types, per-atom type index and the (c1, c2, Ax, Ay, Az) table."""
    names = sorted(set(typ), key=str)
    index = {t: i for i, t in enumerate(names)}
    bdict = get_borders(rad, dr, names)
    maxes = [max(v) for v in bdict.values()]
    nborder = int(max(maxes))
    tab = np.zeros((len(names), 5))
    for i, t in enumerate(names):
        sig = rad[t][1]
        Nel = rad[t][0]
        tab[i, 0] = Nel / np.power(sig, 3.)          # dens.py:308
        tab[i, 1] = 2 * np.power(sig, 2.)            # dens.py:308
        tab[i, 2:5] = bdict[t].astype(int)           # dens.py:287
    tidx = np.fromiter((index[t] for t in typ), dtype=np.int32, count=len(typ))
    return names, tidx, tab, nborder


def compute_sf_arrays(r, L, typ, rad, ucell, Sres, mode="gauss", device=None):
    """compute_sf without the file write: returns the six npz arrays."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    r, Lm = rescale(r, L)
    N = grid_dims(Lm, Sres)
    dr = np.divide(Lm, N)
    wrap_positions(r, Lm)
    if PRINT_DETAILS:
        print("Using a spatial grid of: %s, actual resolution %s" % (N, Lm / N))
    dims = tuple(int(n) for n in N)
    plan = get_plan(dims, Lm, device=device, max_atoms=r.shape[1])
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device=device)
    T, nat = r.shape[0], r.shape[1]
    with torch.cuda.device(device):
        st = stream_ptr(device)
        if RANDOM_NOISE > 0:
            # dens.py:279-280: density replaced by uniform noise
            for it in range(T):
                d1 = np.random.rand(*dims)
                api.power_accum(to_device(d1, device), sf, device=device)
        elif mode == "hist":
            w = np.array([int(rad[t][0]) for t in typ], dtype=np.int32)
            rd = to_device(np.ascontiguousarray(r, np.float64), device)
            wd = to_device(w, device)
            call("msf_hist_sf_f64", plan.handle, _ptr(rd), _ptr(wd), nat, T, _ptr(None), 0, _ptr(sf), st)
        elif mode == "gauss":
            names, tidx, tab, nborder = _type_table(rad, typ, dr)
            if nborder > min(dims):
                raise ValueError("Gaussian border (%d voxels) exceeds the grid %s" % (nborder, dims))
            geom = np.zeros(16)
            geom[0:3] = dr
            geom[3:12] = np.asarray(ucell, np.float64).reshape(9)
            geom[12] = nborder
            geom[13] = 2 * int(tab[:, 2:5].max())   # largest footprint: separable evaluation when <= 64
            geom_c = _ptr_np(geom)
            td = to_device(tidx, device)
            tabd = to_device(tab, device)
            nb = FRAMES_PER_LAUNCH
            grids = torch.empty((nb,) + dims, dtype=torch.float64, device=device)
            for f0 in range(0, T, nb):
                k = min(nb, T - f0)
                rd = to_device(np.ascontiguousarray(r[f0:f0 + k], np.float64), device)
                for j in range(k):
                    call("msf_gauss_grid_f64", plan.handle, _ptr(rd[j]), _ptr(td), nat, _ptr(tabd),
                         len(names), geom_c, _ptr(grids[j]), st)
                call("msf_power_accum_f64", plan.handle, _ptr(grids), k, _ptr(sf), st)
            plan.status()
        else:
            raise ValueError("mode must be 'gauss' or 'hist'")
        sfplt_t = api.get_dplot(sf)
    sf_h = sf.cpu().numpy()
    sfplt = sfplt_t.cpu().numpy()
    return dict(sf=sf_h, sfplt=sfplt, L=Lm, N=N, kgrid=kgrid(sf_h.shape, Lm),
                kgridplt=kgridplt(sfplt, Lm))


def compute_sf(r, L, typ, out_filename, rad, ucell, Sres, mode="gauss", device=None):
    """Drop-in for dens.compute_sf (dens.py:166-346): writes ``out_filename``.npz."""
    out = compute_sf_arrays(r, L, typ, rad, ucell, Sres, mode=mode, device=device)
    np.savez_compressed(out_filename, **out)
