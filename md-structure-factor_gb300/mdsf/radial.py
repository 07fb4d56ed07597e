"""Histogram reductions over the structure factor: ``radial_integrate``.

``plot2d.radial_integrate(D, Nbins, outputname)`` (plot2d.py:160-173) bins
S over R = |q|^2 computed in float16, normalises the weighted histogram by
the counts, zeroes the first bin and divides by the maximum.  The per-voxel
work -- R, the float16 bin search of numpy's equal-width histogram and the
weighted and plain bincounts -- runs in libmsf (``msf_radial_*``); the host
computes what numpy computes once per call (the float16 range and
``linspace`` edges) and the 2 x Nbins normalisation.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from ._lib import call
from .api import _ptr, to_device
from .plan import stream_ptr

MAX_BINS = 2048


def _edges(first, last, nbins):
    """numpy.histogram's float16 range handling and edges
    (_get_outer_edges, _get_bin_edges)."""
    if first == last:
        first = first - 0.5
        last = last + 0.5
    bin_type = np.result_type(first, last, np.empty(0, np.float16))
    edges = np.linspace(first, last, nbins + 1, endpoint=True, dtype=bin_type)
    if np.any(edges[:-1] >= edges[1:]):
        raise ValueError(f"Too many bins for data range. Cannot create {nbins} finite-sized bins.")
    return edges


def _check_bins(nbins):
    nbins = int(nbins)
    if nbins < 1 or nbins > MAX_BINS:
        raise ValueError(f"Nbins must be in [1, {MAX_BINS}] (float16-exact bin counts)")
    return nbins


def _finish(hist, count, edges, outputname):
    """plot2d.py:166-173 on the two histograms."""
    H = hist.cpu().numpy()
    Hc = count.cpu().numpy()
    Hc = np.where(Hc != 0, Hc, 1.0)
    H /= Hc
    H[:1] = 0.0
    with np.errstate(invalid="ignore", divide="ignore"):
        H /= np.amax(H)
    if outputname:
        np.savez(os.path.splitext(str(outputname))[0] + "_radial.npz", E=edges[:-1], H=H)
    return edges[:-1], H


def _bins_out(nbins, dev):
    hist = torch.zeros(nbins, dtype=torch.float64, device=dev)
    count = torch.zeros(nbins, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    return hist, count, status


def _check_status(status):
    if int(status.item()) != 0:
        raise RuntimeError("radial bin index left the histogram (float16 bin search)")


def radial_histograms(D, Nbins, device=None):
    """The two histograms of plot2d.py:164-165 on the GPU: (H, Hc, E) =
    (np.histogram(R, Nbins, weights=S)[0], np.histogram(R, Nbins)[0], edges)
    for D (..., 4) = (qx, qy, qz, S), numpy or CUDA float64.  H and Hc are
    CUDA tensors (float64, int64), E the float16 edges."""
    nbins = _check_bins(Nbins)
    if isinstance(D, torch.Tensor) and D.is_cuda:
        dev = D.device
        Dd = D.to(torch.float64).contiguous()
    else:
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        Dd = to_device(np.ascontiguousarray(np.asarray(D, np.float64)), dev)
    if Dd.shape[-1] != 4:
        raise ValueError("D must have 4 channels (qx, qy, qz, S)")
    nv = Dd.numel() // 4
    hist, count, status = _bins_out(nbins, dev)
    if nv == 0:   # numpy: empty sample -> range (0, 1), all bins empty
        return hist, count, _edges(0, 1, nbins)
    with torch.cuda.device(dev):
        stats = torch.empty(3, dtype=torch.int32, device=dev)
        call("msf_radial_range", _ptr(Dd), nv, _ptr(stats), stream_ptr(dev))
        lo, hi, bad = (int(v) & 0xFFFFFFFF for v in stats.cpu().tolist())
        if bad:
            raise ValueError("autodetected range of R is not finite")
        first = np.array([lo], np.uint16).view(np.float16)[0]
        last = np.array([hi], np.uint16).view(np.float16)[0]
        edges = _edges(first, last, nbins)
        ed = to_device(edges.view(np.int16), dev)
        call("msf_radial_bin_points", _ptr(Dd), nv, _ptr(ed), nbins, _ptr(hist), _ptr(count), _ptr(status),
             stream_ptr(dev))
        _check_status(status)
    return hist, count, edges


def radial_integrate(D, Nbins, outputname=None, device=None):
    """Drop-in for plot2d.radial_integrate (plot2d.py:160-173).

    D: (..., 4) array of (qx, qy, qz, S) -- numpy or CUDA float64, e.g. the
    ``kgridplt`` of ``compute_sf``.  Returns (E[:-1], H) as the reference
    plots them; with ``outputname`` the curve is also saved beside it as
    ``<outputname stem>_radial.npz`` (the reference saves a PNG plot).
    """
    hist, count, edges = radial_histograms(D, Nbins, device)
    return _finish(hist, count, edges, outputname)


def radial_histograms_grid(S, X, Y, Z, Nbins):
    """radial_histograms of the kgridplt built from the centred grid S
    (p0, p1, p2) CUDA float64 and its axes X, Y, Z (``plot_axes``), without
    materialising the (..., 4) array: the same bins and counts, 8 bytes read
    per voxel instead of 64."""
    nbins = _check_bins(Nbins)
    dev = S.device
    S = S.to(torch.float64).contiguous()
    p0, p1, p2 = S.shape
    tabs = [(np.asarray(a, np.float64) ** 2).astype(np.float16) for a in (X, Y, Z)]
    if any(len(t) != p for t, p in zip(tabs, (p0, p1, p2))):
        raise ValueError("axes must match the grid shape")
    if not all(np.all(np.isfinite(t)) for t in tabs):
        raise ValueError("autodetected range of R is not finite")
    # float16 rounding and addition are monotone: the extremes of R over the
    # product grid come from the extremes of each table
    first = (tabs[0].min() + tabs[1].min()) + tabs[2].min()
    last = (tabs[0].max() + tabs[1].max()) + tabs[2].max()
    if not (np.isfinite(first) and np.isfinite(last)):
        raise ValueError("autodetected range of R is not finite")
    edges = _edges(first, last, nbins)
    hist, count, status = _bins_out(nbins, dev)
    with torch.cuda.device(dev):
        hx, hy, hz = (to_device(t.view(np.int16), dev) for t in tabs)
        ed = to_device(edges.view(np.int16), dev)
        call("msf_radial_bin_grid", _ptr(S), p0, p1, p2, _ptr(hx), _ptr(hy), _ptr(hz), _ptr(ed), nbins,
             _ptr(hist), _ptr(count), _ptr(status), stream_ptr(dev))
        _check_status(status)
    return hist, count, edges


def radial_integrate_grid(S, X, Y, Z, Nbins, outputname=None):
    """radial_integrate of the kgridplt of (S, X, Y, Z), read in grid form."""
    hist, count, edges = radial_histograms_grid(S, X, Y, Z, Nbins)
    return _finish(hist, count, edges, outputname)
