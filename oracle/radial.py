"""Oracle: ``plot2d.radial_integrate`` (plot2d.py:160-173).

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

The reference's lines, in numpy: R = f16(x^2) + f16(y^2) + f16(z^2)
(plot2d.py:163), the weighted and plain ``np.histogram`` of R with Nbins
equal-width bins (plot2d.py:164-165), division by the counts with empty bins
counted as 1, the first bin zeroed and the maximum scaled to 1
(plot2d.py:166-169).  Returns what the reference plots: (E[:-1], H).  With
numpy >= 2 the range, edges and bin search of a float16 sample are float16
arithmetic; this module runs whatever numpy is installed, so the fixtures
in ``tests/golden/radial_*.npz`` (made by the reference itself) pin it.
"""
from __future__ import annotations

import numpy as np


def radial_integrate(D, Nbins):
    SF = D[:, :, :, 3]
    R = (D[:, :, :, 0] ** 2).astype(np.float16) + (D[:, :, :, 1] ** 2).astype(np.float16) + \
        (D[:, :, :, 2] ** 2).astype(np.float16)
    H, E = np.histogram(R, bins=Nbins, weights=SF)
    Hc, E = np.histogram(R, bins=Nbins)
    Hc = np.where(Hc != 0, Hc, 1.0)
    H /= Hc
    H[:1] = 0.0
    with np.errstate(invalid="ignore", divide="ignore"):
        H /= np.amax(H)
    return E[:-1], H


def radial_counts(D, Nbins):
    """The two raw histograms and the edges (before the normalisation)."""
    SF = D[..., 3]
    R = (D[..., 0] ** 2).astype(np.float16) + (D[..., 1] ** 2).astype(np.float16) + \
        (D[..., 2] ** 2).astype(np.float16)
    H, E = np.histogram(R, bins=Nbins, weights=SF)
    Hc, _ = np.histogram(R, bins=Nbins)
    return H, Hc, E
