"""Oracle: FP64 direct-sum structure factor and its gradient.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

The reference has no direct sum; S(q) = |sum_j f_j exp(i q.r_j)|^2 is the
continuous-position quantity whose gridded form is the reference's
``rfftn`` power (dens.py:313-316).  With A = sum f cos(q.r), B = sum f sin(q.r):

    dS/dr_j = 2 f_j q (B cos(q.r_j) - A sin(q.r_j))
    dS/df_j = 2 (A cos(q.r_j) + B sin(q.r_j))

and for a loss L(S), dL/dr_j = sum_q (dL/dS_q) dS_q/dr_j.
"""
from __future__ import annotations

import numpy as np


def amplitudes(r, f, q, chunk=4096):
    """(A, B) in FP64 for positions r (N,3), weights f (N,), q (M,3)."""
    r = np.asarray(r, np.float64)
    f = np.asarray(f, np.float64)
    q = np.asarray(q, np.float64)
    A = np.empty(len(q))
    B = np.empty(len(q))
    for s in range(0, len(q), chunk):
        ph = q[s:s + chunk] @ r.T
        A[s:s + chunk] = np.cos(ph) @ f
        B[s:s + chunk] = np.sin(ph) @ f
    return A, B


def sf(r, f, q):
    A, B = amplitudes(r, f, q)
    return A * A + B * B


def grad(r, f, q, g, chunk=4096):
    """dL/dr (N,3) and dL/df (N,) for upstream g = dL/dS (M,)."""
    r = np.asarray(r, np.float64)
    f = np.asarray(f, np.float64)
    q = np.asarray(q, np.float64)
    g = np.asarray(g, np.float64)
    A, B = amplitudes(r, f, q)
    gr = np.zeros_like(r)
    gf = np.zeros(len(r))
    for s in range(0, len(q), chunk):
        qs = q[s:s + chunk]
        ph = qs @ r.T                      # (m, N)
        c, sn = np.cos(ph), np.sin(ph)
        gb = (g[s:s + chunk] * B[s:s + chunk])[:, None]
        ga = (g[s:s + chunk] * A[s:s + chunk])[:, None]
        w = gb * c - ga * sn               # (m, N)
        gr += 2.0 * f[:, None] * (w.T @ qs)
        gf += 2.0 * ((ga * c + gb * sn).sum(0))
    return gr, gf


def loss_log1p_mse(S, target):
    """MSE(log(1+S), log(1+target)) and dL/dS."""
    d = np.log1p(S) - np.log1p(target)
    return float(np.mean(d * d)), 2.0 * d / (1.0 + S) / len(S)


def fd_grad(r, f, q, target, h=1e-5, atoms=None):
    """Central finite differences of the log1p-MSE loss in FP64."""
    r = np.array(r, np.float64)
    atoms = range(len(r)) if atoms is None else atoms
    out = np.zeros((len(list(atoms)), 3))
    for k, j in enumerate(atoms):
        for d in range(3):
            rp = r.copy(); rp[j, d] += h
            rm = r.copy(); rm[j, d] -= h
            lp, _ = loss_log1p_mse(sf(rp, f, q), target)
            lm, _ = loss_log1p_mse(sf(rm, f, q), target)
            out[k, d] = (lp - lm) / (2 * h)
    return out


def grad_chunk(r, f, q, g, A, B):
    """The part of (dL/dr, dL/df) that the q vectors ``q`` (with their dL/dS
    ``g`` and amplitudes A, B of the whole system) contribute: :func:`grad`
    is the sum of these over any split of the q set."""
    r = np.asarray(r, np.float64)
    f = np.asarray(f, np.float64)
    q = np.asarray(q, np.float64)
    ph = q @ r.T
    c, sn = np.cos(ph), np.sin(ph)
    gb = (np.asarray(g, np.float64) * B)[:, None]
    ga = (np.asarray(g, np.float64) * A)[:, None]
    w = gb * c - ga * sn
    return 2.0 * f[:, None] * (w.T @ q), 2.0 * ((ga * c + gb * sn).sum(0))


def fd_grad_moved(r, f, q, target, A, B, h=1e-5, atoms=(0,)):
    """Central finite differences of the log1p-MSE loss in FP64, one atom
    coordinate at a time: moving atom j changes only its own term of the
    amplitudes, so A, B of the unmoved system are updated by that term
    instead of being summed again (the same FP64 loss, O(M) per point)."""
    r = np.asarray(r, np.float64)
    f = np.asarray(f, np.float64)
    q = np.asarray(q, np.float64)
    out = np.zeros((len(atoms), 3))
    for k, j in enumerate(atoms):
        ph0 = q @ r[j]
        c0, s0 = np.cos(ph0), np.sin(ph0)
        for d in range(3):
            lv = []
            for sgn in (1.0, -1.0):
                rj = r[j].copy()
                rj[d] += sgn * h
                ph = q @ rj
                Ap = A + f[j] * (np.cos(ph) - c0)
                Bp = B + f[j] * (np.sin(ph) - s0)
                lv.append(loss_log1p_mse(Ap * Ap + Bp * Bp, target)[0])
            out[k, d] = (lv[0] - lv[1]) / (2 * h)
    return out
