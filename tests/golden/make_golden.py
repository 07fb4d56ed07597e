"""Generate the golden fixtures in this directory from the reference itself.

Run in a container where the reference checkout is present, giving its
path (required):

    python tests/golden/make_golden.py <reference dir> [--radial | --rz | --water]

It imports the reference's ``dens.py`` and ``plot2d.py`` directly (their
missing third-party modules -- ``past.utils``, ``tqdm`` progress bars and
``matplotlib`` -- are replaced by small stubs that do not touch the
arithmetic), runs ``dens.compute_sf`` on small seeded systems and
``plot2d.Plot_Ewald_Sphere_Correction`` on the resulting ``kgridplt``, and
saves inputs and outputs as compressed npz files.  Nothing is written into
the reference tree (``sys.dont_write_bytecode``).

Fixtures:
  gauss_*.npz  -- inputs of ``dens.compute_sf`` and all six saved arrays.
  ewald_*.npz  -- ``kgridplt``, wavelength and the three Ewald slices as
                  recorded from the reference's ``contourf`` calls.
  hist_edges.npz -- ``numpy.histogramdd`` on positions placed on and around
                  bin edges (pins the binning semantics the CUDA deposit
                  must match on numpy versions other than the one here).
  cyl_*.npz    -- the cylindrical (r, z) average of ``PLOT_RAD_NEW``.
  radial_*.npz -- ``plot2d.radial_integrate`` inputs and the (E[:-1], H)
                  it plots (``--radial`` makes these alone).
  rz_*.npz     -- ``measure_intensity.py`` run as a script: the inputs and
                  outputs of its two ``histogram2d`` calls, the plotted Hrz
                  and the line it writes (``--rz`` makes these alone).
  gauss_water.npz -- ``dens.compute_sf`` on the 1,500-water box (4,500 O/H
                  atoms, 25 Angstrom, 2 frames, Sres giving 64^3): the seed
                  and the inputs, ``sf`` and ``sfplt`` stored as float32 (the
                  parity bar is 1e-5 of max(S)), ``L``, ``N``, the in-place
                  ``r`` and SHA-256 digests of the float64 ``kgrid`` and of
                  the q channels of ``kgridplt`` (``--water`` makes it alone).
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    sys.dont_write_bytecode = True
    past = types.ModuleType("past")
    pu = types.ModuleType("past.utils")

    def old_div(a, b):
        if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
            return a // b
        return a / b
    pu.old_div = old_div
    past.utils = pu
    sys.modules["past"] = past
    sys.modules["past.utils"] = pu

    calls = []

    class _Rec:
        def __getattr__(self, name):
            def f(*a, **k):
                calls.append((name, a, k))
            return f
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    rec = _Rec()
    for name in ("figure", "suptitle", "xlabel", "ylabel", "contourf", "savefig", "clf",
                 "xlim", "ylim", "colorbar", "plot", "title", "close", "tight_layout"):
        setattr(plt, name, getattr(rec, name))
    ticker = types.ModuleType("matplotlib.ticker")
    widgets = types.ModuleType("matplotlib.widgets")
    widgets.Slider = widgets.Button = widgets.RadioButtons = object
    mpl.pyplot, mpl.ticker, mpl.widgets = plt, ticker, widgets
    mpl.rc = lambda *a, **k: None
    sys.modules.update({"matplotlib": mpl, "matplotlib.pyplot": plt,
                        "matplotlib.ticker": ticker, "matplotlib.widgets": widgets})
    return calls


class _Quiet:
    def __init__(self, it, *a, **k):
        self.it = it

    def __iter__(self):
        return iter(self.it)


def gauss_cases():
    rng = np.random.default_rng(20261203)
    cases = {}

    # orthorhombic, per-frame boxes (rescale), atoms on 0 / L / outside (wrap)
    T, N = 2, 40
    L = np.array([[12.0, 10.0, 8.0], [12.3, 9.8, 8.1]])
    r = rng.uniform(0.0, 1.0, (T, N, 3)) * L[:, None, :]
    r[0, 0] = [0.0, 0.0, 0.0]
    r[0, 1] = L[0]
    r[1, 2] = [-0.3, 10.2, 4.0]
    r[1, 3] = [12.5, -0.01, 8.05]
    typ = np.array((["O", "H", "H", "C", "N"] * 8)[:N], dtype=object)
    cases["gauss_ortho"] = dict(r=r, L=L, typ=typ, ucell=np.eye(3), Sres=0.6)

    # monoclinic cell (theta = 120 deg, main_gromacs.py:79-80), three frames
    T, N = 3, 36
    th = 120 * np.pi / 180.0
    ucell = np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]])
    L = np.array([[9.0, 9.0, 11.0], [9.1, 8.9, 11.2], [8.95, 9.05, 10.9]])
    r = rng.uniform(0.0, 1.0, (T, N, 3)) * L[:, None, :]
    typ = np.array((["C", "O", "H", "H"] * 9)[:N], dtype=object)
    cases["gauss_tcl"] = dict(r=r, L=L, typ=typ, ucell=ucell, Sres=0.7)

    # atoms packed near the 8 corners: exercises the corner fold quirk
    T, N = 1, 24
    L = np.array([[7.0, 8.0, 9.0]])
    corners = np.array([[a, b, c] for a in (0, 1) for b in (0, 1) for c in (0, 1)], float)
    r = np.empty((T, N, 3))
    for j in range(N):
        c = corners[j % 8]
        d = rng.uniform(0.05, 0.6, 3)
        r[0, j] = np.where(c > 0, L[0] - d, d)
    typ = np.array((["O", "N", "C"] * 8)[:N], dtype=object)
    cases["gauss_corner"] = dict(r=r, L=L, typ=typ, ucell=np.eye(3), Sres=0.5)
    return cases


def hist_edges_case():
    rng = np.random.default_rng(7)
    L = np.array([2.5, 3.1, 1.7])
    dims = np.array([16, 20, 10])
    pts = [rng.uniform(0, 1, (200, 3)) * L]
    for a in range(3):
        e = np.linspace(0.0, L[a], dims[a] + 1)
        p = rng.uniform(0, 1, (len(e), 3)) * L
        p[:, a] = e
        pts.append(p)
        p2 = p.copy()
        p2[:, a] = np.nextafter(e, -np.inf)
        pts.append(p2)
        p3 = p.copy()
        p3[:, a] = np.nextafter(e, np.inf)
        pts.append(p3)
    extra = np.array([[0.0, 0.0, 0.0], L, [-0.0, 1.0, 1.0], [-1e-12, 1.0, 1.0],
                      [L[0] + 1e-12, 1.0, 1.0], [np.nan, 1.0, 1.0], [1.0, np.inf, 1.0]])
    pts.append(extra)
    pos = np.concatenate(pts)
    w = rng.choice([1, 6, 7, 8], len(pos)).astype(np.int32)
    H, _ = np.histogramdd(pos, bins=dims, range=[(0, L[i]) for i in range(3)], weights=w.astype(float))
    pos32 = pos.astype(np.float32)
    H32, _ = np.histogramdd(pos32, bins=dims, range=[(0, L[i]) for i in range(3)], weights=w.astype(float))
    F = np.fft.rfftn(H)
    return dict(pos=pos, pos32=pos32, weights=w, L=L, dims=dims, grid=H.astype(np.int32),
                grid32=H32.astype(np.int32), sf=(F.real ** 2 + F.imag ** 2))


def main(ref):
    calls = _install_stubs()
    sys.path.insert(0, ref)
    import dens
    import plot2d
    dens.tqdm.tqdm = _Quiet
    rad = dens.load_radii(os.path.join(ref, "radii.txt"))
    tmp = tempfile.mkdtemp()
    for name, c in gauss_cases().items():
        r_in = c["r"].copy()
        L_in = c["L"].copy()
        out = os.path.join(tmp, name)
        with contextlib.redirect_stdout(io.StringIO()):
            dens.compute_sf(c["r"], c["L"], c["typ"], out, rad, c["ucell"], c["Sres"])
        z = np.load(out + ".npz")
        names = sorted(set(c["typ"]))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), r=r_in, L_in=L_in,
                            r_after=c["r"], typ=c["typ"].astype(str), ucell=c["ucell"],
                            Sres=c["Sres"], rad_names=np.array(names),
                            rad_nel=np.array([rad[n][0] for n in names]),
                            rad_sigma=np.array([rad[n][1] for n in names]),
                            **{"out_" + k: z[k] for k in z.files})
        print(name, {k: z[k].shape for k in z.files})

    plot2d.path = tmp + os.sep
    for name, lam in (("gauss_ortho", 1.54), ("gauss_tcl", 1.54), ("gauss_corner", 0.9)):
        D = np.load(os.path.join(HERE, name + ".npz"))["out_kgridplt"]
        del calls[:]
        with contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):
            plot2d.Plot_Ewald_Sphere_Correction(D, lam)
        cf = [c for c in calls if c[0] == "contourf"]
        # figures 1, 3, 5 plot the linear slices xy, xz, yz (plot2d.py:280-324)
        xy, xz, yz = cf[0][1][2], cf[2][1][2], cf[4][1][2]
        np.savez_compressed(os.path.join(HERE, "ewald_" + name.split("_", 1)[1] + ".npz"),
                            D=D, wavelength=lam, xy=xy, xz=xz, yz=yz)
        print("ewald", name, xy.shape, xz.shape, yz.shape, np.isnan(xy).sum())

    np.savez_compressed(os.path.join(HERE, "hist_edges.npz"), **hist_edges_case())
    print("hist_edges done")

    # cylindrical (r, z) average of PLOT_RAD_NEW (plot2d.py:559-640), the step
    # the reference CLI runs after compute_sf (main_gromacs.py:231 ->
    # plot2d.py:1008-1011); `final` is recorded from its first contourf call.
    th = 120 * np.pi / 180.0
    for name, ucell in (("gauss_ortho", np.eye(3)),
                        ("gauss_tcl", np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]]))):
        D = np.load(os.path.join(HERE, name + ".npz"))["out_kgridplt"]
        del calls[:]
        with contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):
            plot2d.trange = range
            try:
                plot2d.PLOT_RAD_NEW(D, 1.54, ucell, format=False)
            except Exception:   # plotting tail after the recorded call; not part of the average
                pass
        cf = [c for c in calls if c[0] == "contourf"]
        rfin, zfin0, finalT = cf[0][1][0], cf[0][1][1], cf[0][1][2]
        np.savez_compressed(os.path.join(HERE, "cyl_" + name.split("_", 1)[1] + ".npz"),
                            D=D, ucell=ucell, rfin=rfin, zfin=zfin0, final=np.asarray(finalT).T)
        print("cyl", name, np.asarray(finalT).shape)


def radial_cases():
    """kgridplt-shaped inputs for radial_integrate: the three compute_sf
    fixtures (by name), a synthetic q grid reaching |q|^2 ~ 400 (float16
    spacing 0.25 there; stored as its axes and S) and a grid of one |q|
    (empty range, widened by 0.5)."""
    cases = {}
    for name in ("gauss_ortho", "gauss_tcl", "gauss_corner"):
        D = np.load(os.path.join(HERE, name + ".npz"))["out_kgridplt"]
        cases[name.split("_", 1)[1]] = (D, 750, dict(source=name))
    rng = np.random.default_rng(11)
    X = np.linspace(-12.0, 12.0, 24, endpoint=False)
    Y = np.linspace(-10.5, 10.5, 20, endpoint=False)
    Z = np.linspace(-9.0, 9.0, 25)
    S = np.round(rng.gamma(2.0, 3.0, (24, 20, 25)), 3)
    cases["wide"] = (radial_grid(X, Y, Z, S), 750, dict(X=X, Y=Y, Z=Z, S=S))
    D1 = np.zeros((3, 4, 5, 4))
    D1[..., 0] = 0.5
    D1[..., 3] = np.round(rng.uniform(0, 1, (3, 4, 5)), 3)
    cases["flat"] = (D1, 12, dict(D=D1))
    return cases


def radial_grid(X, Y, Z, S):
    D = np.zeros(S.shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    return D


def main_radial(ref):
    """radial_integrate (plot2d.py:160-173) run by the reference, its
    plt.plot(E[:-1], H) call recorded."""
    calls = _install_stubs()
    sys.path.insert(0, ref)
    import plot2d
    for name, (D, nb, store) in radial_cases().items():
        del calls[:]
        with contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):
            plot2d.radial_integrate(D.copy(), nb, "radial.png")
        pl = [c for c in calls if c[0] == "plot"][0]
        np.savez_compressed(os.path.join(HERE, "radial_" + name + ".npz"), nbins=nb,
                            E=np.asarray(pl[1][0]), H=np.asarray(pl[1][1]), **store)
        print("radial", name, D.shape, nb)


def main_rz(ref):
    """measure_intensity.py run as a script (``-l <kgridplt npz> -f -y``) on
    the compute_sf fixtures.  numpy >= 1.24 no longer takes its
    ``histogram2d(..., normed=)``; a wrapper passes it on as ``density=`` (the
    same histogramdd option) and records the inputs and outputs of both
    calls.  PIL and the interactive plotting are stubbed."""
    import runpy
    calls = _install_stubs()
    import matplotlib.pyplot as plt
    plt.pcolormesh = lambda *a, **k: calls.append(("pcolormesh", a, k))
    plt.show = lambda *a, **k: None
    pil = types.ModuleType("PIL")
    pil.Image = types.ModuleType("PIL.Image")
    tq = types.ModuleType("tqdm")
    tq.trange = range
    tq.tqdm = _Quiet
    sys.modules.update({"PIL": pil, "PIL.Image": pil.Image, "tqdm": tq})
    rec = []
    real = np.histogram2d

    def histogram2d(x, y, bins=10, range=None, normed=None, weights=None, density=None):
        out = real(x, y, bins=bins, range=range, weights=weights, density=normed if normed is not None else density)
        rec.append(dict(x=np.array(x), y=np.array(y), w=None if weights is None else np.array(weights),
                        H=out[0], density=bool(normed or density)))
        return out
    cwd = os.getcwd()
    tmp = os.path.join(tempfile.gettempdir(), "mdsfgolden")
    os.makedirs(tmp, exist_ok=True)
    np.histogram2d = histogram2d
    try:
        for name in ("gauss_ortho", "gauss_tcl"):
            D = np.load(os.path.join(HERE, name + ".npz"))["out_kgridplt"]
            os.chdir(tmp)
            np.savez("out_x_sf_7.npz", kgridplt=D)
            if os.path.exists("intens.txt"):
                os.remove("intens.txt")
            del calls[:], rec[:]
            sys.argv = ["measure_intensity.py", "-l", "out_x_sf_7.npz", "-f", "-y", "-o", "intens.txt"]
            with contextlib.redirect_stdout(io.StringIO()), np.errstate(all="ignore"):
                runpy.run_path(os.path.join(ref, "measure_intensity.py"), run_name="__main__")
            line = open("intens.txt").read()
            os.chdir(cwd)
            pc = [c for c in calls if c[0] == "pcolormesh"][0]
            cnt = [r for r in rec if r["w"] is None][0]
            val = [r for r in rec if r["w"] is not None][0]
            np.savez_compressed(os.path.join(HERE, "rz_" + name.split("_", 1)[1] + ".npz"), source=name,
                                rpts=val["x"], zpts=val["y"], w=val["w"], Hcount=cnt["H"], Hval_density=val["H"],
                                HrzT=np.asarray(pc[1][2]), line=line)
            print("rz", name, val["H"].shape, np.isnan(val["w"]).sum(), repr(line))
    finally:
        np.histogram2d = real
        os.chdir(cwd)


def water_case(seed=1, frames=2):
    """The water box of the plain-method workload (1,500 rigid waters, O-H
    0.9572 A, 104.52 deg), in Angstrom for the reference: 25 A cube, types
    O / H, Sres = 25/64 A, so the grid is 64^3."""
    root = os.path.dirname(os.path.dirname(HERE))
    sys.path.insert(0, os.path.join(root, "md-structure-factor_gb300"))
    from mdsf import synth
    pos, box, _ = synth.water_box(n_waters=1500, L=2.5, frames=frames, seed=seed)
    r = pos * 10.0
    L = np.tile(box * 10.0, (frames, 1))
    typ = np.array(["O", "H", "H"] * 1500, dtype=object)
    return dict(r=r, L=L, typ=typ, ucell=np.eye(3), Sres=25.0 / 64)


def main_water(ref, seed=1, frames=2):
    """dens.compute_sf run by the reference on the 4,500-atom water box."""
    import hashlib
    _install_stubs()
    sys.path.insert(0, ref)
    import dens
    dens.tqdm.tqdm = _Quiet
    rad = dens.load_radii(os.path.join(ref, "radii.txt"))
    c = water_case(seed, frames)
    r_in, L_in = c["r"].copy(), c["L"].copy()
    out = os.path.join(tempfile.mkdtemp(), "water")
    with contextlib.redirect_stdout(io.StringIO()):
        dens.compute_sf(c["r"], c["L"], c["typ"], out, rad, c["ucell"], c["Sres"])
    z = np.load(out + ".npz")

    def digest(a):
        return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()
    np.savez_compressed(os.path.join(HERE, "gauss_water.npz"), seed=seed, frames=frames, Sres=c["Sres"],
                        r=r_in, L_in=L_in, r_after=c["r"], rad_names=np.array(["H", "O"]),
                        rad_nel=np.array([rad["H"][0], rad["O"][0]]),
                        rad_sigma=np.array([rad["H"][1], rad["O"][1]]),
                        out_sf32=z["sf"].astype(np.float32), out_sfplt32=z["sfplt"].astype(np.float32),
                        out_sf_max=z["sf"].max(), out_L=z["L"], out_N=z["N"],
                        kgrid_sha256=digest(z["kgrid"]), kgridplt_q_sha256=digest(z["kgridplt"][..., :3]),
                        shapes=np.array([z["sf"].shape, z["sfplt"].shape]))
    print("gauss_water", {k: z[k].shape for k in z.files})


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        sys.exit("usage: make_golden.py <reference dir> [--radial | --rz | --water]")
    ref_dir = args[0]
    if "--water" in sys.argv:
        main_water(ref_dir)
    elif "--radial" in sys.argv:
        main_radial(ref_dir)
    elif "--rz" in sys.argv:
        main_rz(ref_dir)
    else:
        main(ref_dir)
        main_radial(ref_dir)
        main_rz(ref_dir)
