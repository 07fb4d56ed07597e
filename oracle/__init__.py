"""CPU oracle for the structure-factor hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU in numpy/scipy, what the reference
(joeyelk/MD-Structure-Factor) computes on the structure-factor path, and is
used exclusively as the *checker*:

* ``tests/`` compare the CUDA library against it,
* ``__graft_entry__.smoke()`` checks one tiny GPU run against it,
* ``bench.py``'s ``cpu_baseline`` leg and ``--impl reference`` arm time it.

Nothing in the product package (``md-structure-factor_gb300/mdsf``) imports,
calls or links anything in here; the product path fails loudly when its CUDA
library is missing instead of falling back to this code.

Modules (each function cites the reference file:line it follows):

* :mod:`oracle.hist`   -- electron-weighted integer histogram on the box grid
  (``numpy.histogramdd`` semantics) -> rfftn -> |F|^2 -> FP64 sum over frames.
  The reference has no histogram mode; this is the plain histogram method
  standing in for ``dens.py:283-318``.
* :mod:`oracle.dens`   -- restatement of ``dens.compute_sf`` (Gaussian splat,
  padding fold with its corner quirk, rfftn, |F|^2, ``get_dplot``, ``kgrid``,
  ``kgridplt``, npz layout).
* :mod:`oracle.ewald`  -- Ewald-sphere slices of ``plot2d.py:218-267``.
* :mod:`oracle.direct` -- FP64 direct-sum S(q) and its analytic gradient.
* :mod:`oracle.cyl`    -- the cylindrical (r, z) average of ``plot2d.PLOT_RAD_NEW``.
* :mod:`oracle.gro`    -- .gro trajectory ingest (``load_traj.py``).
* :mod:`oracle.trr`    -- .trr trajectory frames (the CLI's trajectory format).

Pinning: ``tests/golden/*.npz`` hold outputs of the reference's own
``dens.compute_sf`` and ``plot2d.Plot_Ewald_Sphere_Correction`` run in the
build container (script: ``tests/golden/make_golden.py``); ``tests/test_oracle.py``
checks these restatements against them.  The histogram and FFT arithmetic is
numpy's own (``histogramdd``, ``fft.rfftn``), i.e. the third-party code the
reference itself calls at ``dens.py:313``.
"""
