"""mdsf -- GB300-native structure factors of MD trajectories.

Drop-in for the structure-factor path of joeyelk/MD-Structure-Factor
(``dens.compute_sf``, dens.py:166-346, and the Ewald slices of
plot2d.py:218-267), computed by hand-written sm_103a CUDA kernels in
``libmsf.so`` behind the C ABI of ``include/msf.h``.

    from mdsf import dens            # instead of `import dens`
    dens.compute_sf(r, L, typ, "out_sf", rad, ucell, Sres)

    import mdsf
    sf = mdsf.structure_factor(positions, box, weights, (256, 256, 128))
"""
from . import _lib
from ._lib import MsfError, load
from .api import (DirectSF, cylindrical_average, direct_sf, ewald_from_sf, ewald_slices, get_dplot,
                  hist_grid, plot_axes, power_accum, release_staging, structure_factor)
from .plan import Plan, get_plan
from . import dens, synth, tune
from .tune import tune_for

__all__ = ["MsfError", "load", "DirectSF", "cylindrical_average", "direct_sf", "ewald_from_sf", "ewald_slices",
           "get_dplot", "hist_grid", "plot_axes", "power_accum", "release_staging", "structure_factor", "Plan",
           "get_plan", "dens", "synth", "tune", "tune_for"]

__version__ = "0.1.0"
