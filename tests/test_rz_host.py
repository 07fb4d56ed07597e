"""(r, z) histograms of measure_intensity.py on the host, no GPU: the oracle
against the script's own run (tests/golden/rz_*.npz: the inputs and outputs
of its histogram2d calls, the plotted Hrz and the line it writes)."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import rz as orz

MI_UCELL = np.array([[1, 0, 0], [np.cos(math.pi / 3.0), np.sin(math.pi / 3.0), 0], [0, 0, 1]])


def rz_case(name):
    z = np.load(os.path.join(GOLDEN, "rz_" + name + ".npz"))
    D = np.load(os.path.join(GOLDEN, str(z["source"]) + ".npz"))["out_kgridplt"]
    return D, z


@pytest.mark.parametrize("name", ["ortho", "tcl"])
def test_oracle_matches_measure_intensity(name):
    D, z = rz_case(name)
    Hval, Hcount, rpts, zpts, w = orz.rz_histogram(D, MI_UCELL, density=True)
    np.testing.assert_array_equal(rpts, z["rpts"])
    np.testing.assert_array_equal(zpts, z["zpts"])
    np.testing.assert_array_equal(w, z["w"])
    np.testing.assert_array_equal(Hcount, z["Hcount"])
    np.testing.assert_array_equal(Hval, z["Hval_density"])
    Hrz = orz.rz_average(Hval, Hcount)
    np.testing.assert_array_equal(Hrz.T, z["HrzT"])
    imax = np.amax(Hrz.T)
    assert str(z["line"]) == "{:<5d}{:6.5f}\n".format(7, imax)
