"""FP32 R2C FFT + |F|^2 + FP64 accumulation against numpy.fft.rfftn (FP64).

Bar: max |S - S_ref| <= 1e-5 * max(S_ref) for every size class: powers of
two, 2^a 3^b 5^c (batched-system sizes), odd last axes, sizes with a prime
factor > 5 (generic radix), the plane, split and smooth (compile-time
mixed-radix) variants."""
import numpy as np
import pytest
import torch

import mdsf
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
TOL = 1e-5

SHAPES = [(64, 64, 64), (256, 256, 128), (48, 50, 54), (75, 81, 125), (96, 100, 243), (64, 74, 26),
          (14, 22, 38), (2, 4, 2), (3, 5, 7), (128, 96, 160), (512, 8, 16), (8, 512, 16), (16, 8, 512),
          (200, 216, 240), (512, 18, 20), (24, 512, 25), (30, 27, 512), (250, 162, 45)]


def grids_for(shape, n, seed, kind="int"):
    rng = np.random.default_rng(seed)
    if kind == "int":
        g = rng.poisson(0.4, (n,) + shape).astype(np.int32) * rng.integers(1, 9, (n,) + shape).astype(np.int32)
    else:
        g = rng.standard_normal((n,) + shape)
    return g


def ref_power(g):
    s = np.zeros(g.shape[1:3] + (g.shape[3] // 2 + 1,))
    for k in range(g.shape[0]):
        s += ohist.power(g[k])
    return s


@pytest.mark.parametrize("shape", SHAPES)
def test_power_accum_int_grids(shape):
    g = grids_for(shape, 3, sum(shape))
    ref = ref_power(g)
    got = mdsf.power_accum(torch.from_numpy(g).cuda(), tuning=dict(batch=2)).cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < TOL, (shape, err)


@pytest.mark.parametrize("shape", [(64, 64, 64), (48, 60, 80), (256, 256, 128)])
@pytest.mark.parametrize("variant", [1, 2, 4])
@pytest.mark.parametrize("tile_w", [4, 8, 16])
def test_variants_and_tiles_agree(shape, variant, tile_w):
    g = grids_for(shape, 2, 7)
    ref = ref_power(g)
    got = mdsf.power_accum(torch.from_numpy(g).cuda(),
                           tuning=dict(variant=variant, tile_w=tile_w, batch=2)).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_power_accum_real_grids(dtype):
    g = grids_for((40, 36, 50), 2, 3, kind="real").astype(dtype)
    ref = ref_power(g.astype(np.float64))
    got = mdsf.power_accum(torch.from_numpy(g).cuda()).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL


def test_batches_accumulate():
    g = grids_for((32, 32, 32), 7, 1)
    ref = ref_power(g)
    got = mdsf.power_accum(torch.from_numpy(g).cuda(), tuning=dict(batch=3)).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL


def test_delta_and_constant_kats():
    g = np.zeros((1, 16, 12, 10), np.int32)
    g[0, 3, 5, 7] = 9
    got = mdsf.power_accum(torch.from_numpy(g).cuda()).cpu().numpy()
    np.testing.assert_allclose(got, 81.0, rtol=1e-6)
    g = np.ones((1, 16, 12, 10), np.int32)
    got = mdsf.power_accum(torch.from_numpy(g).cuda()).cpu().numpy()
    assert abs(got[0, 0, 0] - (16 * 12 * 10) ** 2) < 1e-6 * (16 * 12 * 10) ** 2
    got[0, 0, 0] = 0
    assert np.abs(got).max() < 1e-6 * (16 * 12 * 10) ** 2
