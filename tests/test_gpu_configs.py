"""The five benchmark workloads at their stated sizes, element by element
against the FP64 oracle, which runs on the host's cores in a spawn pool.

Bars: S(q) within 1e-5 * max(S) of the FP64 numpy oracle (histogramdd +
rfftn + FP64 frame sum); get_dplot bit-exact and the Ewald slices within
1e-12 relative of the scipy restatement applied to the same S(q); the
direct-sum S(q) within 2e-5 (norm) of the FP64 direct sum and dL/dr within
1e-4 (norm) of the FP64 analytic gradient and of FP64 central finite
differences (h = 1e-5 nm).  Every test prints its max and RMS error as a
fraction of max(S) (norms for the direct sum): the per-configuration error
record.
"""
import math

import numpy as np
import pytest
import torch
from scipy.interpolate import RegularGridInterpolator

import mdsf
from mdsf import synth
from mdsf._lib import c_p, call
from mdsf.api import _ptr
from oracle import dens as odens
from oracle import direct as odirect
from oracle import ewald as oewald
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
TOL = 1e-5


def errors(got, ref):
    m = float(np.abs(ref).max())
    return float(np.abs(got - ref).max() / m), float(np.sqrt(np.mean((got - ref) ** 2)) / m)


def pool_hist_sf(pool, jobs, frames_per_job=8):
    """FP64 oracle sums for several systems (pos (T,N,3), box (3,), w, dims),
    frames split into jobs of `frames_per_job` over the pool."""
    tasks, owner = [], []
    for i, (pos, box, w, dims) in enumerate(jobs):
        assert np.ndim(box) == 1, "one box per system: frame chunks bin alike"
        for a in range(0, pos.shape[0], frames_per_job):
            tasks.append((np.ascontiguousarray(pos[a:a + frames_per_job]), np.asarray(box), w, tuple(dims)))
            owner.append(i)
    parts = pool.starmap(ohist.hist_sf, tasks, chunksize=1)
    out = [None] * len(jobs)
    for i, p in zip(owner, parts):
        out[i] = p if out[i] is None else out[i] + p
    return out


def check_post(sf, L, wavelength=0.154):
    """get_dplot of the device sf bit-exact with the restatement of
    dens.py:142-163, and its Ewald slices within 1e-12 of scipy's
    RegularGridInterpolator at the points of plot2d.py:236-255."""
    host = sf.cpu().numpy()
    D = mdsf.get_dplot(sf)
    Dn = D.cpu().numpy()
    np.testing.assert_array_equal(Dn, odens.get_dplot(host))
    X, Y, Z = mdsf.plot_axes(tuple(sf.shape), L)
    xy, xz, yz = mdsf.ewald_slices(D, X, Y, Z, wavelength)
    ES = RegularGridInterpolator((X, Y, Z), Dn, bounds_error=False)
    pts = oewald.slice_points_vec(X, Y, Z, 2.0 * math.pi / wavelength)
    for got, p, shape in ((xy, pts[0], (len(X), len(Y))), (xz, pts[1], (len(X), len(Z))),
                          (yz, pts[2], (len(Y), len(Z)))):
        ref = ES(p).reshape(shape)
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.nanmax(np.abs(ref)),
                                   equal_nan=True)


# ------------------------------------------------------------ configuration 1
def test_config1_water_box(oracle_pool):
    """1,500 rigid waters (4,500 atoms), 2.5 nm, 10 float64 frames, 64^3."""
    pos, box, w = synth.water_box(n_waters=1500, L=2.5, frames=10, seed=1)
    ref, = pool_hist_sf(oracle_pool, [(pos, box, w, (64, 64, 64))], frames_per_job=2)
    got = mdsf.structure_factor(pos, box, w, (64, 64, 64)).cpu().numpy()
    e, rms = errors(got, ref)
    print(f"config 1 (water 4,500 atoms, 64^3, 10 f64 frames): max err {e:.2e}, rms {rms:.2e} of max(S)")
    assert e < TOL


# ------------------------------------------------------------ configuration 2
def test_config2_benchmarked_chain(oracle_pool):
    """The benchmarked step exactly: the columnar system (200,000 atoms,
    16.0 x 13.856 x 8.0 nm, seed 2), 100 float32 frames, 256 x 256 x 128, on
    the default plan (bucketed chain, batches of at most 64 frames -- two of
    50 here --, x pass overlapped on the plan's side stream) called through
    the C ABI, then get_dplot and the
    Ewald slices at lambda = 0.154 nm."""
    dims, n, T = (256, 256, 128), 200_000, 100
    pos, box, w = synth.columnar(n_atoms=n, frames=T, seed=2)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda()
    plan = mdsf.get_plan(dims, box, max_atoms=n)
    assert plan.tuning()["variant"] == "bucketed" and plan.batch == 64 and plan.tma
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    call("msf_hist_sf_f32", plan.handle, _ptr(p4), n, T, c_p(0), 0, _ptr(sf),
         c_p(torch.cuda.current_stream().cuda_stream))
    plan.status()
    ref, = pool_hist_sf(oracle_pool, [(pos, box, w, dims)])
    got = sf.cpu().numpy()
    e, rms = errors(got, ref)
    print(f"config 2 (columnar 200k atoms, 256x256x128, 100 frames, two 50-frame batches): "
          f"max err {e:.2e}, rms {rms:.2e} of max(S)")
    assert e < TOL
    check_post(sf, box)


@pytest.mark.parametrize("variant", [1, 3, 4])
def test_batch_of_256_frames(oracle_pool, variant):
    """The largest batch a plan accepts (256 frames in one pass): the x pass
    adds its FP32 partial sums to the FP64 sf every 32 frames, so the error
    stays at the level of short batches."""
    pos, box, w = synth.water_box(n_waters=1500, L=2.5, frames=256, seed=3, dtype=np.float32)
    ref, = pool_hist_sf(oracle_pool, [(pos, box, w, (64, 64, 64))], frames_per_job=16)
    got = mdsf.structure_factor(synth.pack_float4(pos, w), box, None, (64, 64, 64),
                                tuning=dict(variant=variant, batch=256)).cpu().numpy()
    e, rms = errors(got, ref)
    print(f"256-frame batch, variant {variant}: max err {e:.2e}, rms {rms:.2e} of max(S)")
    assert e < TOL


# ------------------------------------------------------------ configuration 3
def _pow2_systems(dev, seed=7):
    """Power-of-two systems (the bucketed chain) to run in the same graph as
    the 2^a 3^b 5^c ones."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    out = []
    for dims, n, t, L in (((256, 256, 128), 200_000, 70, (16.0, 13.856, 8.0)), ((128, 64, 256), 40_000, 24, (6, 3, 12)),
                          ((64, 64, 64), 5_000, 20, (3.0, 3.0, 3.0))):
        p = torch.rand((t, n, 4), generator=g, device=dev)
        p[..., :3] *= torch.tensor(L, dtype=torch.float32, device=dev)
        p[..., 3] = torch.tensor([1.0, 6.0, 7.0, 8.0], device=dev)[torch.randint(0, 4, (n,), generator=g, device=dev)]
        out.append(dict(pos_w=p, box=np.asarray(L, np.float64), dims=list(dims)))
    return out


def test_config3_uneven_systems_one_graph(oracle_pool):
    """The 64 uneven systems of the benchmark (random_batch(64, seed=5): 5k-300k
    atoms, 3-16 nm boxes, 2^a 3^b 5^c grids in 48-256) plus three power-of-two
    systems, in one CUDA graph over 8 streams.  The system with the most
    atoms, the one with the largest grid and the power-of-two systems run
    every frame; the others their first 3 frames (their atom counts, boxes
    and grids unchanged).  Every system is compared with the oracle."""
    from mdsf.batch import BatchedSystems, random_batch
    dev = torch.device("cuda", torch.cuda.current_device())
    systems = random_batch(64, seed=5, device=dev)
    big = max(range(64), key=lambda i: systems[i]["pos_w"].shape[1])
    grid = max(range(64), key=lambda i: int(np.prod(systems[i]["dims"])))
    for i, s in enumerate(systems):
        if i not in (big, grid):
            s["pos_w"] = s["pos_w"][:3].contiguous()
    systems += _pow2_systems(dev)
    b = BatchedSystems(systems, n_streams=8, device=dev)
    b.run()
    torch.cuda.synchronize()
    variants = [b.tuning(i)["variant"] for i in range(len(systems))]
    assert 3 in variants and 4 in variants, variants
    jobs = []
    for s in systems:
        p = s["pos_w"].cpu().numpy()
        jobs.append((p[..., :3], np.asarray(s["box"], np.float64), p[0, :, 3].astype(np.int32), tuple(s["dims"])))
    refs = pool_hist_sf(oracle_pool, jobs)
    worst = (0.0, 0.0, None)
    for i, ref in enumerate(refs):
        e, rms = errors(b.sf[i].cpu().numpy(), ref)
        if e > worst[0]:
            worst = (e, rms, i)
        assert e < TOL, (i, systems[i]["dims"], systems[i]["pos_w"].shape, e)
    e, rms, i = worst
    print(f"config 3 ({len(systems)} systems; largest {systems[big]['pos_w'].shape[1]} atoms x "
          f"{systems[big]['pos_w'].shape[0]} frames, largest grid {systems[grid]['dims']}): worst system {i} "
          f"{systems[i]['dims']} max err {e:.2e}, rms {rms:.2e} of max(S)")


# ------------------------------------------------------------ configuration 4
def pool_amplitudes(pool, r, f, q, chunk=1024):
    parts = pool.starmap(odirect.amplitudes, [(r, f, q[a:a + chunk]) for a in range(0, len(q), chunk)],
                         chunksize=1)
    return np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts])


def pool_grad(pool, r, f, q, g, A, B, chunk=1024):
    parts = pool.starmap(odirect.grad_chunk, [(r, f, q[a:a + chunk], g[a:a + chunk], A[a:a + chunk],
                                               B[a:a + chunk]) for a in range(0, len(q), chunk)], chunksize=1)
    return sum(p[0] for p in parts), sum(p[1] for p in parts)


def _loss_and_grad(r, f, q, target):
    rt = torch.from_numpy(r).cuda().requires_grad_(True)
    S = mdsf.direct_sf(rt, torch.from_numpy(f).cuda(), q)
    loss = torch.mean((torch.log1p(S) - torch.log1p(target)) ** 2, dim=-1).sum()
    loss.backward()
    return S.detach().cpu().numpy(), rt.grad.cpu().numpy()


def test_config4_forward_and_adjoint_at_size(oracle_pool):
    """20,000 atoms in a 6 nm cube, 65,536 q (three Ewald-sphere slices and a
    5-15 nm^-1 shell), target S from positions perturbed by sigma = 0.05 nm,
    loss MSE(log(1 + S)).  Forward vs the FP64 direct sum; dL/dr on every atom
    vs the FP64 analytic gradient; 10 atoms vs FP64 central differences."""
    r, f, r_t = synth.direct_system(20_000, 6.0, seed=0)
    q = synth.ewald_q_set(65_536)
    qd = torch.from_numpy(q).cuda()
    with torch.no_grad():
        target = mdsf.direct_sf(torch.from_numpy(r_t).cuda(), torch.from_numpy(f).cuda(), qd)
    S, gr = _loss_and_grad(r, f, qd, target)
    A, B = pool_amplitudes(oracle_pool, r, f, q)
    S64 = A * A + B * B
    e_norm = float(np.linalg.norm(S - S64) / np.linalg.norm(S64))
    e_max, rms = errors(S, S64)
    print(f"config 4 forward (20k atoms, 65,536 q): norm err {e_norm:.2e}, max err {e_max:.2e}, rms {rms:.2e} of max(S)")
    assert e_norm < 2e-5
    tgt = target.cpu().numpy().astype(np.float64)
    _, g = odirect.loss_log1p_mse(S64, tgt)
    gr_ref, _ = pool_grad(oracle_pool, r, f, q, g, A, B)
    e_g = float(np.linalg.norm(gr - gr_ref) / np.linalg.norm(gr_ref))
    atoms = list(range(0, 20_000, 1999))[:10]
    fd = odirect.fd_grad_moved(r, f, q, tgt, A, B, h=1e-5, atoms=atoms)
    np.testing.assert_allclose(gr_ref[atoms], fd, rtol=1e-4, atol=1e-4 * np.abs(gr_ref[atoms]).max())
    e_fd = float(np.linalg.norm(gr[atoms] - fd) / np.linalg.norm(fd))
    print(f"config 4 adjoint: dL/dr norm err {e_g:.2e} vs FP64 gradient (all atoms), {e_fd:.2e} vs FP64 central "
          f"differences (h = 1e-5 nm, {len(atoms)} atoms)")
    assert e_g < 1e-4 and e_fd < 1e-4


def test_config4_batch_of_32_systems(oracle_pool):
    """32 systems of 20,000 atoms per launch (shared q set): systems 0 and 31
    forward vs FP64, system 31's gradient vs the FP64 analytic gradient."""
    rs, fs, ts = zip(*[synth.direct_system(20_000, 6.0, seed=100 + s) for s in range(32)])
    q = synth.ewald_q_set(65_536)
    qd = torch.from_numpy(q).cuda()
    R, Fw = np.stack(rs), np.stack(fs)
    with torch.no_grad():
        target = mdsf.direct_sf(torch.from_numpy(np.stack(ts)).cuda(), torch.from_numpy(Fw).cuda(), qd)
    S, gr = _loss_and_grad(R, Fw, qd, target)
    for s in (0, 31):
        A, B = pool_amplitudes(oracle_pool, rs[s], fs[s], q)
        S64 = A * A + B * B
        e = float(np.linalg.norm(S[s] - S64) / np.linalg.norm(S64))
        print(f"config 4 batch: system {s} forward norm err {e:.2e}")
        assert e < 2e-5
    _, g = odirect.loss_log1p_mse(S64, target[31].cpu().numpy().astype(np.float64))
    gr_ref, _ = pool_grad(oracle_pool, rs[31], fs[31], q, g, A, B)
    e_g = float(np.linalg.norm(gr[31] - gr_ref) / np.linalg.norm(gr_ref))
    print(f"config 4 batch: system 31 dL/dr norm err {e_g:.2e}")
    assert e_g < 1e-4


# ------------------------------------------------------------ configuration 5
def test_config5_512_cubed_streamed(oracle_pool):
    """1,000,000 atoms in a 25 nm cube (6 x 6 columns) on the 512^3 grid,
    4 frames streamed from pinned host memory in 2-frame chunks through the
    public API, then get_dplot and the Ewald slices."""
    pos, box, w = synth.columnar(n_atoms=1_000_000, box=(25.0, 25.0, 25.0), n_cols=(6, 6), lattice=25.0 / 6,
                                 frames=4, seed=11)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).pin_memory()
    sf = mdsf.structure_factor(p4, box, None, (512, 512, 512), stream_chunk=2)
    ref, = pool_hist_sf(oracle_pool, [(pos, box, w, (512, 512, 512))], frames_per_job=1)
    e, rms = errors(sf.cpu().numpy(), ref)
    print(f"config 5 (1M atoms, 512^3, 4 frames streamed): max err {e:.2e}, rms {rms:.2e} of max(S)")
    assert e < TOL
    del ref
    check_post(sf, box)
