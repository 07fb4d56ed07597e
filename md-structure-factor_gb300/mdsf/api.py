"""Device API of the structure-factor path (torch tensors in, torch tensors out).

Every function here launches libmsf kernels on the current CUDA stream; there
is no CPU implementation behind any of them.

* :func:`structure_factor` -- frames -> electron-weighted histogram -> rfftn
  -> |F|^2 -> FP64 sum over frames (the per-frame loop of dens.py:277-318 in
  histogram form, rescale dens.py:46-62 and wrap dens.py:204-221 fused).
* :func:`hist_grid`, :func:`power_accum` -- the two halves separately.
* :func:`get_dplot` -- dens.py:142-163 on the device.
* :func:`ewald_slices` -- plot2d.py:218-267 on the device.
* :class:`DirectSF` -- differentiable direct-sum S(q).
"""
from __future__ import annotations

import math
import threading

import numpy as np
import torch

from . import tune as _tune
from ._lib import MSF_CONTINUE, MSF_WRAP, c_p, call
from .plan import get_plan, stream_ptr


def _dev(device):
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


def to_device(x, device, dtype=None):
    """Tensor on `device` (host numpy arrays go through pinned memory)."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.from_numpy(np.ascontiguousarray(x))
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if t.device != device:
        if t.device.type == "cpu" and not t.is_pinned():
            t = t.pin_memory()
        t = t.to(device, non_blocking=True)
    return t.contiguous()


def frame_scale(box):
    """(scale (T,3) or None, binning box (3,)) as dens.py:52-53 computes them."""
    b = np.asarray(box.detach().cpu().numpy() if isinstance(box, torch.Tensor) else box,
                   dtype=np.float64)
    if b.ndim == 1:
        return None, b
    avg = np.average(b, axis=0)
    return avg / b, avg


def _ptr(t):
    return c_p(t.data_ptr()) if t is not None else c_p(0)


_side_streams = {}


def check_axes(*axes):
    """RegularGridInterpolator's condition on grid axes: 1-D, finite,
    strictly ascending (the GPU interpolation assumes it)."""
    for i, a in enumerate(axes):
        a = np.asarray(a, np.float64)
        if a.ndim != 1 or a.size < 2 or not np.all(np.isfinite(a)):
            raise ValueError(f"axis {i} must be a finite 1-D array of at least 2 points")
        if not np.all(np.diff(a) > 0):
            raise ValueError(f"The points in dimension {i} must be strictly ascending")


def _side_stream(device):
    s = _side_streams.get(device)
    if s is None:
        s = torch.cuda.Stream(device)
        _side_streams[device] = s
    return s


class _Staging:
    """The ring of device buffers host-streamed chunks are copied into, one
    ring per device, kept across calls.  ``free[b]`` is an event recorded on
    the caller's stream after the last chain that reads buffer b -- in this
    call or an earlier one -- and every copy into b waits on it first, so a
    call issued while an earlier call's kernels are still queued cannot
    overwrite positions they have yet to bin.  (Per-call buffers from the
    caching allocator cannot give that: a block freed at the end of one call
    is handed to the next as soon as the copy stream is idle, while the
    caller's stream may still be behind.)  Chunk i of a call takes slot
    (turn + i) mod 3 and ``turn`` advances by the call's chunk count, so the
    copies of a call issued back to back with the previous one (three chunks
    each by default) wait on that call's chains one by one rather than on
    its end.  The buffers are allocated on the copy stream and only grow;
    :func:`release_staging` frees them."""

    SLOTS = 3

    def __init__(self):
        self.bufs = [None] * self.SLOTS
        self.free = [None] * self.SLOTS
        self.turn = 0
        self.lock = threading.Lock()

    def view(self, b, side, shape, dtype):
        """Buffer b as a `shape` tensor of `dtype`, grown if needed; call
        on the copy stream after it has waited on ``free[b]``."""
        nbytes = math.prod(shape) * torch.empty((), dtype=dtype).element_size()
        buf = self.bufs[b]
        if buf is None or buf.numel() < nbytes:
            with torch.cuda.stream(side):
                self.bufs[b] = None   # the old block returns to the copy stream's pool, behind the wait
                buf = self.bufs[b] = torch.empty(nbytes, dtype=torch.uint8, device=side.device)
        return buf[:nbytes].view(dtype).view(shape)


_stagings = {}


def release_staging(device=None):
    """Free the host-streaming staging buffers of `device` (all devices if
    None) once the kernels that read them have finished (the next streamed
    call allocates them again)."""
    for dev in ([_dev(device)] if device is not None else list(_stagings)):
        stg = _stagings.pop(dev, None)
        if stg is None:
            continue
        with stg.lock:
            side = _side_stream(dev)
            for ev in stg.free:
                if ev is not None:
                    side.wait_event(ev)
            stg.bufs = [None] * stg.SLOTS


_CHAIN = {4: "msf_hist_sf_f32", 3: "msf_hist_sf_f32xyz", 8: "msf_hist_sf_f64"}


def _chunk_sizes(T, chunk, lead=True):
    """Frames per host-to-device chunk: `chunk` each, or (lead) a first
    chunk of a quarter of it -- its copy is the one no kernel hides -- and
    the rest in near-equal chunks of at most `chunk` frames.  For 100 frames
    in chunks of 64 that is 16 + 42 + 42: 25.0 against 25.9 us per frame for
    64 + 36 on the GB300, copies and kernels together."""
    if not lead or T <= chunk:
        return [min(chunk, T - f) for f in range(0, T, chunk)]
    first = max(1, chunk // 4)
    rest = T - first
    n = -(-rest // chunk)
    return [first] + [rest // n + (1 if i < rest % n else 0) for i in range(n)]


def _launch_chain(plan, code, p, w, N, T, sc, flags, sf, st):
    if code == 4:
        call("msf_hist_sf_f32", plan.handle, c_p(p), N, T, c_p(sc), flags, _ptr(sf), st)
    else:
        call(_CHAIN[code], plan.handle, c_p(p), c_p(w), N, T, c_p(sc), flags, _ptr(sf), st)


def structure_factor(positions, box, weights=None, grid_dims=None, *, wrap=False, mean=False,
                     out=None, device=None, tuning=None, stream_chunk=None, zero_copy=False, scale=None):
    """Sum over frames of |rfftn(histogram)|^2, FP64, shape (n0, n1, n2//2+1).

    positions: (T, N, 3) or (N, 3) float32/float64, or (T, N, 4) float32 with
      the electron count in the 4th component (then ``weights`` is ignored).
      Host arrays are copied to the device in chunks of ``stream_chunk``
      frames on a side stream (double-buffered, pinned memory), overlapping
      the copies with the kernels of the previous chunk.  With ``zero_copy``
      the kernels instead read them in place from page-locked memory (one
      chain over all frames, no device copy of the trajectory; on GB300 the
      reads go over NVLink-C2C, measured slower than the staged copies for
      the 200k-atom workload: 23k against 35k frames/s).  A pinned tensor
      passed in must then stay unchanged until the stream has finished the
      call; anything else is first copied into pinned memory and the call
      waits for the kernels.
    box: (3,) box edges, or (T, 3) per-frame boxes (frames are rescaled to
      the mean box as dens.py:46-62 does and binned in the mean box).
    weights: (N,) integer electron counts.
    grid_dims: (n0, n1, n2).
    wrap: apply the reference's periodic wrap before binning (dens.py:211-212);
      otherwise atoms outside [0, L] are dropped (numpy.histogramdd range).
    mean: divide by the frame count (the reference saves the undivided sum).
    out: FP64 tensor to accumulate into (not zeroed).
    tuning: plan fields (variant, batch, tile_w, ...); None takes the
      autotuner's cached tuning for this grid shape on this GPU (see
      :mod:`mdsf.tune`), or the plan defaults when the cache has none.
    scale: (T, 3) per-frame rescale factors given explicitly, with ``box``
      the (3,) binning box: a slice of a longer trajectory then bins as the
      whole trajectory does (factors and mean box of dens.py:50-53 computed
      over every frame, see :func:`mdsf.shard.shard_inputs`).
    """
    device = _dev(device)
    pos = positions
    if pos.ndim == 2:
        pos = pos[None]
    T, N, C = pos.shape
    if scale is None:
        scale, L = frame_scale(box)
    else:
        L = np.asarray(box.detach().cpu().numpy() if isinstance(box, torch.Tensor) else box, dtype=np.float64)
        scale = np.asarray(scale.detach().cpu().numpy() if isinstance(scale, torch.Tensor) else scale,
                           dtype=np.float64)
        if L.shape != (3,) or scale.shape != (T, 3):
            raise ValueError("with scale=, box must be the (3,) binning box and scale (T, 3)")
    kw = dict(tuning) if tuning is not None else dict(_tune.lookup(grid_dims) or {})
    kw.setdefault("max_atoms", N)
    plan = get_plan(grid_dims, L, device=device, **kw)
    if out is None:
        sf = torch.zeros(plan.half_shape, dtype=torch.float64, device=device)
    else:
        sf = out
        if tuple(sf.shape) != plan.half_shape or sf.dtype != torch.float64 or not sf.is_contiguous():
            raise ValueError("out must be a contiguous float64 tensor of shape %s" % (plan.half_shape,))
    flags = MSF_WRAP if wrap else 0
    is64 = (pos.dtype == torch.float64) if isinstance(pos, torch.Tensor) else (pos.dtype == np.float64)
    if C == 4:
        code, tdt, esz = 4, torch.float32, 16
    elif C == 3:
        if weights is None:
            raise ValueError("weights are required for (T, N, 3) positions")
        code, tdt, esz = (8, torch.float64, 24) if is64 else (3, torch.float32, 12)
    else:
        raise ValueError("positions must be (T, N, 3) or (T, N, 4)")
    host = not (isinstance(pos, torch.Tensor) and pos.device.type == "cuda")
    with torch.cuda.device(device):
        st = stream_ptr(device)
        sc = None if scale is None else to_device(scale, device, torch.float64)
        wd = None
        if code != 4:
            wd = to_device(weights, device, torch.int32)
            if wd.numel() != N:
                raise ValueError("weights must have one entry per atom")
        wptr = wd.data_ptr() if wd is not None else 0
        scp = sc.data_ptr() if sc is not None else 0
        chunk = int(stream_chunk or plan.batch)   # one batch: the first copy hides soonest
        if host and zero_copy and N > 0 and T > 0:
            hp = pos if isinstance(pos, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(pos))
            owned = not (hp.dtype == tdt and hp.is_contiguous() and hp.is_pinned())
            if owned:
                hp = hp.to(tdt).contiguous().pin_memory()
            _launch_chain(plan, code, hp.data_ptr(), wptr, N, T, scp, flags, sf, st)
            if owned:   # the kernels read hp in place: it must outlive them
                torch.cuda.current_stream(device).synchronize()
        elif not host or T <= chunk or N == 0:
            p = to_device(pos, device, tdt)
            _launch_chain(plan, code, p.data_ptr(), wptr, N, T, scp, flags, sf, st)
        else:
            hp = pos if isinstance(pos, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(pos))
            if hp.dtype != tdt:
                hp = hp.to(tdt)
            if not hp.is_pinned():
                hp = hp.contiguous().pin_memory()
            main = torch.cuda.current_stream(device)
            side = _side_stream(device)
            # the short lead chunk pays only where the chunk calls overlap
            # (bucketed plans): 7% of an isolated 100-frame call against two
            # 50-frame chunks, and a tie back to back (42.5k against 42.4k
            # frames/s, interleaved on one GB300).  The chunks set the chain's
            # batches and so the rounding of the FP32 frame sums: the split
            # depends on the call's sizes only, never on the GPU's state.
            sizes = _chunk_sizes(T, chunk, lead=stream_chunk is None and plan.variant == 3)
            copied = [torch.cuda.Event() for _ in range(_Staging.SLOTS)]
            stg = _stagings.get(device)
            if stg is None:
                stg = _stagings[device] = _Staging()
            with stg.lock:
                f0 = 0
                for i, k in enumerate(sizes):
                    b = stg.turn % stg.SLOTS
                    stg.turn += 1
                    with torch.cuda.stream(side):
                        if stg.free[b] is not None:
                            side.wait_event(stg.free[b])
                        buf = stg.view(b, side, (k, N, C), tdt)
                        buf.copy_(hp[f0:f0 + k], non_blocking=True)
                        copied[b].record(side)
                    main.wait_event(copied[b])
                    # one chain over the chunks: a bucketed plan's x pass of
                    # one chunk then overlaps the plane FFT of the next
                    more = MSF_CONTINUE if i + 1 < len(sizes) else 0
                    _launch_chain(plan, code, buf.data_ptr(), wptr, N, k,
                                  scp + 24 * f0 if scp else 0, flags | more, sf, st)
                    ev = torch.cuda.Event()
                    ev.record(main)
                    stg.free[b] = ev
                    f0 += k
    if mean and T > 0:
        sf.div_(T)
    return sf


def hist_grid(positions, box, weights=None, grid_dims=None, *, scale=None, wrap=False, device=None,
              out=None):
    """int32 density grid of one frame (bit-exact numpy.histogramdd)."""
    device = _dev(device)
    plan = get_plan(grid_dims, np.asarray(box, np.float64), device=device)
    g = out if out is not None else torch.zeros(tuple(plan.dims), dtype=torch.int32, device=device)
    N = positions.shape[0]
    flags = MSF_WRAP if wrap else 0
    with torch.cuda.device(device):
        st = stream_ptr(device)
        sc = None if scale is None else to_device(np.asarray(scale, np.float64), device, torch.float64)
        if positions.shape[-1] == 4:
            p = to_device(positions, device, torch.float32)
            call("msf_hist_grid_f32", plan.handle, _ptr(p), N, _ptr(sc), flags, _ptr(g), st)
        else:
            w = to_device(weights, device, torch.int32)
            is64 = (positions.dtype == torch.float64) if isinstance(positions, torch.Tensor) \
                else (positions.dtype == np.float64)
            if is64:
                p = to_device(positions, device, torch.float64)
                call("msf_hist_grid_f64", plan.handle, _ptr(p), _ptr(w), N, _ptr(sc), flags, _ptr(g), st)
            else:
                p = to_device(positions, device, torch.float32)
                call("msf_hist_grid_f32xyz", plan.handle, _ptr(p), _ptr(w), N, _ptr(sc), flags,
                     _ptr(g), st)
    return g


def power_accum(grids, sf=None, *, device=None, tuning=None):
    """sf += sum_g |rfftn(g)|^2 for grids (G, n0, n1, n2) int32 / float32 / float64."""
    device = _dev(device)
    g = to_device(grids, device)
    if g.ndim == 3:
        g = g[None]
    dims = tuple(g.shape[1:])
    plan = get_plan(dims, (1.0, 1.0, 1.0), device=device, **(tuning or {}))
    if sf is None:
        sf = torch.zeros(plan.half_shape, dtype=torch.float64, device=device)
    fn = {torch.int32: "msf_power_accum_i32", torch.float32: "msf_power_accum_f32",
          torch.float64: "msf_power_accum_f64"}[g.dtype]
    with torch.cuda.device(device):
        call(fn, plan.handle, _ptr(g), g.shape[0], _ptr(sf), stream_ptr(device))
    return sf


def get_dplot(sf):
    """dens.py:142-163 on the device: (n0, n1, nh) -> (n0-2, n1-2, 2nh-3)."""
    n0, n1, nh = sf.shape
    out = torch.empty((n0 - 2, n1 - 2, 2 * nh - 3), dtype=torch.float64, device=sf.device)
    with torch.cuda.device(sf.device):
        call("msf_sfplt", _ptr(sf), n0, n1, nh, _ptr(out), stream_ptr(sf.device))
    return out


def plot_axes(half_shape, L):
    """kgridplt axis coordinates, dens.py:336-342: (ix - n/2)*2*pi/L with true division."""
    n = (half_shape[0] - 2, half_shape[1] - 2, half_shape[2] * 2 - 3)
    return [np.array([(ix - n[a] / 2) * 2.0 * math.pi / L[a] for ix in range(n[a])]) for a in range(3)]


def ewald_slices(D, X, Y, Z, wavelength):
    """Ewald-sphere slices (xy, xz, yz) of D (p0, p1, p2) with axes X, Y, Z."""
    dev = D.device
    p0, p1, p2 = D.shape
    if not any(isinstance(a, torch.Tensor) for a in (X, Y, Z)):
        check_axes(X, Y, Z)
    if (len(X), len(Y), len(Z)) != (p0, p1, p2):
        raise ValueError("axes must match the grid shape")
    X = to_device(np.asarray(X, np.float64) if not isinstance(X, torch.Tensor) else X, dev, torch.float64)
    Y = to_device(np.asarray(Y, np.float64) if not isinstance(Y, torch.Tensor) else Y, dev, torch.float64)
    Z = to_device(np.asarray(Z, np.float64) if not isinstance(Z, torch.Tensor) else Z, dev, torch.float64)
    xy = torch.empty((p0, p1), dtype=torch.float64, device=dev)
    xz = torch.empty((p0, p2), dtype=torch.float64, device=dev)
    yz = torch.empty((p1, p2), dtype=torch.float64, device=dev)
    K = 2.0 * math.pi / float(wavelength)
    with torch.cuda.device(dev):
        call("msf_ewald", _ptr(D.contiguous()), p0, p1, p2, _ptr(X), _ptr(Y), _ptr(Z), K,
             _ptr(xy), _ptr(xz), _ptr(yz), stream_ptr(dev))
    return xy, xz, yz


def ewald_from_sf(sf, L, wavelength):
    """get_dplot + kgridplt axes + Ewald slices, all on the device."""
    D = get_dplot(sf)
    X, Y, Z = plot_axes(tuple(sf.shape), L)
    return ewald_slices(D, X, Y, Z, wavelength)


def cylindrical_average(D, X, Y, Z, ucell, format=False):
    """PLOT_RAD_NEW's cylindrical (r, z) average (plot2d.py:578-645) with the
    ring sums on the GPU.  D: centred S (p0, p1, p2) CUDA float64 (e.g.
    ``get_dplot(sf)``); X, Y, Z its axes; ucell 3x3.  Returns numpy
    (final, rfin, zfin, oa) as the reference builds them: 400 radii up to 0.95
    of half the smaller in-plane q extent, max(int(20*2*pi*r), 1) angles per
    ring, NaN -> smallest average, division by the mean unless ``format``,
    mirrored to (-r, r)."""
    dev = D.device
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    Z = np.asarray(Z, np.float64)
    check_axes(X, Y, Z)
    if (len(X), len(Y), len(Z)) != tuple(D.shape):
        raise ValueError("axes must match the grid shape")
    u = np.asarray(ucell, np.float64)
    a1, a2, a3 = u[0], u[1], u[2]
    b1 = (np.cross(a2, a3)) / (np.dot(a1, np.cross(a2, a3)))
    b2 = (np.cross(a3, a1)) / (np.dot(a2, np.cross(a3, a1)))
    b3 = (np.cross(a1, a2)) / (np.dot(a3, np.cross(a1, a2)))
    b_inv = np.ascontiguousarray(np.linalg.inv(np.vstack((b1, b2, b3))))
    Rmax = min((X[-1] - X[0]) * u[0][0], (Y[-1] - Y[0]) * u[1][1]) / 2.0
    Rmax *= 0.95
    rarr = np.linspace(0.0, Rmax, 400)
    zar = np.linspace(Z[0], Z[-1], Z.shape[0])
    circ = 2. * np.pi * rarr
    nth = np.array([max(int(20.0 * c), 1) for c in circ], dtype=np.int32)
    p0, p1, p2 = D.shape
    oa = torch.empty((400, Z.shape[0]), dtype=torch.float64, device=dev)
    Xd, Yd, Zd = (to_device(a, dev) for a in (X, Y, Z))
    rd, nd, zd = to_device(rarr, dev), to_device(nth, dev), to_device(zar, dev)
    with torch.cuda.device(dev):
        call("msf_cyl_average", _ptr(D.contiguous()), p0, p1, p2, _ptr(Xd), _ptr(Yd), _ptr(Zd),
             c_p(b_inv.ctypes.data), _ptr(rd), _ptr(nd), 400, _ptr(zd), Z.shape[0], _ptr(oa), stream_ptr(dev))
    o = oa.cpu().numpy()
    mn = np.nanmin(o)
    o = np.where(np.isnan(o), mn, o)
    if not format:
        o /= np.average(o)
    final = np.append(o[::-1, :], o[1:], axis=0)
    rfin = np.append(-rarr[::-1], rarr[1:])
    return final, rfin, zar, o


# ------------------------------------------------------------ direct sum
def _pack_rf(r, f):
    if f.dim() == r.dim() - 1:
        return torch.cat([r, f.unsqueeze(-1)], dim=-1).contiguous()
    raise ValueError("f must have one weight per atom")


class DirectSF(torch.autograd.Function):
    """S(q) = |sum_j f_j exp(i q.r_j)|^2 with a hand-written adjoint.

    r: (N, 3) or (S, N, 3) float32 CUDA; f: (N,) or (S, N); q: (M, 3) shared
    or (S, M, 3).  Returns (M,) or (S, M).  Gradients flow to r and f.
    """

    @staticmethod
    def forward(ctx, r, f, q):
        squeeze = r.dim() == 2
        r3 = r.unsqueeze(0) if squeeze else r
        f2 = f.unsqueeze(0) if f.dim() == 1 and not squeeze else (f.unsqueeze(0) if squeeze else f)
        if f2.shape[0] != r3.shape[0]:
            f2 = f2.expand(r3.shape[0], -1)
        S_, N = r3.shape[0], r3.shape[1]
        rf = _pack_rf(r3.float(), f2.float())
        q_shared = q.dim() == 2
        M = q.shape[-2]
        q4 = torch.cat([q.float(), torch.zeros(q.shape[:-1] + (1,), device=q.device)], -1).contiguous()
        Sq = torch.empty((S_, M), dtype=torch.float32, device=r.device)
        AB = torch.empty((S_, M, 2), dtype=torch.float32, device=r.device)
        with torch.cuda.device(r.device):
            call("msf_direct_fwd", _ptr(rf), N, _ptr(q4), M, S_, int(q_shared), _ptr(Sq), _ptr(AB),
                 stream_ptr(r.device))
        ctx.save_for_backward(rf, q4, AB)
        ctx.meta = (squeeze, q_shared, f.dim())
        return Sq[0] if squeeze else Sq

    @staticmethod
    def backward(ctx, gS):
        rf, q4, AB = ctx.saved_tensors
        squeeze, q_shared, fdim = ctx.meta
        S_, N = rf.shape[0], rf.shape[1]
        M = q4.shape[-2]
        g = (gS.unsqueeze(0) if squeeze else gS).float().contiguous()
        grad = torch.empty((S_, N, 4), dtype=torch.float32, device=rf.device)
        with torch.cuda.device(rf.device):
            call("msf_direct_bwd", _ptr(rf), N, _ptr(q4), M, S_, int(q_shared), _ptr(g), _ptr(AB),
                 _ptr(grad), stream_ptr(rf.device))
        gr = grad[..., :3]
        gf = grad[..., 3]
        if squeeze:
            gr, gf = gr[0], gf[0]
        elif fdim == 1:
            gf = gf.sum(0)
        return gr, gf, None


def direct_sf(r, f, q):
    return DirectSF.apply(r, f, q)
