"""Many systems of uneven size and grid shape in one CUDA graph.

:class:`BatchedSystems` wraps ``msf_batch`` (``include/msf.h``): every system
(its own atom count, frame count, box and grid) gets a plan; the workspaces
share one device buffer; all histogram chains are captured into one CUDA
graph spread over several streams; :meth:`run` replays it with one launch.
Replaces calling ``dens.compute_sf`` (dens.py:166) once per trajectory.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import c_p, call, load
from .plan import stream_ptr


class BatchedSystems:
    """systems: list of dicts with keys
    ``pos_w`` (T, N, 4) float32 CUDA tensor (x, y, z, electrons), ``box`` (3,),
    ``dims`` (n0, n1, n2) and optionally ``wrap``, ``batch``, ``variant``, ``tile_w``.
    The ``sf`` attribute holds one FP64 accumulator per system.  A system
    without ``batch``/``variant``/``tile_w`` takes the autotuner's cached
    tuning of its grid shape (:mod:`mdsf.tune`); with ``autotune=True`` shapes
    missing from the cache are tuned first (``tune_candidates`` candidates
    each, at the system's atom count).
    """

    def __init__(self, systems, n_streams=4, device=None, autotune=False, tune_candidates=4):
        from . import tune as _tune
        self._lib = load()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.systems = list(systems)
        n = len(self.systems)
        self.tuned_shapes = 0
        tunings = []
        for s in self.systems:
            dims = tuple(int(v) for v in s["dims"])
            if any(k in s for k in ("batch", "variant", "tile_w")):
                tunings.append({})
                continue
            t = _tune.lookup(dims)
            if t is None and autotune:
                t = _tune.tune(dims, n_atoms=int(s["pos_w"].shape[1]), max_candidates=tune_candidates,
                               frames=16, device=self.device)
                self.tuned_shapes += 1
            tunings.append(t or {})
        arr = (_lib.BatchSystem * n)()
        self.sf = []
        self._keep = []
        for i, s in enumerate(self.systems):
            p = s["pos_w"]
            if p.dtype != torch.float32 or p.dim() != 3 or p.shape[-1] != 4 or not p.is_contiguous():
                raise ValueError("pos_w must be a contiguous (T, N, 4) float32 CUDA tensor")
            d0, d1, d2 = (int(v) for v in s["dims"])
            sf = torch.zeros((d0, d1, d2 // 2 + 1), dtype=torch.float64, device=self.device)
            self.sf.append(sf)
            self._keep.append(p)
            arr[i].pos_w = c_p(p.data_ptr())
            arr[i].scale = c_p(0)
            arr[i].sf = c_p(sf.data_ptr())
            arr[i].n_atoms = p.shape[1]
            arr[i].n_frames = p.shape[0]
            arr[i].box = (C.c_double * 3)(*[float(b) for b in s["box"]])
            arr[i].n0, arr[i].n1, arr[i].n2 = d0, d1, d2
            arr[i].flags = _lib.MSF_WRAP if s.get("wrap") else 0
            arr[i].batch = int(s.get("batch", tunings[i].get("batch", 0)))
            arr[i].variant = int(s.get("variant", tunings[i].get("variant", 0)))
            arr[i].tile_w = int(s.get("tile_w", tunings[i].get("tile_w", 0)))
        h = c_p()
        call("msf_batch_create", C.byref(h), arr, n, int(n_streams))
        self._h = h
        nbytes = self._lib.msf_batch_workspace_bytes(h)
        with torch.cuda.device(self.device):
            self.workspace = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
            call("msf_batch_bind", h, c_p(self.workspace.data_ptr()), nbytes, stream_ptr(self.device))
        self.workspace_bytes = nbytes

    def run(self):
        """Replay the graph: sf += the frame sum of every system (stream ordered)."""
        with torch.cuda.device(self.device):
            call("msf_batch_run", self._h, stream_ptr(self.device))

    def zero(self):
        for s in self.sf:
            s.zero_()

    def tuning(self, i):
        q = (_lib.c_int * 8)()
        call("msf_batch_query", self._h, i, q)
        return dict(variant=int(q[0]), tile_w=int(q[1]), batch=int(q[3]), tma=bool(q[6]))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and getattr(self, "_lib", None) is not None:
            self._lib.msf_batch_destroy(h)
            self._h = None


def random_batch(n_systems=64, seed=5, atoms=(5_000, 300_000), box=(3.0, 16.0), frames=(20, 200),
                 sizes=None, device=None):
    """Config-3-like systems generated on the device (log-uniform atom counts,
    boxes in [3, 16] nm, grid dims from 2^a 3^b 5^c sizes in [48, 256],
    20-200 frames, weights from {1, 6, 7, 8})."""
    from .synth import smooth_sizes
    rng = np.random.default_rng(seed)
    sizes = sizes or smooth_sizes(48, 256)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    out = []
    for _ in range(n_systems):
        n = int(np.exp(rng.uniform(np.log(atoms[0]), np.log(atoms[1]))))
        t = int(rng.integers(frames[0], frames[1] + 1))
        L = rng.uniform(box[0], box[1], 3)
        if rng.random() < 0.3:
            L[:] = L[0]
        dims = [int(rng.choice(sizes)) for _ in range(3)]
        p = torch.rand((t, n, 4), generator=g, device=dev, dtype=torch.float32)
        p[..., :3] *= torch.tensor(L, dtype=torch.float32, device=dev)
        w = torch.tensor([1.0, 6.0, 7.0, 8.0], device=dev)[torch.randint(0, 4, (n,), generator=g, device=dev)]
        p[..., 3] = w
        out.append(dict(pos_w=p, box=L, dims=dims))
    return out
