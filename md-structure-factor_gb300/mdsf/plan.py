"""Plans: a grid shape bound to one device workspace.

A :class:`Plan` wraps ``msf_plan`` (``include/msf.h``): it fixes the grid
(n0, n1, n2), the binning box and the number of frames processed per batch,
owns one device workspace (a torch uint8 tensor) holding the FFT tables,
the histogram bin edges, a batch of int32 density grids and their half
spectra, and is reused by every call.  One plan serves one stream at a time.
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import _lib
from ._lib import c_p, call, load

VARIANTS = {0: "auto", 1: "plane", 2: "split", 3: "bucketed", 4: "smooth"}


def stream_ptr(device=None):
    return c_p(torch.cuda.current_stream(device).cuda_stream)


class Plan:
    """``msf_plan`` plus its workspace on ``device``."""

    def __init__(self, dims, box, batch=0, variant=0, tile_w=0, rows_per_block=0,
                 deposit_block=0, max_atoms=0, options=0, device=None):
        lib = load()
        if not torch.cuda.is_available():
            raise RuntimeError("mdsf needs a CUDA device (GB300); no CPU fallback exists")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.dims = tuple(int(d) for d in dims)
        self.box = tuple(float(b) for b in box)
        desc = _lib.PlanDesc(self.dims[0], self.dims[1], self.dims[2], int(batch),
                             (C.c_double * 3)(*self.box), int(variant), int(tile_w),
                             int(rows_per_block), int(deposit_block), int(max_atoms), int(options))
        self.max_atoms = int(max_atoms)
        self.options = int(options)
        h = c_p()
        call("msf_plan_create", C.byref(h), C.byref(desc))
        self._h = h
        self._lib = lib
        nbytes = lib.msf_plan_workspace_bytes(h)
        with torch.cuda.device(self.device):
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            call("msf_plan_bind", h, c_p(self.workspace.data_ptr()), nbytes, stream_ptr())
        q = (_lib.c_int * 8)()
        call("msf_plan_query", h, q)
        self.variant, self.tile_w, self.rows_per_block, self.batch = q[0], q[1], q[2], q[3]
        self.deposit_block, self.plane_threads, self.nh = q[4], q[5], q[7]
        self.tma = bool(q[6])      # x pass fed by TMA tile loads
        self.workspace_bytes = nbytes

    @property
    def handle(self):
        return self._h

    @property
    def half_shape(self):
        return (self.dims[0], self.dims[1], self.dims[2] // 2 + 1)

    def status(self):
        """Synchronise and raise if a kernel latched an error (e.g. MSF_E_RANGE)."""
        call("msf_plan_status", self._h, stream_ptr(self.device))

    def tuning(self):
        return dict(variant=VARIANTS[self.variant], tile_w=self.tile_w,
                    rows_per_block=self.rows_per_block, batch=self.batch,
                    deposit_block=self.deposit_block, tma=self.tma,
                    overlap=not (self.options & 1))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and self._lib is not None:
            self._lib.msf_plan_destroy(h)
            self._h = None


_cache = {}
_cache_lock = threading.Lock()


def get_plan(dims, box, device=None, **tuning):
    """Cached plan for (device, dims, box, tuning)."""
    dev = torch.cuda.current_device() if device is None else torch.device(device).index
    key = (dev, tuple(int(d) for d in dims), tuple(float(b) for b in box),
           tuple(sorted((k, int(v)) for k, v in tuning.items())))
    with _cache_lock:
        p = _cache.get(key)
        if p is None:
            p = Plan(dims, box, device=torch.device("cuda", dev), **tuning)
            _cache[key] = p
        return p


def clear_plans():
    with _cache_lock:
        _cache.clear()
