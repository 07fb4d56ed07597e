"""The C ABI library without a GPU: it loads, exports every symbol that
include/msf.h declares, and its host-side argument checks return the
documented status codes (no kernel is launched by any call here)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

import mdsf
from mdsf import _lib

HEADER = os.path.join(ROOT, "include", "msf.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(msf_[a-z0-9_]+)\s*\(", src)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = mdsf.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)


def test_strerror_and_version():
    lib = mdsf.load()
    assert lib.msf_version() >= 100
    for code in _lib.ERRORS:
        assert lib.msf_strerror(code)
    assert lib.msf_strerror(-5) == b"atom outside the padded grid"


def _desc(dims=(64, 64, 64), box=(2.5, 2.5, 2.5), **kw):
    d = _lib.PlanDesc(*dims, kw.get("batch", 0), (C.c_double * 3)(*box), kw.get("variant", 0),
                      kw.get("tile_w", 0), kw.get("rows_per_block", 0), kw.get("deposit_block", 0),
                      kw.get("max_atoms", 0), kw.get("options", 0))
    return d


def create(**kw):
    lib = mdsf.load()
    h = C.c_void_p()
    st = lib.msf_plan_create(C.byref(h), C.byref(_desc(**kw)))
    return st, h


@pytest.mark.parametrize("kw,code", [
    (dict(dims=(1, 64, 64)), -2), (dict(dims=(64, 2048, 64)), -2), (dict(box=(0.0, 1, 1)), -1),
    (dict(box=(float("nan"), 1, 1)), -1), (dict(batch=-1), -1), (dict(variant=5), -1),
    (dict(tile_w=12), -1), (dict(deposit_block=100), -1), (dict(max_atoms=-1), -1),
    (dict(dims=(48, 48, 48), variant=3), -2), (dict(options=4), -1),
])
def test_plan_create_rejects(kw, code):
    st, h = create(**kw)
    assert st == code


def test_plan_layout_and_query():
    lib = mdsf.load()
    st, h = create(dims=(256, 256, 128), box=(16.0, 13.856, 8.0), batch=4, max_atoms=200_000)
    assert st == 0
    ws = lib.msf_plan_workspace_bytes(h)
    V, Vh = 256 * 256 * 128, 256 * 256 * 65
    assert ws >= 4 * (2 * 8 * Vh + 8 * 200_000)   # double-buffered spectra + atom buckets
    st2, h2 = create(dims=(256, 256, 128), box=(16.0, 13.856, 8.0), batch=4, max_atoms=200_000, options=1)
    assert st2 == 0
    assert lib.msf_plan_workspace_bytes(h2) < 4 * (4 * V + 8 * Vh)   # no density grids, one spectrum buffer
    lib.msf_plan_destroy(h2)
    q = (C.c_int32 * 8)()
    assert lib.msf_plan_query(h, q) == 0
    assert q[0] == 3 and q[3] == 4 and q[7] == 65   # bucketed variant, batch 4, nh
    st1, h1 = create(dims=(256, 256, 128), box=(16.0, 13.856, 8.0), batch=4, variant=1)
    assert st1 == 0 and lib.msf_plan_workspace_bytes(h1) >= 4 * (4 * V + 8 * Vh)
    lib.msf_plan_destroy(h1)
    # an unbound plan refuses work before touching the GPU
    assert lib.msf_hist_sf_f32(h, C.c_void_p(16), 10, 1, None, 0, C.c_void_p(16), None) == -6
    assert lib.msf_power_accum_i32(h, C.c_void_p(16), 1, C.c_void_p(16), None) == -6
    assert lib.msf_hist_sf_f32(h, C.c_void_p(16), 10, 1, None, 4, C.c_void_p(16), None) == -6
    assert lib.msf_plan_status(h, None) == -6
    assert lib.msf_plan_destroy(h) == 0


def test_plan_options_accepted():
    lib = mdsf.load()
    for opt in (0, 1, 2, 3):    # MSF_PLAN_NO_OVERLAP, MSF_PLAN_DIAG_STALL
        st, h = create(dims=(64, 64, 64), max_atoms=1000, options=opt)
        assert st == 0, opt
        lib.msf_plan_destroy(h)


def test_noalloc_host_checks():
    """Argument checks of the allocation-free entry points that return before
    any CUDA call."""
    lib = mdsf.load()
    box = (C.c_double * 3)(1.0, 1.0, 1.0)
    bx = C.cast(box, C.c_void_p)
    assert lib.msf_hist_sf_f32_noalloc(None, 10, 1, bx, 8, 8, 8, 0, None, None) == -1     # no sf
    assert lib.msf_hist_sf_f32_noalloc(None, 10, 1, bx, 8, 8, 8, 0, C.c_void_p(16), None) == -1   # no positions
    assert lib.msf_hist_sf_f32_noalloc(C.c_void_p(16), 10, 1, bx, 8, 8, 8, 2, C.c_void_p(16), None) == -1
    assert lib.msf_noalloc_init(8, 8, 8, None, None) == -1


def test_split_variant_for_odd_and_prime_sizes():
    lib = mdsf.load()
    for dims, variant in (((75, 81, 48), 4), ((64, 74, 26), 2), ((48, 48, 48), 4), ((512, 512, 512), 4),
                          ((48, 48, 14), 2), ((1024, 16, 16), 1)):
        st, h = create(dims=dims)
        assert st == 0
        q = (C.c_int32 * 8)()
        lib.msf_plan_query(h, q)
        assert q[0] == variant, dims
        lib.msf_plan_destroy(h)
    st, h = create(dims=(75, 81, 48), variant=1)
    assert st == -2


def test_null_arguments():
    lib = mdsf.load()
    assert lib.msf_plan_create(None, None) == -1
    assert lib.msf_hist_sf_f32(None, None, 0, 0, None, 0, None, None) == -1
    assert lib.msf_sfplt(None, 4, 4, 3, None, None) == -1
    assert lib.msf_sfplt(C.c_void_p(16), 5, 4, 3, C.c_void_p(16), None) == -2
    assert lib.msf_ewald(None, 2, 2, 2, None, None, None, 1.0, None, None, None, None) == -1
    assert lib.msf_direct_fwd(None, 10, None, 10, 0, 1, None, None, None) == -1
    assert lib.msf_direct_bwd(None, 0, None, 0, 1, 1, None, None, None, None) == 0
    assert lib.msf_gauss_grid_f64(None, None, None, 0, None, 1, None, None, None) == -1


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of msf_plan_desc and msf_batch_system have the C
    sizes and field offsets (compiled from include/msf.h with the host C
    compiler)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    from conftest import ROOT
    fields = {"msf_plan_desc": [f for f, _ in _lib.PlanDesc._fields_],
              "msf_batch_system": [f for f, _ in _lib.BatchSystem._fields_]}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "msf.h"', "int main(void) {"]
    for st, fs in fields.items():
        lines.append('printf("%%zu\\n", sizeof(%s));' % st)
        for f in fs:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (st, f))
    lines.append("return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for cls in (_lib.PlanDesc, _lib.BatchSystem):
        want.append(C.sizeof(cls))
        want += [getattr(cls, f).offset for f, _ in cls._fields_]
    assert out == want

