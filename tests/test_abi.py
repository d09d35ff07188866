"""C-ABI checks that need no GPU: every function declared in include/gpe.h is exported by libgpe.so, status
names are stable, and argument errors are reported before any device work."""
import ctypes as C
import re

import numpy as np

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "gpe.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gpe_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(gpe_mod):
    lib = gpe_mod.lib()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_error_names(gpe_mod):
    lib = gpe_mod.lib()
    for code, name in [(0, b"GPE_OK"), (-1, b"GPE_ERR_CUDA"), (-4, b"GPE_ERR_BAD_ARG"), (-6, b"GPE_ERR_CAPACITY"),
                       (-8, b"GPE_ERR_TIMEOUT"), (42, b"GPE_ERR_UNKNOWN")]:
        assert lib.gpe_error_name(code) == name
    assert lib.gpe_version() >= 100


def test_bad_arguments_rejected_without_device(gpe_mod):
    lib = gpe_mod.lib()
    from gpe import scenes

    p = scenes.dam_params()
    doms = gpe_mod.make_domains([(0, 0, 1, 1)])
    h = C.c_void_p()
    # null output handle, no scenes, negative capacity: rejected before the device is touched
    assert lib.gpe_pbf_create(C.byref(p), doms, 1, 10, None) == gpe_mod.ERR_BAD_ARG
    assert lib.gpe_pbf_create(C.byref(p), doms, 0, 10, C.byref(h)) == gpe_mod.ERR_BAD_ARG
    assert lib.gpe_pbf_create(C.byref(p), doms, 1, -1, C.byref(h)) == gpe_mod.ERR_BAD_ARG
    bad = p.copy()
    bad.h = -1.0
    assert lib.gpe_pbf_create(C.byref(bad), doms, 1, 10, C.byref(h)) == gpe_mod.ERR_BAD_ARG
    flat = gpe_mod.make_domains([(0, 0, 0, 1)])
    assert lib.gpe_pbf_create(C.byref(p), flat, 1, 10, C.byref(h)) == gpe_mod.ERR_BAD_ARG
    mp = scenes.elastic_params(16, 32)
    mp.nx = 2
    assert lib.gpe_mpm_create(C.byref(mp), 10, C.byref(h)) == gpe_mod.ERR_BAD_ARG
    for fn in ("gpe_pbf_step", "gpe_pbf_stage", "gpe_mpm_step", "gpe_mpm_stage"):
        assert getattr(lib, fn)(None, 1, None) == gpe_mod.ERR_BAD_ARG
    assert lib.gpe_pbf_destroy(None) == gpe_mod.ERR_BAD_ARG


def test_no_device_reports_device_error(gpe_mod, monkeypatch):
    # on a machine without a GPU the create call fails with a status, never a crash
    lib = gpe_mod.lib()
    cnt = C.c_int(0)
    try:
        rt = C.CDLL("libcudart.so")
        have = rt.cudaGetDeviceCount(C.byref(cnt)) == 0 and cnt.value > 0
    except OSError:
        have = False
    if have:
        return
    from gpe import scenes

    p = scenes.dam_params()
    h = C.c_void_p()
    rc = lib.gpe_pbf_create(C.byref(p), gpe_mod.make_domains([(0, 0, 1, 1)]), 1, 10, C.byref(h))
    assert rc == gpe_mod.ERR_DEVICE
    assert b"cuda" in lib.gpe_last_error_message().lower()


def test_extents_beyond_the_cell_range_are_refused(gpe_mod):
    """A scene whose extent / cell is not finite or reaches 2^30 cells along an edge is refused with
    GPE_ERR_CAPACITY before the cell count is cast to int32 (and before the device is touched)."""
    lib = gpe_mod.lib()
    from gpe import scenes

    p = scenes.dam_params()
    h = C.c_void_p()
    for ext in ((1e30, 1.0), (1.0, float("inf")), (float(2 ** 31) * 0.02, 1.0)):
        doms = gpe_mod.make_domains([(0.0, 0.0, ext[0], ext[1])])
        assert lib.gpe_pbf_create(C.byref(p), doms, 1, 10, C.byref(h)) == gpe_mod.ERR_CAPACITY, ext
        fn = lib.gpe_pbf_predict_sort_noalloc
        fn.restype = C.c_int32
        fn.argtypes = [C.POINTER(gpe_mod.PbfParams), C.POINTER(gpe_mod.Domain), C.c_void_p, C.c_void_p, C.c_int64,
                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        base = 0x10000
        rc = fn(C.byref(p), doms, base, base, 4, base, base, base, base, base, 16, None)
        assert rc == gpe_mod.ERR_CAPACITY, ext


def test_noalloc_refuses_misaligned_buffers_before_any_launch(gpe_mod):
    """The allocation-free sort reads and writes caller memory as float2 and 32-bit words; a pointer that is
    not aligned for that (here one float past an aligned base) is refused with GPE_ERR_BAD_ARG before any
    device work, so the call is safe to make without a GPU."""
    lib = gpe_mod.lib()
    from gpe import scenes

    p = scenes.dam_params()
    fn = lib.gpe_pbf_predict_sort_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.POINTER(gpe_mod.PbfParams), C.POINTER(gpe_mod.Domain), C.c_void_p, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    doms = gpe_mod.make_domains([(0.0, 0.0, 0.32, 0.32)])
    cells = 16 * 16
    base = 0x100000
    good = [base] * 7
    for slot, off in ((0, 4), (1, 4), (2, 4), (3, 4), (4, 2), (5, 2), (6, 2)):
        args = list(good)
        args[slot] = base + off
        rc = fn(C.byref(p), doms, args[0], args[1], 64, args[2], args[3], args[4], args[5], args[6], cells, None)
        assert rc == gpe_mod.ERR_BAD_ARG, slot
        assert b"aligned" in lib.gpe_last_error_message()
