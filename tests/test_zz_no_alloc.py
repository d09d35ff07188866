"""gpe_pbf_predict_sort_noalloc, the allocation-free predict + sort entry point, checked through the C ABI
against the engine's own PREDICT_SORT stage.

Some callers cannot call cudaMalloc: a plugin whose host framework owns all device memory, or a real-time
loop that must not allocate once running. This entry point serves them by keeping its scratch in a static
device array. Its results must equal the regular stage bit for bit (the sort tolerance used everywhere),
on two calls in a row — the second with fewer particles, so scratch left by the first call must not leak
into it. This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(seed, n_side):
    from gpe import scenes

    p = scenes.dam_params(iters=2)
    pos, vel, boxes = scenes.dam_break(n_side=n_side, seed=seed)
    vel = np.random.default_rng(seed + 100).normal(0, 0.4, pos.shape).astype(np.float32)
    return p, pos, vel, boxes[0]


def _engine_stage(gpe_mod, p, pos, vel, box):
    e = gpe_mod.Pbf(p, [box], capacity=len(pos))
    e.set_state(pos, vel)
    e.stage(gpe_mod.PBF_STAGE_PREDICT_SORT)
    out = {"pos": e.field(gpe_mod.PBF_FIELD_POS), "disp": e.field(gpe_mod.PBF_FIELD_DISP),
           "key": e.field(gpe_mod.PBF_FIELD_KEY), "perm": e.field(gpe_mod.PBF_FIELD_PERM),
           "cell_start": e.field(gpe_mod.PBF_FIELD_CELL_START)}
    n_cells = e.num_cells
    e.close()
    return out, n_cells


def _fn(gpe_mod):
    fn = gpe_mod.lib().gpe_pbf_predict_sort_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.POINTER(gpe_mod.PbfParams), C.POINTER(gpe_mod.Domain), C.c_void_p, C.c_void_p, C.c_int64,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    return fn


def _noalloc(gpe_mod, p, pos, vel, box, n_cells):
    import torch

    n = len(pos)
    d_pos = torch.from_numpy(pos).cuda()
    d_vel = torch.from_numpy(vel).cuda()
    o_pos = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    o_pred = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    o_key = torch.empty(n, dtype=torch.int32, device="cuda")
    o_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    o_cs = torch.empty(n_cells + 1, dtype=torch.int32, device="cuda")
    dom = gpe_mod.make_domains([box])
    torch.cuda.synchronize()
    rc = _fn(gpe_mod)(C.byref(p), dom, d_pos.data_ptr(), d_vel.data_ptr(), n, o_pos.data_ptr(), o_pred.data_ptr(),
                      o_key.data_ptr(), o_perm.data_ptr(), o_cs.data_ptr(), n_cells, None)
    gpe_mod.check(rc, "gpe_pbf_predict_sort_noalloc")
    torch.cuda.synchronize()
    return {"pos": o_pos.cpu().numpy(), "pred": o_pred.cpu().numpy(),
            "key": o_key.cpu().numpy().view(np.uint32), "perm": o_perm.cpu().numpy().view(np.uint32),
            "cell_start": o_cs.cpu().numpy().view(np.uint32)}


def test_noalloc_sort_matches_stage_twice(gpe_mod, cuda_ok):
    for seed, n_side in ((0, 96), (5, 40)):
        p, pos, vel, box = _scene(seed, n_side)
        want, n_cells = _engine_stage(gpe_mod, p, pos, vel, box)
        got = _noalloc(gpe_mod, p, pos, vel, box, n_cells)
        for k in ("key", "perm", "cell_start"):
            assert np.array_equal(got[k], want[k]), f"{k} differs (scene {seed})"
        assert np.array_equal(got["pos"].view(np.uint32), want["pos"].view(np.uint32)), f"pos differs (scene {seed})"
        # the engine's step holds x and d = x* - x: the FP32 difference of the no-alloc sort's x* and x
        disp = (got["pred"] - got["pos"]).astype(np.float32)
        assert np.array_equal(disp.view(np.uint32), want["disp"].view(np.uint32)), f"x* differs (scene {seed})"


def test_noalloc_rejects_sizes_beyond_its_scratch(gpe_mod, cuda_ok):
    import torch

    p, pos, vel, box = _scene(1, 16)
    buf = torch.zeros(16, dtype=torch.float32, device="cuda").data_ptr()
    dom = gpe_mod.make_domains([box])
    fn = _fn(gpe_mod)
    too_many = (1 << 18) + 1
    rc = fn(C.byref(p), dom, buf, buf, too_many, buf, buf, buf, buf, buf, 128 * 128, None)
    assert rc == gpe_mod.ERR_CAPACITY
    assert b"static scratch" in gpe_mod.lib().gpe_last_error_message()
    ext = (np.float32(2048 * p.h), np.float32(1024 * p.h))  # about 2^21 cells
    big = gpe_mod.make_domains([(0.0, 0.0, float(ext[0]), float(ext[1]))])
    cells = int(np.ceil(ext[0] / np.float32(p.h))) * int(np.ceil(ext[1] / np.float32(p.h)))
    rc = fn(C.byref(p), big, buf, buf, 4, buf, buf, buf, buf, buf, cells, None)
    assert rc == gpe_mod.ERR_CAPACITY
