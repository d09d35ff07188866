"""The drop-in layer around the reference's tick: emitters, device-resident particle counts, publish into a
chunk view, graph-capturable step sequences, and the cuda-engine.h compatibility library driven by the two
headless example loops (the reference's PBF-master.cpp / MPM-master.cpp without the window thread).

Tolerances: emitted lattice positions within 1e-4 absolute of a float64 restatement of the hose layout (the
device may contract the lattice arithmetic into FMAs); everything the engine computes twice on the same
input (a dynamic-count graph against a fixed-count engine, a captured enqueue against step) bit for bit,
except MPM, whose node sums are float atomics (relative 1e-5 of the field's scale).
"""
import ctypes as C
import json
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
BIN = ROOT / "gpu-physics-engine_gb300" / "compat" / "bin"


def _hose_lattice(origin, velocity, nozzle, spacing, dt, steps):
    """Jitter-free hose layout (emitterKernel, PBF.cu:984-1011): column i % width, row i / width."""
    speed = math.hypot(*velocity)
    w = max(1, int(math.floor(nozzle / spacing + 0.5)))
    r = max(1, int(math.floor(speed * dt * steps / spacing + 0.5)))
    t = np.array(velocity, np.float64) / speed
    nrm = np.array([-t[1], t[0]])
    i = np.arange(w * r)
    across = ((i % w) - 0.5 * (w - 1)) * spacing
    along = -((i // w) + 0.5) * spacing
    return np.asarray(origin, np.float64) + across[:, None] * nrm + along[:, None] * t


def _sorted_rows(a):
    a = np.asarray(a, np.float64)
    return a[np.lexsort(a.T[::-1])]


def _pbf(gpe_mod, dynamic=True, capacity=20000, iters=2):
    from gpe import scenes

    p = scenes.reference_pbf_params(iters=iters)
    if dynamic:
        p.flags |= gpe_mod.PBF_DYNAMIC_COUNT
    pos, vel, boxes = scenes.reference_pbf_block()
    e = gpe_mod.Pbf(p, boxes, capacity=capacity)
    e.set_state(pos, vel)
    return e, p, pos, vel, boxes


def test_pbf_emit_lattice_velocity_and_count(gpe_mod, cuda_ok):
    e, p, pos, vel, _ = _pbf(gpe_mod)
    hose = gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 0.0, 20)
    req = e.emit(hose, seed=3)
    want = _hose_lattice((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 1.0, 20)
    assert req == len(want) == 160
    assert e.n == len(pos) + req
    x, v, _ = e.get_state()
    np.testing.assert_array_equal(x[:len(pos)], pos)  # existing particles untouched, new ones appended
    got = _sorted_rows(x[len(pos):])
    np.testing.assert_allclose(got, _sorted_rows(want), rtol=0, atol=1e-4)
    # the stream velocity is clamped to v_max (velocityClamp in emitterKernel, PBF.cu:990-991)
    vs = np.float64(1.0) / math.hypot(1.0, -0.3)
    np.testing.assert_allclose(v[len(pos):], np.tile([1.0 * vs, -0.3 * vs], (req, 1)), rtol=2e-6, atol=0)
    assert e.status() == 0


def test_pbf_emit_drops_atoms_outside_the_scene(gpe_mod, cuda_ok):
    e, p, pos, vel, _ = _pbf(gpe_mod)
    origin, velo = (4.3, 150.0), (1.0, -0.3)
    want = _hose_lattice(origin, velo, 8.0, 1.05, 1.0, 20)
    assert np.abs(want[:, 0]).min() > 1e-2  # no lattice point sits on the wall
    keep = want[want[:, 0] >= 0.0]
    assert 0 < len(keep) < len(want)
    req = e.emit(gpe_mod.make_hose(origin, velo, 8.0, 1.05, 0.0, 20), seed=1)
    assert req == len(want)
    assert e.n == len(pos) + len(keep)
    x, _, _ = e.get_state()
    np.testing.assert_allclose(_sorted_rows(x[len(pos):]), _sorted_rows(keep), rtol=0, atol=1e-4)


def test_pbf_emit_jitter_is_seeded(gpe_mod, cuda_ok):
    hose = gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 0.05, 20)
    want = _sorted_rows(_hose_lattice((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 1.0, 20))
    outs = []
    for seed in (5, 5, 6):
        e, _, pos, _, _ = _pbf(gpe_mod)
        e.emit(hose, seed=seed)
        x, _, _ = e.get_state()
        outs.append(_sorted_rows(x[len(pos):]))
    np.testing.assert_array_equal(outs[0], outs[1])
    assert not np.array_equal(outs[0], outs[2])
    # every atom stays within 6 standard deviations of the jitter of a lattice point
    d = np.linalg.norm(outs[0][:, None, :] - want[None, :, :], axis=2).min(1)
    assert d.max() < 6 * 0.05 * math.sqrt(2)


def test_pbf_emit_respects_capacity(gpe_mod, cuda_ok):
    from gpe import scenes

    pos, _, _ = scenes.reference_pbf_block()
    e, _, _, _, _ = _pbf(gpe_mod, capacity=len(pos) + 100)
    req = e.emit(gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 0.0, 20), seed=0)
    assert req == 160
    assert e.n == len(pos) + 100
    assert e.status() & gpe_mod.STATUS_CAPACITY


def test_emit_refuses_a_hose_beyond_int32_or_capacity(gpe_mod, cuda_ok):
    """Width x rows is computed in 64-bit: a hose whose count overflows int32 (or exceeds the engine's
    capacity) is refused with GPE_ERR_CAPACITY instead of wrapping to a wrong count."""
    from gpe import scenes

    e, _, pos, _, _ = _pbf(gpe_mod, capacity=5000)
    n0 = e.n
    for nozzle, spacing in ((1e9, 1e-3), (8.0, 1e-5), (4e5, 1.05)):
        with pytest.raises(gpe_mod.GpeError) as ei:
            e.emit(gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), nozzle, spacing, 0.0, 20))
        assert ei.value.status == gpe_mod.ERR_CAPACITY
    assert e.n == n0 and e.status() == 0
    mp = scenes.elastic_params(2048, 64)
    mp.flags |= gpe_mod.MPM_FLAG_DYNAMIC_COUNT
    m = gpe_mod.Mpm(mp, capacity=4096)
    m.set_state(np.full((16, 2), 0.5, np.float32))
    with pytest.raises(gpe_mod.GpeError) as ei:
        m.emit(gpe_mod.make_hose((0.5, 0.5), (1.0, 0.0), 1e9, 1e-4, 0.0, 10))
    assert ei.value.status == gpe_mod.ERR_CAPACITY
    m.close()


def test_pbf_emit_needs_dynamic_count(gpe_mod, cuda_ok):
    e, _, _, _, _ = _pbf(gpe_mod, dynamic=False)
    with pytest.raises(gpe_mod.GpeError) as ei:
        e.emit(gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 0.0, 20))
    assert ei.value.status == gpe_mod.ERR_NOT_READY


def test_pbf_dynamic_graph_follows_emitted_atoms(gpe_mod, cuda_ok):
    """A step graph captured with a device-resident count, replayed after an emit, equals a fixed-count
    engine started from the same particles, bit for bit."""
    a, p, pos, vel, boxes = _pbf(gpe_mod)
    a.step(2)
    a.emit(gpe_mod.make_hose((50.0, 150.0), (1.0, -0.3), 8.0, 1.05, 0.02, 20), seed=9)
    x1, v1, _ = a.get_state()
    a.step(2)  # same cached graph, more atoms
    xa, va, _ = a.get_state()
    b, _, _, _, _ = _pbf(gpe_mod, dynamic=False)
    b.set_state(x1, v1)
    b.step(2)
    xb, vb, _ = b.get_state()
    assert len(xa) == len(x1) > len(pos)
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(va, vb)


# ----- publish ------------------------------------------------------------------------------------------
def _view(gpe_mod, torch, chunks_x, chunks_y, dim, cap):
    pos = torch.full((chunks_x * chunks_y * cap, 2), float("nan"), device="cuda")
    vel = torch.full_like(pos, float("nan"))
    counts = torch.full((chunks_x * chunks_y,), -1, dtype=torch.int32, device="cuda")
    v = gpe_mod.View(pos.data_ptr(), vel.data_ptr(), counts.data_ptr(), chunks_x, chunks_y, dim, cap)
    return v, (pos, vel, counts)


def _device_struct(torch, view):
    raw = bytes(C.string_at(C.addressof(view), C.sizeof(view)))
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()


def _check_pbf_publish(bufs, x, v, cx, cy, dim, cap):
    pos, vel, counts = (t.cpu().numpy() for t in bufs)
    assert counts.sum() == len(x) and counts.max() <= cap
    rows = []
    for c in range(cx * cy):
        k = counts[c]
        px, pv = pos[c * cap:c * cap + k], vel[c * cap:c * cap + k]
        ox, oy = (c % cx) * dim, (c // cx) * dim
        assert np.all((px[:, 0] >= ox) & (px[:, 0] <= ox + dim) & (px[:, 1] >= oy) & (px[:, 1] <= oy + dim))
        rows.append(np.concatenate([px, pv], 1))
    np.testing.assert_array_equal(_sorted_rows(np.concatenate(rows)), _sorted_rows(np.concatenate([x, v], 1)))


def test_pbf_publish_host_and_device_view(gpe_mod, cuda_ok):
    torch = pytest.importorskip("torch")
    e, p, pos, vel, _ = _pbf(gpe_mod)
    e.step(3)
    x, v, _ = e.get_state()
    view, bufs = _view(gpe_mod, torch, 12, 6, 32.0, 1536)
    e.publish(view)
    torch.cuda.synchronize()
    _check_pbf_publish(bufs, x, v, 12, 6, 32.0, 1536)
    view2, bufs2 = _view(gpe_mod, torch, 12, 6, 32.0, 1536)
    dv = _device_struct(torch, view2)
    e.publish(dv.data_ptr(), view_mem=gpe_mod.MEM_DEVICE)
    torch.cuda.synchronize()
    _check_pbf_publish(bufs2, x, v, 12, 6, 32.0, 1536)


def test_pbf_publish_overflowing_chunks(gpe_mod, cuda_ok):
    """Chunks with more particles than chunk_capacity keep exactly chunk_capacity of them (PBFOutputKernel's
    give-back of slots past the capacity), all distinct particles of that chunk, and raise the capacity
    status bit."""
    torch = pytest.importorskip("torch")
    e, p, pos, vel, _ = _pbf(gpe_mod)
    e.step(2)
    x, v, _ = e.get_state()
    cx, cy, dim, cap = 12, 6, 32.0, 64
    view, bufs = _view(gpe_mod, torch, cx, cy, dim, cap)
    e.publish(view)
    torch.cuda.synchronize()
    vpos, vvel, counts = (t.cpu().numpy() for t in bufs)
    inv = np.float32(1.0 / dim)  # exact for dim = 32, as the kernel's x * (1 / chunk_dim)
    kx = np.clip(np.floor(x[:, 0].astype(np.float32) * inv).astype(np.int64), 0, cx - 1)
    ky = np.clip(np.floor(x[:, 1].astype(np.float32) * inv).astype(np.int64), 0, cy - 1)
    true = np.bincount(kx + ky * cx, minlength=cx * cy)
    assert true.max() > cap  # the block overflows some chunks
    np.testing.assert_array_equal(counts, np.minimum(true, cap))
    allrows = {tuple(r) for r in np.concatenate([x, v], 1).tolist()}
    for c in range(cx * cy):
        rows = np.concatenate([vpos[c * cap:c * cap + counts[c]], vvel[c * cap:c * cap + counts[c]]], 1)
        got = [tuple(r) for r in rows.tolist()]
        assert len(set(got)) == len(got) and all(r in allrows for r in got)
    assert e.status() & gpe_mod.STATUS_CAPACITY


def test_pbf_enqueue_captured_with_publish_replays(gpe_mod, cuda_ok):
    """enqueue + publish recorded into the caller's CUDA graph (instantiatePBFGraph's pattern), replayed with
    the device-resident view retargeted between replays (the reference's triple-buffered output), equals
    step() on a twin engine, bit for bit."""
    torch = pytest.importorskip("torch")
    a, p, pos, vel, _ = _pbf(gpe_mod)
    b, _, _, _, _ = _pbf(gpe_mod, dynamic=False)
    views = [_view(gpe_mod, torch, 12, 6, 32.0, 1536) for _ in range(2)]
    dv = _device_struct(torch, views[0][0])
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        st = torch.cuda.current_stream().cuda_stream
        a.enqueue(2, stream=st)
        a.publish(dv.data_ptr(), view_mem=gpe_mod.MEM_DEVICE, stream=st)
    for r in range(2):
        dv.copy_(_device_struct(torch, views[r][0]))
        g.replay()
        torch.cuda.synchronize()
        b.step(2)
        xb, vb, _ = b.get_state()
        xa, va, _ = a.get_state()
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(va, vb)
        _check_pbf_publish(views[r][1], xb, vb, 12, 6, 32.0, 1536)
    # the first target still holds the first replay's output
    assert views[0][1][2].sum().item() == len(pos)


# ----- MPM ----------------------------------------------------------------------------------------------
def _mpm(gpe_mod, dynamic=True, capacity=50000):
    from gpe import scenes

    p = scenes.reference_mpm_params()
    p.sort_interval = 0
    if dynamic:
        p.flags |= gpe_mod.MPM_FLAG_DYNAMIC_COUNT
    pos, vel = scenes.reference_mpm_block()[:2]
    e = gpe_mod.Mpm(p, capacity=capacity)
    e.set_state(pos, vel)
    return e, p, pos, vel


def test_mpm_emit_publish_and_buffers(gpe_mod, cuda_ok):
    torch = pytest.importorskip("torch")
    e, p, pos, vel = _mpm(gpe_mod)
    origin, velo = (60.0, 100.0), (2.0, -1.0)
    req = e.emit(gpe_mod.make_hose(origin, velo, 8.0, 1.0, 0.0, 10), seed=2)
    want = _hose_lattice(origin, velo, 8.0, 1.0, p.dt, 10)
    assert req == len(want)
    assert e.n == len(pos) + req
    x, v, Cm, F, J = e.get_state()
    np.testing.assert_allclose(_sorted_rows(x[len(pos):]), _sorted_rows(want), rtol=0, atol=1e-4)
    np.testing.assert_array_equal(v[len(pos):], np.tile(np.float32(velo), (req, 1)))
    np.testing.assert_array_equal(F[len(pos):], np.tile(np.float32([1, 0, 0, 1]), (req, 1)))
    np.testing.assert_array_equal(J[len(pos):], np.ones(req, np.float32))
    cap = 1000
    view, bufs = _view(gpe_mod, torch, 4, 2, 32.0, cap)
    e.publish(view)
    torch.cuda.synchronize()
    pp, pv, counts = (t.cpu().numpy() for t in bufs)
    n = e.n
    want_counts = np.clip(n - np.arange(8) * cap, 0, cap)
    np.testing.assert_array_equal(counts, want_counts)
    k = min(n, 8 * cap)
    np.testing.assert_array_equal(pp[:k], x[:k])
    np.testing.assert_array_equal(pv[:k], v[:k])
    bp = e.buffers()
    assert all(bp[k2] for k2 in ("pos", "vel", "C", "F", "J", "count"))
    cnt = (C.c_int32 * 2)()
    assert _cudart().cudaMemcpy(cnt, C.c_void_p(bp["count"]), C.c_size_t(8), 2) == 0  # device to host
    assert list(cnt) == [n, n]  # count[1] = count[0] at publish (MPMOutputKernel, MPM.cu:317)
    px = np.empty((n, 2), np.float32)
    assert _cudart().cudaMemcpy(px.ctypes.data_as(C.c_void_p), C.c_void_p(bp["pos"]), C.c_size_t(px.nbytes), 2) == 0
    np.testing.assert_array_equal(px, x)


def _cudart():
    import glob

    try:
        return C.CDLL("libcudart.so")
    except OSError:
        return C.CDLL(sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))[0])


def test_mpm_enqueue_captured_matches_step(gpe_mod, cuda_ok):
    torch = pytest.importorskip("torch")
    a, p, pos, vel = _mpm(gpe_mod)
    b, _, _, _ = _mpm(gpe_mod, dynamic=False)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        a.enqueue(3, stream=torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        b.step(3)
        xa, va = a.get_state()[:2]
        xb, vb = b.get_state()[:2]
        np.testing.assert_allclose(xa, xb, rtol=0, atol=1e-5 * np.abs(xb).max())
        np.testing.assert_allclose(va, vb, rtol=0, atol=1e-5 * max(np.abs(vb).max(), 1e-3))


# ----- the cuda-engine.h layer, end to end --------------------------------------------------------------
@pytest.mark.parametrize("prog", ["pbf_headless", "mpm_headless"])
def test_compat_headless_loop(gpe_mod, cuda_ok, prog):
    exe = BIN / prog
    assert exe.exists(), f"{exe} is not built"
    r = subprocess.run([str(exe), "200"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["published"] > 0 and out["misplaced"] == 0
    if prog == "pbf_headless":  # the arena's chunk-major members are live
        assert out["arena_atoms"] == out["engine_atoms"] and out["arena_inconsistent"] == 0
