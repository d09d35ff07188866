"""MLS-MPM parity of the CUDA engine (through the C ABI) against the oracle.

Stage tests feed both sides identical FP32 inputs. The grid after P2G is a sum of float atomics whose order
is not fixed, so grid fields are compared to 1e-5 of the field's scale; particle fields after G2P to 1e-5 of
their scale plus the FP32 rounding of the coordinates.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS32 = np.finfo(np.float32).eps


def _scene(kind):
    import gpe
    from gpe import scenes

    g = np.random.default_rng(12)
    if kind == "reference":
        p = scenes.reference_mpm_params()
        x, v, Cm, F, J = scenes.reference_mpm_block()
        return p, x, v, Cm, F, J, None
    p = scenes.elastic_params(4096, 64)
    n = 4096
    x = g.uniform(0.25, 0.75, (n, 2)).astype(np.float32)
    v = g.normal(0, 0.5, (n, 2)).astype(np.float32)
    Cm = g.normal(0, 2.0, (n, 4)).astype(np.float32)
    F = (np.tile(np.eye(2).ravel(), (n, 1)) + g.normal(0, 0.02, (n, 4))).astype(np.float32)
    J = g.uniform(0.97, 1.03, n).astype(np.float32)
    mat = None
    if kind == "corotated":
        p.material = gpe.MPM_MAT_COROTATED
    elif kind == "snow":
        p.material = gpe.MPM_MAT_SNOW
    elif kind == "fluid":
        p.material = gpe.MPM_MAT_FLUID
        p.k_bulk, p.gamma = 10.0, 1.0
    elif kind == "neohookean":
        p.material = gpe.MPM_MAT_NEOHOOKEAN
    elif kind == "sand":
        p.material = gpe.MPM_MAT_SAND
        p.nu = 0.3
        J = (1.0 + g.uniform(0.0, 0.5, n)).astype(np.float32)  # J = 1 + q, q the plastic strain so far
    elif kind == "mixed":
        # every material of the library, in fifths of the particle array
        p.flags = gpe.MPM_FLAG_PER_PARTICLE_MATERIAL
        p.k_bulk, p.gamma = 10.0, 1.0
        mat = (np.arange(n) * 5 // n).astype(np.int32)
    return p, x, v, Cm, F, J, mat


KINDS = ["reference", "corotated", "snow", "fluid", "neohookean", "sand", "mixed"]


def _engine(gpe_mod, p, x, v, Cm, F, J, mat, sort_interval=0):
    p = p.copy()
    p.sort_interval = sort_interval
    e = gpe_mod.Mpm(p, capacity=len(x))
    e.set_state(x, v, Cm, F, J, mat)
    return e


def _close(a, b, scale, what, rel=1e-5, floor=0.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    err = np.abs(a - b)
    tol = rel * scale + floor
    bad = err > tol
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} beyond tolerance; max err {err.max():.3e}"


@pytest.mark.parametrize("kind", KINDS)
def test_p2g_stage(gpe_mod, oracle, cuda_ok, kind):
    p, x, v, Cm, F, J, mat = _scene(kind)
    e = _engine(gpe_mod, p, x, v, Cm, F, J, mat)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    e.stage(gpe_mod.MPM_STAGE_P2G)
    g = e.grid()
    want = oracle.MpmOracle(p).p2g(x, v, Cm, F, J, mat)
    _close(g[:, 2], want[:, 2], np.abs(want[:, 2]).max(), "grid mass")
    _close(g[:, :2], want[:, :2], np.abs(want[:, :2]).max(), "grid momentum", rel=2e-5)
    assert e.status() == 0


@pytest.mark.parametrize("sort", [False, True])
def test_p2g_odd_count_sorted_and_unsorted(gpe_mod, oracle, cuda_ok, sort):
    """P2G takes two consecutive particles per thread: an odd count leaves the last thread one particle;
    unsorted input puts almost every pair across a run boundary (the first particle scattered on its own),
    sorted input joins most pairs and makes long runs."""
    p, x, v, Cm, F, J, mat = _scene("corotated")
    n = 4093
    x, v, Cm, F, J = x[:n], v[:n], Cm[:n], F[:n], J[:n]
    e = _engine(gpe_mod, p, x, v, Cm, F, J, mat)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    if sort:
        e.stage(gpe_mod.MPM_STAGE_SORT)
    e.stage(gpe_mod.MPM_STAGE_P2G)
    g = e.grid()
    want = oracle.MpmOracle(p).p2g(x, v, Cm, F, J, mat)
    _close(g[:, 2], want[:, 2], np.abs(want[:, 2]).max(), "grid mass")
    _close(g[:, :2], want[:, :2], np.abs(want[:, :2]).max(), "grid momentum", rel=2e-5)
    assert e.status() == 0


@pytest.mark.parametrize("kind", KINDS)
def test_grid_and_g2p_stages(gpe_mod, oracle, cuda_ok, kind):
    p, x, v, Cm, F, J, mat = _scene(kind)
    e = _engine(gpe_mod, p, x, v, Cm, F, J, mat)
    o = oracle.MpmOracle(p)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    e.stage(gpe_mod.MPM_STAGE_P2G)
    raw = e.grid()[:, :3].astype(np.float64)
    e.stage(gpe_mod.MPM_STAGE_GRID)
    upd = e.grid()
    want = o.grid_update(raw)
    vs = np.abs(want[:, :2]).max()
    _close(upd[:, :2], want[:, :2], vs, "grid velocity", rel=1e-6, floor=0.0)
    e.stage(gpe_mod.MPM_STAGE_G2P)
    x1, v1, C1, F1, J1 = e.get_state()
    wx, wv, wC, wF, wJ = o.g2p(upd[:, :3].astype(np.float64), x, v, Cm, F, J, mat)
    _close(x1, wx, np.abs(wx), "x", rel=1e-6, floor=4 * EPS32 * np.abs(wx).max())
    _close(v1, wv, np.abs(wv).max(), "v")
    _close(C1, wC, np.abs(wC).max(), "C", rel=2e-5)
    if kind != "fluid" and kind != "mixed":
        _close(F1, wF, np.abs(wF).max(), "F", rel=2e-5)
    if kind != "corotated":
        sel = slice(None) if mat is None else (mat != gpe_mod.MPM_MAT_COROTATED)
        _close(J1[sel], wJ[sel], np.abs(wJ[sel]).max(), "J", rel=2e-5)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("steps", [1, 4])
def test_multi_step_calls(gpe_mod, oracle, cuda_ok, kind, steps):
    p, x, v, Cm, F, J, mat = _scene(kind)
    e = _engine(gpe_mod, p, x, v, Cm, F, J, mat)
    e.step(steps)
    x1, v1, C1, F1, J1 = e.get_state()
    wx, wv, wC, wF, wJ = oracle.MpmOracle(p).step(x, v, Cm, F, J, mat, n_steps=steps)
    rel = 1e-5 * steps
    _close(x1, wx, np.abs(wx), "x", rel=rel, floor=8 * EPS32 * np.abs(wx).max())
    _close(v1, wv, np.abs(wv).max(), "v", rel=10 * rel)
    _close(C1, wC, np.abs(wC).max(), "C", rel=10 * rel)
    if kind in ("corotated", "snow", "neohookean", "sand") or kind == "reference":
        _close(F1, wF, np.abs(wF).max(), "F", rel=10 * rel)
    if kind == "mixed":  # the engine keeps no F for fluid particles
        sel = mat != gpe_mod.MPM_MAT_FLUID
        _close(F1[sel], wF[sel], np.abs(wF[sel]).max(), "F", rel=10 * rel)
    if kind in ("snow", "sand"):
        _close(J1, wJ, np.abs(wJ).max(), "J", rel=10 * rel)
    assert e.status() == 0


def test_spatial_sort_keeps_results_and_order(gpe_mod, cuda_ok):
    p, x, v, Cm, F, J, mat = _scene("mixed")
    perm = np.random.default_rng(3).permutation(len(x))
    a = _engine(gpe_mod, p, x, v, Cm, F, J, mat, sort_interval=0)
    b = _engine(gpe_mod, p, x, v, Cm, F, J, mat, sort_interval=1)
    for _ in range(3):
        a.step(2)
        b.step(2)
    sa, sb = a.get_state(), b.get_state()
    # get_state returns particles at their original indices even after re-sorting
    for fa, fb, nm in zip(sa, sb, "xvCFJ"):
        _close(fb, fa, np.abs(fa).max() + 1e-30, nm, rel=1e-4)
    del perm


def test_mpm_edge_cases(gpe_mod, cuda_ok):
    from gpe import scenes

    p = scenes.elastic_params(16, 32)
    e = gpe_mod.Mpm(p, capacity=8)
    e.set_state(np.zeros((0, 2), np.float32))
    e.step(3)
    e.set_state(np.array([[0.5, 0.5]], np.float32))
    e.step(2)
    x, v, _, _, _ = e.get_state()
    assert x[0, 1] < 0.5 and v[0, 1] < 0
    with pytest.raises(gpe_mod.GpeError) as ei:
        e.set_state(np.zeros((9, 2), np.float32))
    assert ei.value.status == gpe_mod.ERR_CAPACITY
    bad = np.array([[0.5, np.nan]], np.float32)
    e.set_state(bad)
    e.step(1)
    x, _, _, _, _ = e.get_state()
    assert np.all(np.isfinite(x))  # handleOOB resets non-finite particles to the box centre
    assert e.status() & gpe_mod.STATUS_NONFINITE
    e.close()


# ----- several scenes in one engine --------------------------------------------------------------------
def _batch(gpe_mod, seed=3):
    """Three scenes of different grids (32 x 48, 64 x 64, 40 x 40 nodes over one dx), every material mixed,
    particles in each scene's interior, given in an order that interleaves the scenes."""
    g = np.random.default_rng(seed)
    p = _scene("mixed")[0]
    sizes = [(32, 48), (64, 64), (40, 40)]
    scenes, parts = [], []
    for q, (nx, ny) in enumerate(sizes):
        lo = (2 * p.dx, 2 * p.dx)
        hi = ((nx - 3) * p.dx, (ny - 3) * p.dx)
        scenes.append(gpe_mod.make_mpm_scene(nx, ny, lo, hi))
        n = 700 + 300 * q
        x = np.stack([g.uniform(0.25, 0.75, n) * nx * p.dx, g.uniform(0.25, 0.75, n) * ny * p.dx], 1)
        v = g.normal(0, 0.5, (n, 2))
        Cm = g.normal(0, 2.0, (n, 4))
        F = np.tile(np.eye(2).ravel(), (n, 1)) + g.normal(0, 0.02, (n, 4))
        J = g.uniform(0.97, 1.03, n)
        mat = g.integers(0, 5, n)
        parts.append((x, v, Cm, F, J, mat, np.full(n, q)))
    cat = [np.concatenate([pp[k] for pp in parts]) for k in range(7)]
    order = g.permutation(len(cat[0]))
    x, v, Cm, F, J, mat, sid = (a[order] for a in cat)
    f32 = np.float32
    return (p, scenes, x.astype(f32), v.astype(f32), Cm.astype(f32), F.astype(f32), J.astype(f32),
            mat.astype(np.int32), sid.astype(np.int32))


def _scene_params(p, sc):
    q = p.copy()
    q.nx, q.ny = sc.nx, sc.ny
    q.clamp_lo[0], q.clamp_lo[1] = sc.clamp_lo[0], sc.clamp_lo[1]
    q.clamp_hi[0], q.clamp_hi[1] = sc.clamp_hi[0], sc.clamp_hi[1]
    return q


@pytest.mark.parametrize("sort_interval", [0, 2])
def test_batched_scenes_match_each_scene_alone(gpe_mod, oracle, cuda_ok, sort_interval):
    """Each scene of a batched engine against the oracle run on that scene alone (its own grid and clamp),
    over several steps, with and without the periodic sort."""
    p, scenes, x, v, Cm, F, J, mat, sid = _batch(gpe_mod)
    p = p.copy()
    p.sort_interval = sort_interval
    e = gpe_mod.Mpm(p, capacity=len(x), scenes=scenes)
    e.set_state(x, v, Cm, F, J, mat, scene_id=sid)
    steps = 4
    e.step(steps)
    x1, v1, C1, F1, J1 = e.get_state()
    assert e.status() == 0
    for q, sc in enumerate(scenes):
        sel = sid == q
        wx, wv, wC, wF, wJ = oracle.MpmOracle(_scene_params(p, sc)).step(x[sel], v[sel], Cm[sel], F[sel], J[sel],
                                                                        mat[sel], n_steps=steps)
        rel = 1e-5 * steps
        _close(x1[sel], wx, np.abs(wx), f"scene {q} x", rel=rel, floor=8 * EPS32 * np.abs(wx).max())
        _close(v1[sel], wv, np.abs(wv).max(), f"scene {q} v", rel=10 * rel)
        _close(C1[sel], wC, np.abs(wC).max(), f"scene {q} C", rel=10 * rel)
        keep = mat[sel] != gpe_mod.MPM_MAT_FLUID
        _close(F1[sel][keep], wF[keep], np.abs(wF[keep]).max(), f"scene {q} F", rel=10 * rel)


def test_batched_grid_holds_each_scene_grid(gpe_mod, oracle, cuda_ok):
    """P2G of a batched engine: the node array is the scenes' grids one after the other, each the oracle's
    P2G of that scene's particles alone."""
    p, scenes, x, v, Cm, F, J, mat, sid = _batch(gpe_mod, seed=5)
    e = gpe_mod.Mpm(p, capacity=len(x), scenes=scenes)
    e.set_state(x, v, Cm, F, J, mat, scene_id=sid)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    e.stage(gpe_mod.MPM_STAGE_P2G)
    g = e.grid()
    off = 0
    for q, sc in enumerate(scenes):
        sel = sid == q
        want = oracle.MpmOracle(_scene_params(p, sc)).p2g(x[sel], v[sel], Cm[sel], F[sel], J[sel], mat[sel])
        got = g[off:off + sc.nx * sc.ny]
        _close(got[:, 2], want[:, 2], np.abs(want[:, 2]).max(), f"scene {q} grid mass")
        _close(got[:, :2], want[:, :2], np.abs(want[:, :2]).max(), f"scene {q} grid momentum", rel=2e-5)
        off += sc.nx * sc.ny
    assert e.status() == 0


def test_batched_scene_ids_are_checked(gpe_mod, cuda_ok):
    torch = pytest.importorskip("torch")
    p, scenes, x, v, Cm, F, J, mat, sid = _batch(gpe_mod)
    e = gpe_mod.Mpm(p, capacity=len(x), scenes=scenes)
    e.set_state(x, v, Cm, F, J, mat)
    bad = sid.copy()
    bad[7] = 3
    with pytest.raises(gpe_mod.GpeError):
        e.set_scene_ids(bad)  # host ids: checked on the host
    dbad = torch.from_numpy(bad).cuda()
    with pytest.raises(gpe_mod.GpeError):
        e.set_scene_ids(dbad)  # device ids: checked by a kernel, reported without a fault
    e.set_scene_ids(torch.from_numpy(sid).cuda())
    e.step(2)
    assert e.status() == 0
    with pytest.raises(gpe_mod.GpeError):
        e.emit(gpe_mod.make_hose((0.2, 0.2), (1.0, 0.0), 0.05, 0.01, 0.0, 4))
