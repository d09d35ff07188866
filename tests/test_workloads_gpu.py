"""Parity of the engine against the oracle on the full-size workloads it is measured on — the same scenes,
parameters and tunings as bench.py — rather than on small scenes only:

  * PBF, 1,048,576 particles (a 960 x 1024 lattice block and a 65,536-particle splash, h = 0.02,
    dt = 1/2000, 4 Jacobi iterations) with the tuning the autotuner picks for it (cell h, 256 threads,
    per-pass launches, candidate masks with skin 0.075 h): one step against the oracle, then the next
    step's predict + sort bit for bit;
  * PBF, 256 independent dam-break scenes (5.1 M particles, dt = 1/480) in one engine with the batched
    tuning (cell h, 128 threads): one step against the oracle, and three steps bit for bit against every
    scene run alone;
  * MLS-MPM, 65,536 fixed-corotated particles on 128^2 nodes (32 per cell, re-sorted by cell): P2G node
    fields and one step against the oracle, with the P2G taking its 5-round run reduction (two particles per
    lane, runs of more than 16 lanes on one stencil base node);
  * MLS-MPM, 4,194,304 mixed-material particles (water, snow, jelly) on 1024^2 nodes: P2G node fields and
    one step against the oracle.

Tolerances: keys, sorted order, cell starts, sorted x and the displacement d = x* - x bit for bit; FP32
fields after one step within 1e-5 of the field's scale (positions: of the coordinate, with a floor of 1e-6 of
the domain; the batched scenes' velocities from rest 2e-5, stated in the test).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS32 = np.finfo(np.float32).eps


def _close(a, b, tol, what):
    err = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    bad = err > tol
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} beyond tolerance; max err {err.max():.3e}"


def _pbf_step_close(p, x, v, r, rel_v=1e-5):
    """One PBF step of the engine (x, v) against the oracle's (r), both in the stable sorted order. Velocities
    are d / dt of the step's displacement, so no rounding of the (up to 1000 m) coordinates enters them."""
    _close(x, r["x"], 1e-5 * (np.abs(r["x"]) + 0.1 * np.abs(r["x"]).max()), "x after one step")
    _close(v, r["v"], rel_v * np.abs(r["v"]).max(), "v after one step")


# ----- PBF, 1M particles -------------------------------------------------------------------------------
def test_pbf_1m_particles_one_step_and_next_sort(gpe_mod, oracle, cuda_ok):
    from gpe import scenes

    p, pos, vel, boxes = scenes.million_workload(iters=4)
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_tuning(cell=0.0, block=256, persistent=0, skin=0.075)
    e.set_state(pos, vel)
    e.step(1)
    x, v, _ = e.get_state()
    assert e.status() == 0
    o = oracle.PbfOracle(p, boxes)
    r = o.step(pos, vel, None, 1)
    _pbf_step_close(p, x, v, r)
    # the next step's predict + cell sort, on the engine's own state, bit for bit
    e.stage(gpe_mod.PBF_STAGE_PREDICT_SORT)
    s = o.predict_sort(x, v)
    assert np.array_equal(e.field(gpe_mod.PBF_FIELD_KEY), s["key"])
    assert np.array_equal(e.field(gpe_mod.PBF_FIELD_PERM), s["perm"])
    assert np.array_equal(e.field(gpe_mod.PBF_FIELD_CELL_START), s["cell_start"])
    assert np.array_equal(e.field(gpe_mod.PBF_FIELD_POS).view(np.uint32), s["x"].view(np.uint32))
    d = (s["xs"] - s["x"]).astype(np.float32)
    assert np.array_equal(e.field(gpe_mod.PBF_FIELD_DISP).view(np.uint32), d.view(np.uint32))
    e.close()


# ----- PBF, 256 batched scenes -------------------------------------------------------------------------
def test_pbf_256_batched_scenes_match_oracle_and_solo_runs(gpe_mod, oracle, cuda_ok):
    from gpe import scenes

    p, pos, vel, dom, boxes = scenes.batched_workload(iters=4)
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_tuning(cell=0.0, block=128, persistent=0, skin=0.075)
    e.set_state(pos, vel, dom)
    e.step(1)
    x, v, d = e.get_state()
    r = oracle.PbfOracle(p, boxes).step(pos, vel, dom, n_steps=1)
    assert np.array_equal(d, r["dom"])
    # from rest, the velocity after one step is the small residual of gravity and the pressure corrections; the
    # FP32 rounding of those neighbour sums shows at up to 1.8e-5 of it (measured; 3e-6 m/s)
    _pbf_step_close(p, x, v, r, rel_v=2e-5)
    e.step(2)
    xb, vb, db = e.get_state()
    assert e.status() == 0
    e.close()
    for q, box in enumerate(boxes):
        m = dom == q
        solo = gpe_mod.Pbf(p, [box], capacity=int(m.sum()))
        solo.set_tuning(cell=0.0, block=128, persistent=0, skin=0.075)
        solo.set_state(pos[m], vel[m])
        solo.step(3)
        xs, vs, _ = solo.get_state()
        solo.close()
        mb = db == q
        assert np.array_equal(xb[mb].view(np.uint32), xs.view(np.uint32)), f"scene {q}: positions differ"
        assert np.array_equal(vb[mb].view(np.uint32), vs.view(np.uint32)), f"scene {q}: velocities differ"


# ----- MLS-MPM ------------------------------------------------------------------------------------------
def _mpm_step_close(x1, v1, C1, F1, J1, want, dx, f_sel=None, j_sel=None):
    wx, wv, wC, wF, wJ = want
    _close(x1, wx, 1e-5 * np.abs(wx) + 8 * EPS32 * np.abs(wx).max(), "x")
    _close(v1, wv, 1e-5 * np.abs(wv).max(), "v")
    # C is a velocity gradient: its scale is the velocity over the node spacing (where the exact gradient
    # vanishes, as in a uniform flow, the FP32 node velocities still leave rounding at that scale)
    _close(C1, wC, 1e-5 * max(np.abs(wC).max(), np.abs(wv).max() / dx), "C")
    fs = slice(None) if f_sel is None else f_sel
    _close(F1[fs], wF[fs], 1e-5 * np.abs(wF[fs]).max(), "F")
    if j_sel is not None:
        _close(J1[j_sel], wJ[j_sel], 1e-5 * np.abs(wJ[j_sel]).max(), "J")


def _grid_close(g, want):
    _close(g[:, 2], want[:, 2], 1e-5 * np.abs(want[:, 2]).max(), "node mass")
    _close(g[:, :2], want[:, :2], 1e-5 * np.abs(want[:, :2]).max(), "node momentum")


def test_mpm_65k_elastic_32_per_cell(gpe_mod, oracle, cuda_ok):
    from gpe import scenes

    p, pos, vel = scenes.elastic_workload()
    n = len(pos)
    C0 = np.zeros((n, 4), np.float32)
    F0 = np.tile(np.eye(2, dtype=np.float32).ravel(), (n, 1))
    J0 = np.ones(n, np.float32)
    o = oracle.MpmOracle(p)
    # P2G of the cell-sorted particles: lanes of a warp share a base node in runs of up to 32
    e = gpe_mod.Mpm(p, capacity=n)
    e.set_state(pos, vel)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    e.stage(gpe_mod.MPM_STAGE_SORT)
    e.p2g_wide_warps()  # clears the counter
    e.stage(gpe_mod.MPM_STAGE_P2G)
    wide = e.p2g_wide_warps()
    _grid_close(e.grid(), o.p2g(pos, vel, C0, F0, J0))
    # the warps with a run longer than 16 lanes, counted on the host from the sorted base nodes: the device
    # took the 5-round reduction in exactly those. A warp holds 64 particles, two per lane; a lane's run key
    # is the base node of its second particle
    # (the device's stencil: g = fma(x, 1/dx, offset) in FP32, base = floor(g - 0.5); the product of two
    # floats is exact in double, so one rounding to float32 reproduces the fma)
    inv_dx = np.float32(1.0) / np.float32(p.dx)
    g = (pos.astype(np.float64) * np.float64(inv_dx) + np.float64(np.float32(p.grid_offset))).astype(np.float32)
    base = np.floor(g - np.float32(0.5)).astype(np.int64)
    key = np.sort(base[:, 1] * p.nx + base[:, 0], kind="stable")
    want_wide = 0
    for w in range(0, n, 64):
        k = key[w + 1:w + 64:2]
        runs = np.diff(np.flatnonzero(np.concatenate([[True], k[1:] != k[:-1], [True]])))
        want_wide += int(runs.max() > 16)
    assert want_wide > 100
    assert wide == want_wide, f"{wide} warps took the 5-round reduction, {want_wide} expected"
    e.close()
    # one full step (the engine sorts on its first step and returns the particles in the caller's order)
    e = gpe_mod.Mpm(p, capacity=n)
    e.set_state(pos, vel)
    e.step(1)
    got = e.get_state()
    assert e.status() == 0
    e.close()
    _mpm_step_close(*got, o.step(pos, vel, C0, F0, J0, None, 1), p.dx)


def test_mpm_4m_mixed_materials(gpe_mod, oracle, cuda_ok):
    from gpe import scenes

    n = 4194304
    p = scenes.mixed_params(n)
    pos, mat = scenes.mixed_discs(n)
    vel = np.zeros_like(pos)
    C0 = np.zeros((n, 4), np.float32)
    F0 = np.tile(np.eye(2, dtype=np.float32).ravel(), (n, 1))
    J0 = np.ones(n, np.float32)
    o = oracle.MpmOracle(p)
    e = gpe_mod.Mpm(p, capacity=n)
    e.set_state(pos, vel, material=mat)
    e.stage(gpe_mod.MPM_STAGE_CLEAR)
    e.stage(gpe_mod.MPM_STAGE_SORT)
    e.stage(gpe_mod.MPM_STAGE_P2G)
    _grid_close(e.grid(), o.p2g(pos, vel, C0, F0, J0, mat))
    e.close()
    e = gpe_mod.Mpm(p, capacity=n)
    e.set_state(pos, vel, material=mat)
    e.step(1)
    got = e.get_state()
    assert e.status() == 0
    e.close()
    keep_f = mat != gpe_mod.MPM_MAT_FLUID  # the engine keeps no F for fluid particles
    keep_j = mat != gpe_mod.MPM_MAT_COROTATED  # jelly keeps no J (its volume is det F)
    _mpm_step_close(*got, o.step(pos, vel, C0, F0, J0, mat, 1), p.dx, f_sel=keep_f, j_sel=keep_j)
