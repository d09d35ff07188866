"""Long runs of the small configurations, as the reference's drivers run them (many steps, no re-seeding):

  * PBF dam break, 16,384 particles on a 128 x 128 lattice (h = 0.02, 4 Jacobi iterations, dt = 1/480, the
    step at which the plain 4-iteration solver is stable on this column): 1000 steps stay finite and inside
    the box, two runs are identical bit for bit, and after 200 steps the centre of mass and the mean speed
    agree with the FP64 oracle's run of the same 200 steps;
  * MLS-MPM, 65,536 fixed-corotated particles in two squares on a 128^2 grid (dt = 1e-4, sticky walls,
    re-sorted every 16 steps): 2000 steps stay finite and inside the particle clamp, and after 200 steps the
    centre of mass and the mean speed agree with the oracle's.

Individual particles of two runs that differ in FP32 rounding drift apart over hundreds of steps (the flow
is chaotic), so the comparisons with the oracle are of averages: the centre of mass to 1e-3 of the box, the
mean speed to 2% (stated in each test).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dam():
    from gpe import scenes

    p = scenes.dam_params(iters=4)
    p.dt = 1.0 / 480.0
    pos, vel, boxes = scenes.dam_break(n_side=128)
    return p, pos, vel, boxes


def test_pbf_dam_break_1000_steps_stays_finite_and_deterministic(gpe_mod, cuda_ok):
    p, pos, vel, boxes = _dam()
    (lo_x, lo_y, hi_x, hi_y) = (boxes[0][0], boxes[0][1], boxes[0][0] + boxes[0][2], boxes[0][1] + boxes[0][3])
    runs = []
    for _ in range(2):
        e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
        e.set_state(pos, vel)
        e.step(1000)
        x, v, _ = e.get_state()
        assert e.status() == 0
        e.close()
        runs.append((x, v))
    x, v = runs[0]
    assert np.isfinite(x).all() and np.isfinite(v).all()
    tol = 1e-6 * max(abs(hi_x), abs(hi_y), 1.0)
    assert (x[:, 0] >= lo_x - tol).all() and (x[:, 0] <= hi_x + tol).all()
    assert (x[:, 1] >= lo_y - tol).all() and (x[:, 1] <= hi_y + tol).all()
    # the column has collapsed: particles have spread along the floor beyond the initial block
    assert x[:, 0].max() > pos[:, 0].max() + 0.1 * (hi_x - lo_x)
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


def test_pbf_dam_break_200_steps_averages_track_oracle(gpe_mod, oracle, cuda_ok):
    p, pos, vel, boxes = _dam()
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_state(pos, vel)
    e.step(200)
    x, v, _ = e.get_state()
    assert e.status() == 0
    e.close()
    r = oracle.PbfOracle(p, boxes).step(pos, vel, None, 200)
    side = max(boxes[0][2], boxes[0][3])
    com, com_o = x.astype(np.float64).mean(0), r["x"].astype(np.float64).mean(0)
    assert np.abs(com - com_o).max() <= 1e-3 * side, (com, com_o)
    sp, sp_o = np.linalg.norm(v.astype(np.float64), axis=1).mean(), np.linalg.norm(r["v"].astype(np.float64), axis=1).mean()
    assert abs(sp - sp_o) <= 0.02 * sp_o, (sp, sp_o)


def _elastic(gpe_mod):
    from gpe import scenes

    p, pos, vel = scenes.elastic_workload()
    n = len(pos)
    C0 = np.zeros((n, 4), np.float32)
    F0 = np.tile(np.eye(2, dtype=np.float32).ravel(), (n, 1))
    J0 = np.ones(n, np.float32)
    return p, pos, vel, C0, F0, J0


def test_mpm_elastic_2000_steps_stays_finite(gpe_mod, cuda_ok):
    p, pos, vel, C0, F0, J0 = _elastic(gpe_mod)
    e = gpe_mod.Mpm(p, capacity=len(pos))
    e.set_state(pos, vel)
    e.step(2000)
    x, v, Cm, F, J = e.get_state()
    assert e.status() == 0
    e.close()
    for a in (x, v, Cm, F, J):
        assert np.isfinite(a).all()
    lo = np.asarray(p.clamp_lo, np.float32)
    hi = np.asarray(p.clamp_hi, np.float32)
    assert (x >= lo).all() and (x <= hi).all()
    # the squares have fallen: their centre of mass is lower than at the start
    assert x[:, 1].mean() < pos[:, 1].mean()


def test_mpm_elastic_200_steps_averages_track_oracle(gpe_mod, oracle, cuda_ok):
    p, pos, vel, C0, F0, J0 = _elastic(gpe_mod)
    e = gpe_mod.Mpm(p, capacity=len(pos))
    e.set_state(pos, vel)
    e.step(200)
    x, v, _, _, _ = e.get_state()
    assert e.status() == 0
    e.close()
    xo, vo, _, _, _ = oracle.MpmOracle(p).step(pos, vel, C0, F0, J0, None, 200)
    side = p.nx * p.dx
    com, com_o = x.astype(np.float64).mean(0), xo.astype(np.float64).mean(0)
    assert np.abs(com - com_o).max() <= 1e-3 * side, (com, com_o)
    sp, sp_o = np.linalg.norm(v.astype(np.float64), axis=1).mean(), np.linalg.norm(vo.astype(np.float64), axis=1).mean()
    assert abs(sp - sp_o) <= 0.02 * sp_o, (sp, sp_o)
