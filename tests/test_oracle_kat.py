"""Known-answer tests of the oracle (CPU only): kernel normalisation, sort invariants, conservation laws of
the PBF position and XSPH updates, B-spline partition of unity and P2G conservation."""
import math

import numpy as np
import pytest

from conftest import ROOT  # noqa: F401


def _params(gpe_mod, **kw):
    from gpe import scenes

    p = scenes.dam_params()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_kernel_normalisation():
    # 2D poly6 4/(pi h^8)(h^2-r^2)^3 and the spiky profile 10/(pi h^5)(h-r)^3 integrate to 1 over the disc;
    # the spiky gradient coefficient 30/(pi h^5) is its derivative (the reference's kCoeffPoly6 / kCoeffSpiky
    # at h = 2, constants.h:38-39)
    h = 0.37
    r = np.linspace(0, h, 200001)
    poly6 = 4 / (math.pi * h ** 8) * (h * h - r * r) ** 3
    spiky = 10 / (math.pi * h ** 5) * (h - r) ** 3
    assert abs(np.trapezoid(poly6 * 2 * math.pi * r, r) - 1) < 1e-6
    assert abs(np.trapezoid(spiky * 2 * math.pi * r, r) - 1) < 1e-6
    assert abs(4 / (math.pi * 2.0 ** 8) - 1 / (64 * math.pi)) < 1e-12
    assert abs(30 / (math.pi * 2.0 ** 5) - 30 / (32 * math.pi)) < 1e-12


def test_isolated_density(gpe_mod, oracle):
    p = _params(gpe_mod)
    o = oracle.PbfOracle(p, [(0, 0, 1, 1)])
    x = np.array([[0.3, 0.3], [0.3 + 0.01, 0.3], [0.8, 0.8]], np.float32)
    s = o.predict_sort(x, np.zeros_like(x))
    rho = o.density(s["xs"], s["dom"], s["cell_start"])
    c6 = 4 / (math.pi * p.h ** 8)
    h2 = np.float32(p.h) ** 2
    r2 = float(np.float32(0.3 + 0.01) - np.float32(0.3)) ** 2
    # particle order after the sort is by cell; match by position
    xs = s["xs"]
    for i in range(3):
        if xs[i, 0] > 0.7:
            assert rho[i] == pytest.approx(p.mass * c6 * h2 ** 3, rel=1e-6)
        else:
            assert rho[i] == pytest.approx(p.mass * c6 * (h2 ** 3 + (h2 - r2) ** 3), rel=1e-5)


def test_sort_invariants(gpe_mod, oracle):
    rng = np.random.default_rng(5)
    p = _params(gpe_mod)
    boxes = [(0, 0, 0.5, 0.3), (1, 0, 0.2, 0.4), (2, 1, 0.3, 0.3)]
    xs, ds = [], []
    for d, (ox, oy, ex, ey) in enumerate(boxes):
        n = 400 + 100 * d
        x = np.stack([rng.uniform(ox - 0.01, ox + ex + 0.01, n), rng.uniform(oy - 0.01, oy + ey + 0.01, n)], 1)
        xs.append(x)
        ds.append(np.full(n, d, np.int32))
    x = np.concatenate(xs).astype(np.float32)
    dom = np.concatenate(ds)
    v = rng.normal(0, 0.3, x.shape).astype(np.float32)
    o = oracle.PbfOracle(p, boxes)
    s = o.predict_sort(x, v, dom)
    key, perm, cs = s["key"], s["perm"], s["cell_start"]
    assert np.all(np.diff(key.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(perm), np.arange(len(x)))
    same = np.diff(key.astype(np.int64)) == 0
    assert np.all(np.diff(perm.astype(np.int64))[same] > 0), "sort must be stable"
    counts = np.bincount(key, minlength=o.num_cells)
    assert cs[0] == 0 and np.array_equal(np.diff(cs.astype(np.int64)), counts)
    # keys stay inside their scene's cell range
    assert np.array_equal(s["dom"], dom[perm])
    # the FP32 prediction is fma(dt, v, x) + dt^2 g
    dt = np.float32(p.dt)
    g2 = np.float32(dt * dt) * np.float32(p.gravity[1])
    pred_y = (np.float64(dt) * v[:, 1].astype(np.float64) + x[:, 1]).astype(np.float32) + g2
    assert np.array_equal(s["xs"][:, 1], pred_y[perm])


def _lattice(n_side, spacing, origin, jitter, seed):
    g = np.random.default_rng(seed)
    ix, iy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy")
    x = np.stack([origin + ix.ravel() * spacing, origin + iy.ravel() * spacing], 1)
    return (x + g.uniform(-jitter, jitter, x.shape)).astype(np.float32)


def test_delta_p_and_xsph_conserve_momentum(gpe_mod, oracle):
    p = _params(gpe_mod, omega=1.25, scorr_k=1e-13)
    box = [(0, 0, 2.0, 2.0)]
    x = _lattice(30, 0.008, 0.7, 0.002, 1)  # compressed block away from the walls
    o = oracle.PbfOracle(p, box)
    p0 = p.copy()
    p0.gravity[1] = 0.0
    o0 = oracle.PbfOracle(p0, box)
    s = o0.predict_sort(x, np.zeros_like(x))
    lam, _ = o0.lambda_(s["xs"], s["dom"], s["cell_start"])
    assert np.all(lam <= 0)
    out = o0.delta_p(s["xs"], s["dom"], s["cell_start"], lam)
    dp = out.astype(np.float64) - s["xs"]
    assert np.abs(dp).max() > 1e-5
    assert np.abs(dp.sum(0)).max() < 1e-6 * np.abs(dp).sum()
    # XSPH: sum_i dv_i = 0 (pairwise antisymmetric)
    g = np.random.default_rng(2)
    xs2 = (s["xs"] + g.normal(0, 1e-4, s["xs"].shape)).astype(np.float32)
    v, _ = o.xsph(s["x"], xs2, s["dom"], s["cell_start"])
    v0 = (xs2.astype(np.float64) - s["x"]) / p.dt
    dv = v - v0
    assert np.abs(dv.sum(0)).max() < 1e-4 * np.abs(dv).sum()


def test_bspline_partition_and_p2g_conservation(gpe_mod, oracle):
    from gpe import scenes

    p = scenes.elastic_params(2048, 64)
    rng = np.random.default_rng(3)
    n = 2048
    x = rng.uniform(0.2, 0.8, (n, 2)).astype(np.float32)
    v = rng.normal(0, 1, (n, 2)).astype(np.float32)
    Cm = rng.normal(0, 1, (n, 4)).astype(np.float32)
    F = np.tile(np.array([1, 0, 0, 1], np.float32), (n, 1))
    J = np.ones(n, np.float32)
    o = oracle.MpmOracle(p)
    g = o.p2g(x, v, Cm, F, J)
    assert g[:, 2].sum() == pytest.approx(n * p.mass, rel=1e-9)
    # with F = I the stress is zero and the affine term sums to zero over the stencil
    mom = g[:, :2].sum(0)
    assert np.allclose(mom, p.mass * v.astype(np.float64).sum(0), rtol=1e-7, atol=1e-9)
    # B-spline partition of unity and first moment
    for f in rng.uniform(0.5, 1.5, 50):
        w = np.array([0.5 * (1.5 - f) ** 2, 0.75 - (f - 1) ** 2, 0.5 * (f - 0.5) ** 2])
        assert w.sum() == pytest.approx(1.0, abs=1e-12)
        assert (w * (np.arange(3) - f)).sum() == pytest.approx(0.0, abs=1e-12)


def test_g2p_uniform_field(gpe_mod, oracle):
    from gpe import scenes

    p = scenes.elastic_params(256, 64)
    p.gravity[1] = 0.0
    n = 256
    rng = np.random.default_rng(4)
    x = rng.uniform(0.3, 0.7, (n, 2)).astype(np.float32)
    grid = np.zeros((p.nx * p.ny, 3))
    grid[:, 0], grid[:, 1], grid[:, 2] = 0.25, -0.5, 1.0
    o = oracle.MpmOracle(p)
    x1, v1, C1, F1, J1 = o.g2p(grid, x, np.zeros((n, 2)), np.zeros((n, 4)),
                               np.tile(np.eye(2).ravel(), (n, 1)), np.ones(n))
    assert np.allclose(v1, [0.25, -0.5], atol=1e-6)
    assert np.abs(C1).max() < 1e-4
    assert np.allclose(x1, x + np.float32(p.dt) * np.array([0.25, -0.5], np.float32), atol=1e-6)


def test_snow_plasticity_clamps_singular_values(gpe_mod, oracle):
    from gpe import MPM_MAT_SNOW, scenes

    p = scenes.elastic_params(64, 64)
    p.material = MPM_MAT_SNOW
    p.gravity[1] = 0.0
    n = 64
    rng = np.random.default_rng(6)
    x = rng.uniform(0.4, 0.6, (n, 2)).astype(np.float32)
    grid = np.zeros((p.nx * p.ny, 3))
    # a linear velocity field stretches F strongly in x
    xs = (np.arange(p.nx) * p.dx)[None, :].repeat(p.ny, 0).ravel()
    grid[:, 0] = 2000.0 * (xs - 0.5)
    grid[:, 2] = 1.0
    F0 = np.tile(np.eye(2).ravel(), (n, 1))
    _, _, _, F1, J1 = oracle.MpmOracle(p).g2p(grid, x, np.zeros((n, 2)), np.zeros((n, 4)), F0, np.ones(n))
    for f in F1:
        s = np.linalg.svd(f.reshape(2, 2), compute_uv=False)
        assert s.max() <= 1 + p.theta_s + 1e-5 and s.min() >= 1 - p.theta_c - 1e-5
    # stretch beyond the clamp moves the excess volume change into the plastic J_p
    assert np.all(J1 > 1.0)
