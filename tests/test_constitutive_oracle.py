"""Known-answer tests (CPU only) of the oracle's constitutive library beyond the reference's J-EOS fluid:
the compressible Neo-Hookean model (tau = mu (F F^T - I) + la ln J I) and Drucker-Prager sand (Klar et al.
2016: Hencky-strain St. Venant-Kirchhoff stress, return mapping of the log singular values onto the
friction cone, J = 1 + q with q the accumulated plastic strain).

P2G of one particle at rest (v = 0, C = 0) puts exactly the stress term on the grid, which is compared to a
numpy evaluation of the closed-form stress; G2P on a zero grid leaves F as it is before the plasticity step,
so the sand projection is seen alone.
"""
import math

import numpy as np
import pytest


def _params(material, E=1e3, nu=0.3):
    import gpe
    from gpe import scenes

    p = scenes.elastic_params(4096, 32)
    p.material = material
    p.E, p.nu = E, nu
    p.gravity[1] = 0.0
    return p


def _lame(p):
    mu = p.E / (2 * (1 + p.nu))
    la = p.E * p.nu / ((1 + p.nu) * (1 - 2 * p.nu))
    return mu, la


def _one(F, J=1.0, pos=(0.5, 0.5)):
    x = np.array([pos], np.float32)
    v = np.zeros((1, 2), np.float32)
    C = np.zeros((1, 4), np.float32)
    Fa = np.array([F], np.float32).reshape(1, 4)
    Ja = np.array([J], np.float32)
    return x, v, C, Fa, Ja


def _p2g_stress_term(p, x, tau):
    """Grid momentum of one particle at rest: w_ab * coeff * (tau . dp_ab), coeff = -dt vol0 4/dx^2."""
    g = np.zeros((p.nx * p.ny, 2))
    gx = x[0] / p.dx + p.grid_offset
    gy = x[1] / p.dx + p.grid_offset
    bx, by = math.floor(gx - 0.5), math.floor(gy - 0.5)
    fx, fy = gx - bx, gy - by
    w = lambda f: [0.5 * (1.5 - f) ** 2, 0.75 - (f - 1) ** 2, 0.5 * (f - 0.5) ** 2]
    wx, wy = w(fx), w(fy)
    coeff = -p.dt * p.vol0 * 4 / p.dx ** 2
    for a in range(3):
        for b in range(3):
            dp = np.array([(a - fx) * p.dx, (b - fy) * p.dx])
            g[(by + b) * p.nx + bx + a] = wx[a] * wy[b] * coeff * (tau @ dp)
    return g


@pytest.mark.parametrize("mat", ["neohookean", "sand"])
def test_stress_vanishes_at_rest(gpe_mod, oracle, mat):
    p = _params(getattr(gpe_mod, f"MPM_MAT_{mat.upper()}"))
    g = oracle.MpmOracle(p).p2g(*_one(np.eye(2).ravel()))
    assert np.abs(g[:, :2]).max() == 0.0
    assert g[:, 2].sum() == pytest.approx(p.mass, rel=1e-12)


@pytest.mark.parametrize("s", [0.9, 1.1])
def test_neohookean_uniform_stretch(gpe_mod, oracle, s):
    p = _params(gpe_mod.MPM_MAT_NEOHOOKEAN)
    mu, la = _lame(p)
    F = np.float32(s) * np.eye(2, dtype=np.float32)
    sf = float(np.float32(s))
    tau = (mu * (sf * sf - 1) + la * math.log(sf * sf)) * np.eye(2)
    x, v, C, Fa, Ja = _one(F.ravel())
    g = oracle.MpmOracle(p).p2g(x, v, C, Fa, Ja)
    want = _p2g_stress_term(p, x[0].astype(np.float64), tau)
    np.testing.assert_allclose(g[:, :2], want, rtol=1e-9, atol=1e-12 * np.abs(want).max())


def test_neohookean_shear_is_symmetric(gpe_mod, oracle):
    p = _params(gpe_mod.MPM_MAT_NEOHOOKEAN)
    mu, la = _lame(p)
    F = np.array([1.0, 0.2, 0.0, 1.0], np.float32)  # simple shear, det F = 1
    Fm = F.astype(np.float64).reshape(2, 2)
    tau = mu * (Fm @ Fm.T - np.eye(2))  # ln J = 0
    x, v, C, Fa, Ja = _one(F)
    g = oracle.MpmOracle(p).p2g(x, v, C, Fa, Ja)
    want = _p2g_stress_term(p, x[0].astype(np.float64), tau)
    np.testing.assert_allclose(g[:, :2], want, rtol=1e-9, atol=1e-12 * np.abs(want).max())


def _sand_g2p(gpe_mod, oracle, F, J=1.0):
    p = _params(gpe_mod.MPM_MAT_SAND)
    grid = np.zeros((p.nx * p.ny, 3))
    x, v, C, Fa, Ja = _one(F, J)
    _, _, _, F1, J1 = oracle.MpmOracle(p).g2p(grid, x, v, C, Fa, Ja)
    return p, F1[0].astype(np.float64).reshape(2, 2), float(J1[0])


def _alpha(q):
    phi = 35 + (9 * q - 10) * math.exp(-0.2 * q)  # the default hardening (Klar et al. 2016)
    sp = math.sin(math.radians(phi))
    return math.sqrt(2 / 3) * 2 * sp / (3 - sp)


def test_sand_expansion_goes_to_the_cone_tip(gpe_mod, oracle):
    F = np.diag([1.1, 1.05]).astype(np.float32).ravel()
    _, F1, J1 = _sand_g2p(gpe_mod, oracle, F)
    np.testing.assert_allclose(np.linalg.svd(F1, compute_uv=False), [1, 1], atol=1e-6)
    e = np.log(np.float32([1.1, 1.05]).astype(np.float64))
    assert J1 - 1 == pytest.approx(np.linalg.norm(e), rel=1e-6)


def test_sand_inside_the_cone_is_elastic(gpe_mod, oracle):
    F = np.diag([0.96, 0.95]).astype(np.float32).ravel()  # nearly isotropic compression
    _, F1, J1 = _sand_g2p(gpe_mod, oracle, F, J=1.2)
    np.testing.assert_array_equal(F1.ravel().astype(np.float32), F)
    assert J1 == np.float32(1.2)


@pytest.mark.parametrize("J0", [1.0, 1.5])
def test_sand_shear_returns_onto_the_yield_surface(gpe_mod, oracle, J0):
    F = np.array([[1.2, 0.1], [0.0, 0.7]], np.float32)
    p, F1, J1 = _sand_g2p(gpe_mod, oracle, F.ravel(), J=J0)
    mu, la = _lame(p)
    cf = (2 * la + 2 * mu) / (2 * mu)
    sg0 = np.linalg.svd(F.astype(np.float64), compute_uv=False)
    e0 = np.log(sg0)
    sg1 = np.linalg.svd(F1, compute_uv=False)
    e1 = np.log(sg1)
    a = _alpha(J0 - 1)
    # the trace is kept, the deviator shrinks onto |dev| + cf tr alpha = 0
    assert e1.sum() == pytest.approx(e0.sum(), abs=1e-6)
    dev1 = e1 - e1.mean()
    assert np.linalg.norm(dev1) + cf * e1.sum() * a == pytest.approx(0.0, abs=1e-6)
    dev0 = e0 - e0.mean()
    assert J1 - J0 == pytest.approx(np.linalg.norm(dev0) - np.linalg.norm(dev1), abs=1e-6)
    # singular directions are kept
    U0, _, V0 = np.linalg.svd(F.astype(np.float64))
    U1, _, V1 = np.linalg.svd(F1)
    assert abs(abs(np.dot(U0[:, 0], U1[:, 0])) - 1) < 1e-6
