"""Pins the oracle to the reference without a GPU: the fixtures in tests/golden were produced by running the
reference's own kernels (tests/golden/make_golden.py); the oracle must reproduce them on the same inputs.

PBF tolerances as in test_reference_parity.py (the reference works in chunk-local coordinates); MPM to 1e-5
of each field's scale (1e-4 for C), the reference's P2G summing with float atomics in no fixed order.
"""
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
EPS32 = np.finfo(np.float32).eps


def _load(name):
    f = GOLD / name
    if not f.exists():
        pytest.fail(f"missing golden fixture {f}; generate it with tests/golden/make_golden.py on a GPU")
    return dict(np.load(f))


def _assert_close(a, b, atol, what):
    err = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    bad = err > atol
    assert not bad.any(), f"{what}: {bad.sum()} beyond tolerance, max err {err.max():.3e}"


def test_oracle_reproduces_reference_pbf_substep(gpe_mod, oracle):
    from gpe import scenes

    g = _load("pbf_reference_substep.npz")
    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_pbf_block()
    assert np.array_equal(pos, g["x"]) and np.array_equal(vel, g["v"]), "fixture inputs changed"
    o = oracle.PbfOracle(p, boxes)
    r = o.step(pos, vel, None, 1, pair_id=g["slot"])
    perm = o.predict_sort(pos, vel)["perm"]
    ox, ov, ol = np.empty_like(pos), np.empty_like(pos), np.empty(len(pos), np.float32)
    ox[perm], ov[perm], ol[perm] = r["x"], r["v"], r["lam"]
    xs0 = (pos + vel).astype(np.float64)
    xs0[:, 1] += p.gravity[1]
    corr = np.abs(g["out_x"] - xs0).max()
    ulp = 8 * EPS32 * np.abs(g["out_x"]).astype(np.float64)
    _assert_close(ox, g["out_x"], 1e-4 * corr + ulp, "x*")
    _assert_close(ov, g["out_v"], 1e-4 * np.abs(g["out_v"]).max() + 2 * ulp, "v")
    _assert_close(ol, g["out_lambda"], 1e-4 * np.abs(g["out_lambda"]).max(), "lambda")


def test_oracle_reproduces_reference_mpm_substep(gpe_mod, oracle):
    from gpe import scenes

    g = _load("mpm_reference_substep.npz")
    p = scenes.reference_mpm_params()
    out = oracle.MpmOracle(p).step(g["x"], g["v"], g["C"], g["F"], g["J"], None, 1)
    for nm, a in zip(["x", "v", "C", "F", "J"], out):
        b = g["out_" + nm].astype(np.float64)
        tol = 1e-5 * np.abs(b).max() + (8 * EPS32 * np.abs(b) if nm == "x" else 0.0)
        if nm == "C":
            tol = 1e-4 * np.abs(b).max()
        _assert_close(a, b, tol, f"MPM {nm}")


def test_oracle_reproduces_reference_migration_and_sort(gpe_mod, oracle):
    """A complete reference substep, migration and the per-chunk cell sort included, on the border band:
    258 atoms queue for one chunk (of its 320 slots). After the oracle's step and the next predict + sort,
    every cell holds as many atoms as in the reference and the same atoms (x and the next prediction x*)."""
    from gpe import scenes
    from refcompare import compare_with_reference_sort

    g = _load("pbf_reference_migration.npz")
    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_border_band()
    assert np.array_equal(pos, g["x"]) and np.array_equal(vel, g["v"]), "fixture inputs changed"
    mig = g["mig_count"]
    assert 240 <= mig.max() < 320, f"the fullest migration queue holds {mig.max()} atoms"
    assert int(mig.sum()) > 250
    o = oracle.PbfOracle(p, boxes)
    r = o.step(pos, vel, None, 1, pair_id=g["slot"])
    s = o.predict_sort(r["x"], r["v"])
    compare_with_reference_sort(g["out_cell"], g["out_x"], g["out_xs"], s["key"], s["x"], s["xs"])


def test_oracle_reproduces_reference_render_frame(oracle):
    """The reference's own backgroundKernel and drawKernel drew this view (every pixel by one thread, up to six
    stacked splats blended in order, splats over the chunk lines, clipping at the image edge): the oracle's
    sequential restatement gives the same image byte for byte."""
    from gpe import scenes

    g = _load("render_reference_frame.npz")
    pos, counts = scenes.reference_render_view()
    assert np.array_equal(pos, g["pos"]) and np.array_equal(counts, g["counts"]), "fixture inputs changed"
    w, h = int(g["width"]), int(g["height"])
    img = oracle.render_frame(w, h, 5.0, 32.0, pos, counts)
    diff = np.argwhere(img != g["image"])
    assert len(diff) == 0, (len(diff), diff[:5])

