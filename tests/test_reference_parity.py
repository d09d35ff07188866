"""Parity with the reference's own kernels (PBF.cu, MPM.cu built unmodified for sm_103a, run through the
driver API by oracle/refrun.py) on the same inputs.

PBF: one substep stopped after XSPHKernel, so no atomic-order sort intervenes; the engine and the oracle seed
the self pair's pseudo-random gradient direction with the reference's chunk slots (GPE_PBF_PAIR_IDS), so
every term matches. The reference works in chunk-local coordinates, the engine in scene coordinates, so
positions differ by the rounding of that change of frame (a few ulp of the scene coordinate). A complete
substep — migration across chunk borders and the reference's per-chunk cell sort — is compared cell by cell
(tests/refcompare.py): the reference's order within a cell follows shared-memory atomics. The splat renderer
is compared with the reference's backgroundKernel and drawKernel byte for byte on a view they draw
deterministically.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS32 = np.finfo(np.float32).eps


def _pbf_case():
    from gpe import scenes

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_pbf_block()
    return p, pos, vel, boxes


def _assert_close(a, b, atol, what):
    err = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    bad = err > atol
    assert not bad.any(), f"{what}: {bad.sum()} beyond tolerance, max err {err.max():.3e}"


def _check_pbf(x_in, out_x, out_v, out_lam, ref_x, ref_v, ref_lam, who):
    corr = np.abs(ref_x.astype(np.float64) - x_in).max()  # size of the position update
    ulp = 8 * EPS32 * np.abs(ref_x).astype(np.float64)
    _assert_close(out_x, ref_x, 1e-4 * corr + ulp, f"{who} x*")
    _assert_close(out_v, ref_v, 1e-4 * np.abs(ref_v).max() + 2 * ulp, f"{who} v")
    _assert_close(out_lam, ref_lam, 1e-4 * np.abs(ref_lam).max(), f"{who} lambda")


def _pbf_three_ways(gpe_mod, oracle, p, pos, vel, boxes):
    """One substep stopped after XSPH by the reference's kernels, by the engine stage by stage through the C
    ABI and by the oracle, all seeded with the reference's chunk slots as pair ids. Returns the start x*
    (x + v + g) and (x*, v, lambda) of each in input order."""
    from oracle import refrun

    ref = refrun.RefPBF((12, 6), 320)
    _, slot = ref.seed(pos, vel, float(p.gravity[1]))
    ref.substep(iters=p.iters, full=False)
    rx, rv, rl = ref.read_seeded()
    xs0 = pos + vel
    xs0[:, 1] += p.gravity[1]

    q = p.copy()
    q.flags |= gpe_mod.PBF_PAIR_IDS
    e = gpe_mod.Pbf(q, boxes, capacity=len(pos))
    e.set_state(pos, vel)
    e.set_field(gpe_mod.PBF_FIELD_ID, slot.astype(np.uint32))
    e.stage(gpe_mod.PBF_STAGE_PREDICT_SORT)
    for _ in range(p.iters):
        e.stage(gpe_mod.PBF_STAGE_LAMBDA)
        e.stage(gpe_mod.PBF_STAGE_DELTA_P)
    e.stage(gpe_mod.PBF_STAGE_XSPH)
    perm = e.field(gpe_mod.PBF_FIELD_PERM)
    ex, ev, el = np.empty_like(pos), np.empty_like(pos), np.empty(len(pos), np.float32)
    ex[perm] = e.field(gpe_mod.PBF_FIELD_PRED)
    ev[perm] = e.field(gpe_mod.PBF_FIELD_VEL)
    el[perm] = e.field(gpe_mod.PBF_FIELD_LAMBDA)
    e.close()

    o = oracle.PbfOracle(p, boxes)
    r = o.step(pos, vel, None, 1, pair_id=slot.astype(np.uint32))
    operm = o.predict_sort(pos, vel)["perm"]
    ox, ov, ol = np.empty_like(pos), np.empty_like(pos), np.empty(len(pos), np.float32)
    ox[operm], ov[operm], ol[operm] = r["x"], r["v"], r["lam"]
    return xs0, (ex, ev, el), (ox, ov, ol), (rx, rv, rl)


def test_pbf_substep_engine_and_oracle_match_reference(gpe_mod, oracle, cuda_ok):
    p, pos, vel, boxes = _pbf_case()
    xs0, eng, orc, ref = _pbf_three_ways(gpe_mod, oracle, p, pos, vel, boxes)
    _check_pbf(xs0, *eng, *ref, "engine")
    _check_pbf(xs0, *orc, *ref, "oracle")


def test_pbf_coincident_atoms_within_the_reference_kernels_own_error(gpe_mod, oracle, cuda_ok):
    """Every 40th atom of the block doubled at the same position. The reference gives a coincident pair a
    pseudo-random gradient direction in lambdaKernel (pairDirection) and skips it in posCorrectionKernel, so
    the twins take different multipliers, part by a sliver in the first correction, and the second
    iteration's gradient along that sliver is ill-conditioned in FP32: near the twins an FP32 substep
    departs from the FP64 oracle by more than 1e-5 of the field's scale. The engine's error against the
    oracle (x*, v and lambda) must be within 1e-5 of scale or within the reference kernels' own error on the
    same substep."""
    p, pos, vel, boxes = _pbf_case()
    pos = np.concatenate([pos, pos[::40]]).astype(np.float32)
    vel = np.concatenate([vel, vel[::40]]).astype(np.float32)
    xs0, eng, orc, ref = _pbf_three_ways(gpe_mod, oracle, p, pos, vel, boxes)
    corr = np.abs(orc[0].astype(np.float64) - xs0).max()
    for k, what, scale in ((0, "x*", corr), (1, "v", np.abs(orc[1]).max()), (2, "lambda", np.abs(orc[2]).max())):
        o = orc[k].astype(np.float64)
        e_err = np.abs(eng[k] - o)
        r_err = np.abs(ref[k] - o)
        if k == 0:  # positions: plus a few ulp of the coordinate, the reference's change of frame included
            e_err = np.maximum(e_err - 8 * EPS32 * np.abs(o), 0.0)
            r_err = np.maximum(r_err - 8 * EPS32 * np.abs(o), 0.0)
        bound = max(1e-5 * scale, r_err.max())
        assert e_err.max() <= bound, f"{what}: engine {e_err.max():.3e}, reference {r_err.max():.3e}, scale {scale:.3e}"


def _engine_substep_then_sort(gpe_mod, p, pos, vel, slot, boxes):
    """The engine's step seeded like the reference (pair directions from the reference's chunk slots), then the
    next step's predict + sort: (cell key, x, x*) in sorted order."""
    q = p.copy()
    q.flags |= gpe_mod.PBF_PAIR_IDS
    e = gpe_mod.Pbf(q, boxes, capacity=len(pos))
    e.set_state(pos, vel)
    e.set_field(gpe_mod.PBF_FIELD_ID, np.asarray(slot, np.uint32))
    e.step(1)
    assert e.status() == 0
    e.stage(gpe_mod.PBF_STAGE_PREDICT_SORT)
    out = (e.field(gpe_mod.PBF_FIELD_KEY), e.field(gpe_mod.PBF_FIELD_POS), e.field(gpe_mod.PBF_FIELD_PRED))
    e.close()
    return out


def test_pbf_complete_substep_with_migration_matches_reference(gpe_mod, cuda_ok):
    """A complete reference substep on the border band — migration of 258 atoms into one chunk (of its 320
    queue slots) and the per-chunk cell sort included — against the engine's step and next predict + sort:
    per-cell counts bit for bit and the same atoms in every cell, both against the reference run here and
    against the committed fixture."""
    import torch
    from oracle import refrun
    from refcompare import compare_with_reference_sort

    from gpe import scenes

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_border_band()
    ref = refrun.RefPBF((12, 6), 320)
    _, slot = ref.seed(pos, vel, float(p.gravity[1]))
    ref.substep(iters=p.iters, full=False)
    ref.migrate()
    torch.cuda.synchronize()
    mig = ref.mig_count.cpu().numpy()
    assert 240 <= mig.max() < 320
    ref.prep()
    cell, rx, rxs = ref.read_sorted()
    assert len(cell) == len(pos)
    key, x, xs = _engine_substep_then_sort(gpe_mod, p, pos, vel, slot, boxes)
    compare_with_reference_sort(cell, rx, rxs, key, x, xs)
    from pathlib import Path

    g = dict(np.load(Path(__file__).resolve().parent / "golden" / "pbf_reference_migration.npz"))
    compare_with_reference_sort(g["out_cell"], g["out_x"], g["out_xs"], key, x, xs)


def test_mpm_substep_engine_and_oracle_match_reference(gpe_mod, oracle, cuda_ok):
    from gpe import scenes
    from oracle import refrun

    p = scenes.reference_mpm_params()
    x, v, Cm, F, J = scenes.reference_mpm_block()
    ref = refrun.RefMPM(400 * 1000, (12, 6))
    ref.seed(x, v, Cm, F, J)
    ref.substep(0)
    R = ref.read()
    e = gpe_mod.Mpm(p, capacity=len(x))
    e.set_state(x, v, Cm, F, J)
    e.step(1)
    E = e.get_state()
    O = oracle.MpmOracle(p).step(x, v, Cm, F, J, None, 1)
    names = ["x", "v", "C", "F", "J"]
    for who, got in (("engine", E), ("oracle", O)):
        for nm, a, b in zip(names, got, R):
            b64 = np.asarray(b, np.float64)
            tol = 1e-5 * np.abs(b64).max() + (8 * EPS32 * np.abs(b64) if nm == "x" else 0.0)
            if nm in ("C",):
                tol = 1e-4 * np.abs(b64).max()
            _assert_close(a, b, tol, f"{who} MPM {nm}")


def test_render_engine_matches_reference_kernels(gpe_mod, cuda_ok):
    """gpe_render_frame against the reference's backgroundKernel + drawKernel (cuda-render.cu:214-310), run
    here on a view they draw deterministically (scenes.reference_render_view), and against the committed
    fixture: byte for byte."""
    import torch
    from pathlib import Path

    from gpe import scenes
    from oracle import refrun

    pos, counts = scenes.reference_render_view()
    w, h = 470, 300
    ref = refrun.RefRender().render(pos, counts, w, h)
    g = dict(np.load(Path(__file__).resolve().parent / "golden" / "render_reference_frame.npz"))
    assert np.array_equal(ref, g["image"]), "the reference's kernels drew another image than the fixture's"
    cx, cy, cap = 12, 6, pos.shape[1]
    d_pos = torch.from_numpy(np.ascontiguousarray(pos.reshape(-1, 2))).cuda()
    d_vel = torch.zeros_like(d_pos)
    d_cnt = torch.from_numpy(counts).cuda()
    view = gpe_mod.View(d_pos.data_ptr(), d_vel.data_ptr(), d_cnt.data_ptr(), cx, cy, 32.0, cap)
    pitch = 4 * w + 64
    img = torch.zeros((h, pitch), dtype=torch.uint8, device="cuda")
    cov = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    gpe_mod.render_frame(gpe_mod.Raster(img.data_ptr(), pitch, w, h, 5.0, 32.0, cov.data_ptr()), view)
    torch.cuda.synchronize()
    got = img[:, : 4 * w].cpu().numpy().reshape(h, w, 4)
    diff = np.argwhere(got != ref)
    assert len(diff) == 0, (len(diff), diff[:5])

