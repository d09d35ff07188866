"""Candidate masks (gpe_pbf_tuning.skin): the first lambda pass of a step records, per particle, which
candidates of its 3 x 3 cells lie within h + skin; the later passes of the step visit only those, and a
particle whose neighbourhood has moved too far (or that left its sort cell) scans in full. Terms of pairs
beyond h are exact zeros, so the state after any number of steps equals the full scans' bit for bit: in
calm and violent scenes (the violent ones mark most neighbourhoods as moved), crowded ones (rows of more
candidates than a mask word holds), one scene or many, with and
without vorticity, the reference's pair-direction flags, the persistent solve, and the network warm start
(whose memory-start step runs more iterations than the masks' move threshold allows for).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(kind):
    from gpe import scenes

    if kind in ("calm", "violent"):
        p = scenes.dam_params(iters=3)
        p.dt = 1.0 / 480.0 if kind == "calm" else 1.0 / 240.0
        pos, vel, boxes = scenes.dam_break(n_side=64)
        sd = 0.2 if kind == "calm" else 2.0
        vel = np.random.default_rng(3).normal(0, sd, pos.shape).astype(np.float32)
        return p, pos, vel, None, boxes
    if kind == "crowded":
        # a block at 0.3 h spacing (about 11 particles a cell) beside one at the rest spacing 0.5 h: many of
        # the dense block's 3-cell rows hold more than 31 candidates, more than a mask word, so those
        # particles scan in full while the others use their masks
        p = scenes.dam_params(iters=3)
        p.dt = 1.0 / 480.0
        dense, _, boxes = scenes.dam_break(n_side=48, spacing=0.006)
        rest, _, _ = scenes.dam_break(n_side=48, seed=1)
        pos = np.concatenate([dense, rest + np.float32(0.6)]).astype(np.float32)
        vel = np.random.default_rng(5).normal(0, 0.2, pos.shape).astype(np.float32)
        return p, pos, vel, None, boxes
    if kind == "batched":
        p = scenes.dam_params(iters=2)
        p.dt = 1.0 / 480.0
        pos, vel, dom, boxes = scenes.batched_scenes(n_scenes=7, seed=5, lo=300, hi=3000)
        vel = np.random.default_rng(4).normal(0, 0.5, pos.shape).astype(np.float32)
        return p, pos, vel, dom, boxes
    p = scenes.reference_pbf_params(iters=4)  # SELF_GRAD | PAIR_IDS | VEL_CLAMP, the reference's block
    pos, vel, boxes = scenes.reference_pbf_block()
    return p, pos, vel, None, boxes


def _run(gpe_mod, p, pos, vel, dom, boxes, skin, steps=6, persistent=False, vort=0.0, iters=None, block=256):
    p = p.copy()
    p.vort_eps = vort
    if iters is not None:
        p.iters = iters
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_tuning(block=block, persistent=persistent, skin=skin)
    e.set_state(pos, vel, dom)
    e.step(steps)
    x, v, d = e.get_state()
    assert e.status() == 0
    return x, v, d


@pytest.mark.parametrize("kind", ["calm", "violent", "batched", "reference", "crowded"])
@pytest.mark.parametrize("vort", [0.0, 5e-4])
def test_masked_steps_equal_full_scans(gpe_mod, cuda_ok, kind, vort):
    p, pos, vel, dom, boxes = _scene(kind)
    ref = _run(gpe_mod, p, pos, vel, dom, boxes, skin=0.0, vort=vort)
    for skin in (0.05, 0.1, 1.0):
        got = _run(gpe_mod, p, pos, vel, dom, boxes, skin=skin, vort=vort)
        for a, b in zip(ref, got):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("kind", ["calm", "violent", "batched", "crowded"])
@pytest.mark.parametrize("iters", [1, 2, 5])
def test_masked_persistent_solve_equals_full_scans(gpe_mod, cuda_ok, kind, iters):
    p, pos, vel, dom, boxes = _scene(kind)
    ref = _run(gpe_mod, p, pos, vel, dom, boxes, skin=0.0, iters=iters)
    got = _run(gpe_mod, p, pos, vel, dom, boxes, skin=0.1, iters=iters, persistent=True, block=512)
    for a, b in zip(ref, got):
        np.testing.assert_array_equal(a, b)


def test_masked_network_warm_start_equals_full_scans(gpe_mod, cuda_ok):
    """The network step (lambda from the network, masks made by the second lambda pass) and the step that
    starts its memory (20 iterations: the masks are rebuilt whenever the move threshold's pass count is
    used up) equal the full scans."""
    p, pos, vel, dom, boxes = _scene("calm")
    p = p.copy()
    p.iters = 2
    net = gpe_mod.Mlp(max_pairs=16 * len(pos), seed=7)
    c = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    c.set_state(pos, vel)
    net.collect(c, n_steps=9, stride=1, seed=3)
    net.train(gpe_mod.make_train_params(epochs=3, batch=2048, lr=3e-3, val_fraction=0.1, seed=5))
    outs = []
    for skin in (0.0, 0.1):
        e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
        e.set_tuning(skin=skin)
        e.set_state(pos, vel)
        e.set_warm_start(gpe_mod.WARM_MLP, net)
        e.step(4)
        assert e.status() == 0
        outs.append(e.get_state())
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def test_stage_by_stage_with_extra_passes_equals_full_scans(gpe_mod, cuda_ok):
    """The stage API may run more delta p passes than the engine's iteration count: the masks stop at the
    count the move threshold allows for, and a written position drops them."""
    p, pos, vel, dom, boxes = _scene("violent")
    p = p.copy()
    p.iters = 2
    outs = []
    for skin in (0.0, 0.1):
        e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
        e.set_tuning(skin=skin)
        e.set_state(pos, vel)
        e.stage(gpe_mod.PBF_STAGE_PREDICT_SORT)
        for _ in range(5):
            e.stage(gpe_mod.PBF_STAGE_LAMBDA)
            e.stage(gpe_mod.PBF_STAGE_DELTA_P)
        xs = e.field(gpe_mod.PBF_FIELD_PRED)
        xs[:, 0] += np.float32(0.3 * p.h)  # every particle moves by 0.3 h: masks made before are stale
        e.set_field(gpe_mod.PBF_FIELD_PRED, xs)
        e.stage(gpe_mod.PBF_STAGE_LAMBDA)
        e.stage(gpe_mod.PBF_STAGE_DELTA_P)
        e.stage(gpe_mod.PBF_STAGE_XSPH)
        e.stage(gpe_mod.PBF_STAGE_FINISH)
        outs.append(e.get_state())
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def test_skin_is_a_tuning_value(gpe_mod, cuda_ok):
    p, pos, vel, dom, boxes = _scene("calm")
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    assert abs(e.tuning().skin - 0.075) < 1e-7  # on by default
    e.set_tuning(skin=0.25)
    assert abs(e.tuning().skin - 0.25) < 1e-7
    with pytest.raises(gpe_mod.GpeError):
        e.set_tuning(skin=-0.1)
    with pytest.raises(gpe_mod.GpeError):
        e.set_tuning(skin=1.5)
