"""Tuning of the PBF step (block size, cell size, the persistent single-launch solve) and the autotuner.

A tuning changes how a step runs, not what it computes: for a given cell size every block size and the
persistent solve give the same state bit for bit; a cell size set by tuning equals the same cell size given
at creation, bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(kind):
    from gpe import scenes

    if kind == "dam":
        p = scenes.dam_params(iters=3)
        p.dt = 1.0 / 480.0
        pos, vel, boxes = scenes.dam_break(n_side=64)
        vel = np.random.default_rng(3).normal(0, 0.2, pos.shape).astype(np.float32)
        return p, pos, vel, None, boxes
    p = scenes.dam_params(iters=2)
    p.dt = 1.0 / 480.0
    pos, vel, dom, boxes = scenes.batched_scenes(n_scenes=7, seed=5, lo=300, hi=3000)
    vel = np.random.default_rng(4).normal(0, 0.2, pos.shape).astype(np.float32)
    return p, pos, vel, dom, boxes


def _run(gpe_mod, p, pos, vel, dom, boxes, steps=3, tuning=None, vort=0.0):
    p = p.copy()
    p.vort_eps = vort
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    if tuning is not None:
        e.set_tuning(**tuning)
    e.set_state(pos, vel, dom)
    e.step(steps)
    x, v, d = e.get_state()
    assert e.status() == 0
    return x, v, d


@pytest.mark.parametrize("kind", ["dam", "batched"])
@pytest.mark.parametrize("block", [128, 256, 512])
@pytest.mark.parametrize("vort", [0.0, 5e-4])
def test_persistent_and_block_sizes_are_bit_exact(gpe_mod, cuda_ok, kind, block, vort):
    p, pos, vel, dom, boxes = _scene(kind)
    ref = _run(gpe_mod, p, pos, vel, dom, boxes, vort=vort)
    for persistent in (0, 1, 2):  # per-pass launches, persistent solve, whole step in one launch
        got = _run(gpe_mod, p, pos, vel, dom, boxes, tuning=dict(block=block, persistent=persistent), vort=vort)
        for a, b in zip(ref, got):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("block", [128, 256, 512])
def test_persistent_ticket_path_is_bit_exact(gpe_mod, cuda_ok, block):
    """A scene with more blocks of particles than the persistent grid holds (262,144 particles: 2,048 blocks
    of 128 against at most 12 resident a SM, and so on), so the persistent kernels hand blocks of particles
    out from their ticket counter; the state after three steps equals the per-pass launches' bit for bit."""
    from gpe import scenes

    p = scenes.dam_params(iters=3)
    p.dt = 1.0 / 480.0
    pos, _, boxes = scenes.dam_break(n_side=512, box=10.24)
    vel = np.random.default_rng(6).normal(0, 0.5, pos.shape).astype(np.float32)
    ref = _run(gpe_mod, p, pos, vel, None, boxes, tuning=dict(block=256, persistent=0))
    for persistent in (1, 2):
        got = _run(gpe_mod, p, pos, vel, None, boxes, tuning=dict(block=block, persistent=persistent))
        for a, b in zip(ref, got):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("kind", ["dam", "batched"])
def test_whole_step_launch_keeps_sort_outputs(gpe_mod, cuda_ok, kind):
    """The whole-step kernel sorts inside the launch: after a step, the sort's keys, order and cell starts
    equal those of the separate sort launches, and a plain step (no vorticity) is one launch."""
    p, pos, vel, dom, boxes = _scene(kind)
    out = {}
    for persistent in (1, 2):
        e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
        e.set_tuning(block=256, persistent=persistent)
        e.set_state(pos, vel, dom)
        e.step(2)
        out[persistent] = [e.field(f) for f in (gpe_mod.PBF_FIELD_KEY, gpe_mod.PBF_FIELD_PERM,
                                                     gpe_mod.PBF_FIELD_CELL_START)]
        if persistent == 2:
            assert e.launches_per_step() == 1
        assert e.status() == 0
        e.close()
    for a, b in zip(out[1], out[2]):
        np.testing.assert_array_equal(a, b)


def test_half_cell_tuning_equals_half_cell_creation(gpe_mod, cuda_ok):
    p, pos, vel, dom, boxes = _scene("batched")
    tuned = _run(gpe_mod, p, pos, vel, dom, boxes, tuning=dict(cell=0.5 * p.h, block=256, persistent=False))
    q = p.copy()
    q.cell = 0.5 * p.h
    created = _run(gpe_mod, q, pos, vel, dom, boxes)
    for a, b in zip(tuned, created):
        np.testing.assert_array_equal(a, b)


def test_tuning_rejects_bad_values(gpe_mod, cuda_ok):
    p, pos, vel, dom, boxes = _scene("dam")
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    with pytest.raises(gpe_mod.GpeError):
        e.set_tuning(block=100)
    with pytest.raises(gpe_mod.GpeError):
        e.set_tuning(cell=0.1 * p.h)  # below h/5
    with pytest.raises(gpe_mod.GpeError) as ei:
        e.set_tuning(cell=0.25 * p.h)  # the engine holds cell arrays for h/2 and its own cell size only
    assert ei.value.status == gpe_mod.ERR_CAPACITY


def test_autotune_restores_state_and_caches(gpe_mod, cuda_ok):
    p, pos, vel, dom, boxes = _scene("batched")
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_state(pos, vel, dom)
    before = e.get_state()
    best, ms = e.autotune(trial_steps=3)
    assert best.block in (128, 256, 512) and best.persistent in (0, 1, 2) and ms > 0
    after = e.get_state()
    for a, b in zip(before, after):
        np.testing.assert_array_equal(a, b)
    # the tuned engine steps exactly like a fresh engine given that tuning
    e.step(2)
    got = e.get_state()
    ref = _run(gpe_mod, p, pos, vel, dom, boxes, steps=2,
               tuning=dict(cell=best.cell, block=best.block, persistent=bool(best.persistent), skin=best.skin))
    for a, b in zip(ref, got):
        np.testing.assert_array_equal(a, b)
    # a second engine with the same scenes takes the choice from the cache
    e2 = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e2.set_state(pos, vel, dom)
    best2, ms2 = e2.autotune(trial_steps=3)
    assert ms2 == -1.0 and (best2.cell, best2.block, best2.persistent) == (best.cell, best.block, best.persistent)
