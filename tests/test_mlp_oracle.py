"""The oracle of the warm-start network and of warm-started steps, checked on the CPU.

* The oracle's analytic gradient (plain FP64 mode) against central finite differences of its own loss:
  relative error of each checked component <= 1e-3 of the gradient's largest magnitude.
* The BF16-operand mode stays within a few BF16 ulps of the FP64 mode (it is the same network with its
  tensor-core operands rounded).
* A cold step that keeps the multiplier sums equals the plain step bit for bit, and its sum equals the
  sum of the per-iteration lambdas of a step run with 1..iters iterations.
"""
import numpy as np
import pytest


def _blob(seed=3, scale_out=0.3):
    g = np.random.default_rng(seed)
    b = np.zeros(5083, np.float32)
    b[0:768] = g.uniform(-0.7, 0.7, 768)          # W1
    b[768:832] = g.uniform(-0.1, 0.1, 64)         # b1
    b[832:4928] = g.uniform(-0.3, 0.3, 4096)      # W2
    b[4928:4992] = g.uniform(-0.1, 0.1, 64)       # b2
    b[4992:5056] = g.uniform(-scale_out, scale_out, 64)  # w3
    b[5056] = 0.05
    b[5057:5069] = g.normal(0, 1, 12)             # feature mean
    b[5069:5081] = g.uniform(0.5, 2.0, 12)        # feature std
    b[5081], b[5082] = 0.3, 1.7                   # target mean, std
    return b


def _data(n=48, seed=4):
    g = np.random.default_rng(seed)
    X = g.normal(0, 1.5, (n, 12)).astype(np.float32)
    T = g.normal(0, 2.0, n).astype(np.float32)
    return X, T


def test_oracle_mlp_gradient_matches_finite_differences(oracle):
    blob = _blob()
    X, T = _data()
    g, loss = oracle.mlp_gradient(blob, X, T, bf16=False)
    assert np.isfinite(loss) and loss > 0
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.choice(768, 40, False), 768 + rng.choice(64, 10, False),
                          832 + rng.choice(4096, 60, False), 4928 + rng.choice(64, 10, False),
                          4992 + rng.choice(64, 10, False), [5056]])
    gmax = np.abs(g).max()
    for p in idx:
        h = 1e-2 * max(abs(float(blob[p])), 1e-2)
        bp, bm = blob.copy(), blob.copy()
        bp[p] += h
        bm[p] -= h
        hp = float(bp[p]) - float(blob[p])
        hm = float(blob[p]) - float(bm[p])
        lp = oracle.mlp_gradient(bp, X, T, bf16=False)[1]
        lm = oracle.mlp_gradient(bm, X, T, bf16=False)[1]
        fd = (lp - lm) / (hp + hm)
        assert abs(fd - g[p]) <= 1e-3 * gmax + 1e-3 * abs(g[p]), (p, fd, g[p])


def test_oracle_mlp_bf16_mode_is_close_to_fp64(oracle):
    blob = _blob()
    X, _ = _data(n=256)
    a = oracle.mlp_forward(blob, X, bf16=True)
    b = oracle.mlp_forward(blob, X, bf16=False)
    scale = np.abs(b - blob[5081]).max()
    assert np.abs(a - b).max() <= 0.05 * scale
    assert not np.array_equal(a, b)


def test_oracle_collecting_step_equals_plain_step(oracle):
    """A pair-collecting step is the plain step; its memory is the sum of its iterations' lambdas."""
    from gpe import scenes

    p = scenes.dam_params(iters=3)
    pos, vel, boxes = scenes.dam_break(n_side=24)
    vel = np.random.default_rng(5).normal(0, 0.2, pos.shape).astype(np.float32)
    o = oracle.PbfOracle(p, boxes)
    plain = o.step(pos, vel)
    warm = o.step_warm(pos, vel, np.zeros(len(pos), np.float32), mode=0)
    np.testing.assert_array_equal(plain["x"], warm["x"])
    np.testing.assert_array_equal(plain["v"], warm["v"])
    lams = [oracle.PbfOracle(scenes.dam_params(iters=k), boxes).step(pos, vel)["lam"].astype(np.float64)
            for k in (1, 2, 3)]  # the k-th iteration's lambda is the last lambda of a k-iteration step
    np.testing.assert_allclose(warm["acc"], sum(lams), rtol=1e-5, atol=1e-6 * np.abs(sum(lams)).max())


def test_oracle_warm_step_from_zero_equals_plain_step(oracle):
    """With lambda_prev = 0 the warm start moves nothing, and with c_min = 0 the projected update of a zero
    sum is the reference's lambda: a warm-started step of 2 iterations is the plain step of 1, bit for bit."""
    from gpe import scenes

    pos, vel, boxes = scenes.dam_break(n_side=24)
    vel = np.random.default_rng(5).normal(0, 0.2, pos.shape).astype(np.float32)
    plain = oracle.PbfOracle(scenes.dam_params(iters=1), boxes).step(pos, vel)
    warm = oracle.PbfOracle(scenes.dam_params(iters=2), boxes).step_warm(pos, vel, np.zeros(len(pos), np.float32),
                                                                          mode=1)
    np.testing.assert_array_equal(plain["x"], warm["x"])
    np.testing.assert_array_equal(plain["v"], warm["v"])
    np.testing.assert_array_equal(np.minimum(plain["lam"], 0), warm["acc"])


def test_oracle_warm_sums_stay_pushing_and_relax(oracle):
    """Summed multipliers never turn positive, and the sum of a particle below rest density is relaxed by
    the next iteration instead of being kept (no ratchet)."""
    from gpe import scenes

    p = scenes.dam_params(iters=6)
    pos, vel, boxes = scenes.dam_break(n_side=24)
    o = oracle.PbfOracle(p, boxes)
    out = o.step_warm(pos, vel, np.zeros(len(pos), np.float32), mode=1, n_steps=3)
    assert np.all(out["acc"] <= 0) and np.all(np.isfinite(out["acc"])) and out["acc"].min() < 0
    # one particle alone in the box: density far below rest, so its sum returns to 0 in one iteration
    p2 = scenes.dam_params(iters=2)
    p2.gravity[1] = 0.0
    lone = oracle.PbfOracle(p2, boxes).step_warm(np.float32([[1.0, 1.0]]), np.zeros((1, 2), np.float32),
                                                  np.float32([-1e-6]), mode=1)
    assert lone["acc"][0] == 0.0
