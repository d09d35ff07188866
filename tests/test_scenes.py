"""The seeded workload scenes the bench and the parity tests use (CPU only): sizes, containment and the
per-scene layout of the batched MLS-MPM workload."""
import numpy as np


def test_mixed_batch_layout(gpe_mod):
    from gpe import scenes

    p, sc, pos, mat, sid = scenes.mixed_batch(n_scenes=32, seed=6)
    assert len(sc) == 32
    counts = np.bincount(sid, minlength=32)
    assert counts.min() >= 65536 and counts.max() <= 524288
    assert np.all(np.diff(sid) >= 0)  # scene-major
    assert set(np.unique(mat)) == {gpe_mod.MPM_MAT_FLUID, gpe_mod.MPM_MAT_SNOW, gpe_mod.MPM_MAT_COROTATED}
    for q, (nx, ny, lo, hi) in enumerate(sc):
        x = pos[sid == q]
        assert nx == ny and nx % 8 == 0 and nx >= 64
        # inside the particle clamp and clear of the 3-node stencil at the grid edge
        assert x.min() > lo[0] and x[:, 0].max() < hi[0] and x[:, 1].max() < hi[1]
        assert hi[0] < (nx - 2) * p.dx
    # the same particle density as the 4M scene: particles per grid node within 20% of it
    ref = 4194304 / (1024 * 1024)
    dens = counts / np.array([s[0] * s[1] for s in sc])
    assert np.all(np.abs(dens / ref - 1.0) < 0.2)


def test_mixed_batch_is_seeded():
    from gpe import scenes

    a = scenes.mixed_batch(n_scenes=4, seed=6, lo=2048, hi=8192, total_ref=65536)
    b = scenes.mixed_batch(n_scenes=4, seed=6, lo=2048, hi=8192, total_ref=65536)
    for u, v in zip(a[2:], b[2:]):
        np.testing.assert_array_equal(u, v)
    c = scenes.mixed_batch(n_scenes=4, seed=7, lo=2048, hi=8192, total_ref=65536)
    assert len(c[2]) != len(a[2]) or not np.array_equal(c[2], a[2])


def test_batched_pbf_scenes_are_disjoint():
    from gpe import scenes

    pos, vel, dom, boxes = scenes.batched_scenes(n_scenes=16, seed=3, lo=256, hi=4096)
    assert len(boxes) == 16 and np.all(np.diff(dom) >= 0)
    for q, (x0, y0, w, h) in enumerate(boxes):
        x = pos[dom == q]
        assert x[:, 0].min() >= x0 and x[:, 0].max() <= x0 + w and x[:, 1].min() >= y0 and x[:, 1].max() <= y0 + h
        if q:
            px0, _, pw, _ = boxes[q - 1]
            assert x0 >= px0 + pw  # boxes side by side, no overlap
