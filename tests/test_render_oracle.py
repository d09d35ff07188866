"""The oracle's restatement of the reference's splat rasteriser, checked by hand on the CPU.

One splat at a known pixel: its 21 footprint pixels get exactly one application of the reference's alpha()
blend (FP32, in its operation order), every other pixel keeps the background; a second coincident splat
applies the blend a second time.
"""
import numpy as np

F = np.float32


def _blend(over, under):
    a = F(100) * (F(1) / F(255))
    ia = F(1) - a
    return np.uint8(F(F(F(over) * a) + F(F(under) * ia)) + F(0.5))


def _background(x, y, w, h, every):
    if x % every == 0 or y % every == 0:
        return (0, 0, 0)
    t = F(100) * (F(y) / F(h))
    return (np.uint8(255 - np.uint8(t)), np.uint8(160 - np.uint8(t)), 80)


def test_single_and_double_splat(oracle):
    W, H, scale, dim = 64, 48, 2.0, 10.0
    every = int(dim * scale)
    pos = np.zeros((1, 4, 2), np.float32)
    pos[0, 0] = (13.3, 9.7)  # pixel (26, 19)
    pos[0, 1] = (13.3, 9.7)
    for n in (1, 2):
        img = oracle.render_frame(W, H, scale, dim, pos, np.array([n], np.int32))
        for y in range(H):
            for x in range(W):
                bg = _background(x, y, W, H, every)
                dx, dy = x - 26, y - 19
                inside = abs(dx) <= 2 and abs(dy) <= 2 and not (abs(dx) == 2 and abs(dy) == 2)
                want = list(bg)
                if inside:
                    for _ in range(n):
                        want = [_blend(o, u) for o, u in zip((140, 210, 255), want)]
                assert tuple(img[y, x, :3]) == tuple(int(c) for c in want), (x, y, n)
                assert img[y, x, 3] == 255


def test_atoms_outside_the_image_and_beyond_capacity_are_skipped(oracle):
    W, H = 32, 32
    pos = np.array([[[-0.3, 5.0], [5.0, 99.0], [5.0, 5.0]]], np.float32)  # (-0.3 * 2) truncates to pixel 0
    img = oracle.render_frame(W, H, 2.0, 100.0, pos, np.array([2], np.int32))  # the third atom is beyond n
    assert (img[10, 0, :3] != np.array(_background(0, 10, W, H, 200))).any()  # x = -0.6 -> pixel 0
    assert (img[10, 10, :3] == np.array(_background(10, 10, W, H, 200))).all()
