"""Comparison of a sorted PBF state with the reference's state after a complete substep (migration and its
per-chunk cell sort included), shared by the oracle pin (test_golden.py) and the engine's parity test
(test_reference_parity.py).

The reference orders the atoms of a cell by shared-memory atomics (prepNextSubstepKernel, PBF.cu:806-812),
so its order within a cell is not reproducible. What must agree: the number of atoms in every cell, bit for
bit, and the set of atoms in every cell — each reference atom is matched to the nearest atom of the same
cell, and both its position x and its next prediction x* must lie within the tolerance.
"""
import numpy as np

EPS32 = np.finfo(np.float32).eps


def compare_with_reference_sort(ref_cell, ref_x, ref_xs, key, x, xs):
    """ref_*: the reference's atoms (global cell, x, x*, absolute); key, x, xs: the sorted state under test.
    Returns the worst errors found (x, x*), for the record."""
    ref_cell = np.asarray(ref_cell, np.int64)
    key = np.asarray(key, np.int64)
    assert len(ref_cell) == len(key), f"{len(key)} atoms against the reference's {len(ref_cell)}"
    nc = int(max(ref_cell.max(), key.max())) + 1
    cr = np.bincount(ref_cell, minlength=nc)
    ce = np.bincount(key, minlength=nc)
    diff = np.flatnonzero(cr != ce)
    assert diff.size == 0, f"cell counts differ in {diff.size} cells, first {diff[:8]}: {cr[diff[:8]]} vs {ce[diff[:8]]}"
    ref_x, ref_xs = np.asarray(ref_x, np.float64), np.asarray(ref_xs, np.float64)
    x, xs = np.asarray(x, np.float64), np.asarray(xs, np.float64)
    # FP32 results agree to 1e-4 of an atom's displacement per substep (|x* - x|, at most the speed clamp) plus
    # the rounding of the absolute coordinates (the reference computes in chunk-local coordinates)
    step = float(np.abs(ref_xs - ref_x).max())
    tol_x = 1e-4 * step + 8 * EPS32 * np.abs(ref_x).max()
    tol_xs = 2 * tol_x
    ro = np.argsort(ref_cell, kind="stable")
    eo = np.argsort(key, kind="stable")
    rc = ref_cell[ro]
    starts = np.flatnonzero(np.r_[True, rc[1:] != rc[:-1]])
    ends = np.r_[starts[1:], len(rc)]
    worst_x = worst_xs = 0.0
    for s, e in zip(starts, ends):
        R, E = ro[s:e], eo[s:e]
        d = np.linalg.norm(ref_xs[R][:, None, :] - xs[E][None, :, :], axis=2)
        used = np.zeros(len(E), bool)
        for a in np.argsort(d.min(1)):
            row = np.where(used, np.inf, d[a])
            b = int(np.argmin(row))
            used[b] = True
            ex = float(np.abs(ref_x[R[a]] - x[E[b]]).max())
            es = float(np.abs(ref_xs[R[a]] - xs[E[b]]).max())
            worst_x, worst_xs = max(worst_x, ex), max(worst_xs, es)
            assert ex <= tol_x and es <= tol_xs, (
                f"cell {rc[s]}: reference atom at x* {ref_xs[R[a]]} has no counterpart within tolerance "
                f"(nearest x* {xs[E[b]]}, x error {ex:.3e} / {tol_x:.3e}, x* error {es:.3e} / {tol_xs:.3e})")
    return worst_x, worst_xs
