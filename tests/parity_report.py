"""Prints, as a markdown table, the error of one engine step against the FP64 oracle for the PBF and MLS-MPM
scenes of the parity tests (run on a GPU: python tests/parity_report.py). Errors are max |engine - oracle|
over particles, relative to the field's largest magnitude; sort results are compared bit for bit."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "gpu-physics-engine_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import gpe  # noqa: E402
from oracle import pyoracle as oracle  # noqa: E402
import test_mpm_gpu as tm  # noqa: E402
import test_pbf_gpu as tp  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / s) if s > 0 else float(np.abs(a - b).max())


def pbf_rows():
    rows = []
    for kind in ("reference", "dam", "dam_half_cell", "batched"):
        p, pos, vel, dom, boxes = tp._scene(kind)
        e = tp._engine(gpe, p, pos, vel, dom, boxes)
        e.stage(gpe.PBF_STAGE_PREDICT_SORT)
        s = oracle.PbfOracle(p, boxes).predict_sort(pos, vel, dom)
        exact = (np.array_equal(e.field(gpe.PBF_FIELD_KEY), s["key"])
                 and np.array_equal(e.field(gpe.PBF_FIELD_PERM), s["perm"])
                 and np.array_equal(e.field(gpe.PBF_FIELD_CELL_START), s["cell_start"])
                 and np.array_equal(e.field(gpe.PBF_FIELD_PRED).view(np.uint32), s["xs"].view(np.uint32)))
        e.close()
        e = tp._engine(gpe, p, pos, vel, dom, boxes)
        e.step(1)
        x, v, _ = e.get_state()
        r = oracle.PbfOracle(p, boxes).step(pos, vel, dom, n_steps=1)
        rows.append((f"PBF {kind} ({len(pos)} particles, K = {p.iters})", exact, rel(x, r["x"]), rel(v, r["v"])))
        e.close()
    return rows


def mpm_rows():
    rows = []
    for kind in tm.KINDS:
        p, x, v, Cm, F, J, mat = tm._scene(kind)
        e = tm._engine(gpe, p, x, v, Cm, F, J, mat)
        e.stage(gpe.MPM_STAGE_CLEAR)
        e.stage(gpe.MPM_STAGE_P2G)
        g = e.grid()
        want = oracle.MpmOracle(p).p2g(x, v, Cm, F, J, mat)
        eg = (rel(g[:, 2], want[:, 2]), rel(g[:, :2], want[:, :2]))
        e.close()
        e = tm._engine(gpe, p, x, v, Cm, F, J, mat)
        e.step(1)
        x1, v1, C1, F1, J1 = e.get_state()
        wx, wv, wC, wF, wJ = oracle.MpmOracle(p).step(x, v, Cm, F, J, mat, n_steps=1)
        sel = slice(None) if mat is None else (mat != gpe.MPM_MAT_FLUID)
        rows.append((f"MPM {kind} ({len(x)} particles)", eg, rel(x1, wx), rel(v1, wv), rel(C1, wC),
                     rel(F1[sel], wF[sel]) if kind != "fluid" else None, rel(J1, wJ)))
        e.close()
    return rows


def main():
    print("| PBF scene | keys, order, cell starts, x* bit-exact | x | v |")
    print("|---|---|---:|---:|")
    for name, exact, ex, ev in pbf_rows():
        print(f"| {name} | {'yes' if exact else 'NO'} | {ex:.1e} | {ev:.1e} |")
    print()
    print("| MPM scene | grid mass after P2G | grid momentum | x | v | C | F | J |")
    print("|---|---:|---:|---:|---:|---:|---:|---:|")
    for name, (gm, gp), ex, ev, ec, ef, ej in mpm_rows():
        f = "—" if ef is None else f"{ef:.1e}"
        print(f"| {name} | {gm:.1e} | {gp:.1e} | {ex:.1e} | {ev:.1e} | {ec:.1e} | {f} | {ej:.1e} |")


if __name__ == "__main__":
    main()
