"""Generates the golden fixtures in this directory by running the reference's own kernels (built headless by
oracle/build_ref.py) on a GPU:

  pbf_reference_substep.npz  one PBF substep of a 48 x 40 atom block that straddles chunk borders, stopped
                             after XSPHKernel (PBF.cu:921-946): inputs x, v (absolute, dt = 1 units), the
                             chunk slot of every atom (the reference's pairDirection seed), and the outputs
                             x* (corrected), v (XSPH + clamp) and lambda of the last iteration, per input atom.
  mpm_reference_substep.npz  one MLS-MPM substep (resetGrid, P2G, grid, G2P; MPM.cu:357-368) of a 30 x 40
                             particle block with random v, C, F, J: inputs and outputs per particle.
  pbf_reference_migration.npz  one complete PBF substep (PBF.cu:921-955: halo, 2 x (lambda, delta p),
                             velocity, XSPH, migration, prepNextSubstepKernel's queue drain, prediction and
                             per-chunk cell sort) of the border band around chunk (5, 2)
                             (gpe.scenes.reference_border_band): inputs x, v and the chunk slot of every
                             atom; the migration queue fill of every destination chunk after migrationKernel;
                             and every atom after the sort, in the reference's order: its global cell (row-major
                             over the 192 x 96 cells of the 12 x 6 chunks), x and the next prediction x*,
                             absolute. The reference's intra-cell order follows shared-memory atomics, so only
                             per-cell counts and per-cell atom sets are comparable.

  render_reference_frame.npz  the reference's splat renderer (backgroundKernel + drawKernel,
                             cuda-render.cu:214-310) on gpe.scenes.reference_render_view into a 470 x 300
                             image: the view (pos, counts), the size and the RGBA8 image. The view is drawn
                             deterministically by the reference (no pixel is written by two threads).

Usage (on a machine with a GPU): python tests/golden/make_golden.py OUT_DIR [fixture stem ...]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "gpu-physics-engine_gb300"))
sys.path.insert(0, str(ROOT))


def make_pbf():
    from gpe import scenes
    from oracle import refrun

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_pbf_block()
    ref = refrun.RefPBF((12, 6), 320)
    _, slot = ref.seed(pos, vel, float(p.gravity[1]))
    ref.substep(iters=2, full=False)
    xs, v, lam = ref.read_seeded()
    return dict(x=pos, v=vel, slot=slot.astype(np.uint32), out_x=xs, out_v=v, out_lambda=lam)


def make_pbf_migration():
    import torch

    from gpe import scenes
    from oracle import refrun

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, _ = scenes.reference_border_band()
    ref = refrun.RefPBF((12, 6), 320)
    _, slot = ref.seed(pos, vel, float(p.gravity[1]))
    ref.substep(iters=2, full=False)
    ref.migrate()
    torch.cuda.synchronize()
    mig = ref.mig_count.cpu().numpy().astype(np.int32)
    ref.prep()
    cell, x, xs = ref.read_sorted()
    return dict(x=pos, v=vel, slot=slot.astype(np.uint32), mig_count=mig, out_cell=cell, out_x=x, out_xs=xs)


def make_render():
    from gpe import scenes
    from oracle import refrun

    pos, counts = scenes.reference_render_view()
    w, h = 470, 300
    img = refrun.RefRender().render(pos, counts, w, h)
    return dict(pos=pos, counts=counts, width=np.int32(w), height=np.int32(h), image=img)


def make_mpm():
    from gpe import scenes
    from oracle import refrun

    x, v, Cm, F, J = scenes.reference_mpm_block(nx=30, ny=40)
    ref = refrun.RefMPM(400 * 1000, (12, 6))
    ref.seed(x, v, Cm, F, J)
    ref.substep(0)
    ox, ov, oC, oF, oJ = ref.read()
    return dict(x=x, v=v, C=Cm, F=F, J=J, out_x=ox, out_v=ov, out_C=oC, out_F=oF, out_J=oJ)


FIXTURES = {"pbf_reference_substep": make_pbf, "mpm_reference_substep": make_mpm,
            "pbf_reference_migration": make_pbf_migration, "render_reference_frame": make_render}

if __name__ == "__main__":
    out = Path(sys.argv[1] if len(sys.argv) > 1 else Path(__file__).parent)
    out.mkdir(parents=True, exist_ok=True)
    for stem in (sys.argv[2:] or list(FIXTURES)):
        np.savez_compressed(out / f"{stem}.npz", **FIXTURES[stem]())
        print("wrote", out / f"{stem}.npz")
