"""Parameter sets and seeded synthetic scenes.

Two parameter regimes:
  * reference mode — the reference's lattice units and constants (libs/common/include/common/constants.h,
    PBF.cu:12-23, MPM.cu), used for parity with the reference's own kernels;
  * the workload configurations the engine is measured on (PBF dam break, MPM elastic squares, 1M-particle
    PBF, batched PBF scenes, mixed-material MPM), built from seeded Philox streams (numpy's Philox4x32-10
    generator, Salmon et al. 2011), one stream per configuration.
"""
from __future__ import annotations

import math

import numpy as np

from . import (MPM_BC_SLIP, MPM_BC_STICKY, MPM_FLAG_FLUID_F, MPM_FLAG_PER_PARTICLE_MATERIAL, MPM_MAT_COROTATED,
               MPM_MAT_FLUID, MPM_MAT_SNOW, PBF_SELF_GRAD, PBF_VEL_CLAMP, MpmParams, PbfParams)

F32 = np.float32


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=seed))


# ===================================================================================================== PBF
def reference_pbf_params(iters: int = 2) -> PbfParams:
    """The reference's PBF constants, evaluated in FP32 in the reference's constexpr order
    (constants.h:24-42, PBF.cu:12-23). Velocities are per-substep displacements (dt = 1)."""
    kPi = F32(3.14159)
    kH = F32(2.0)
    kDt = F32(0.032)
    kPBF_dt = F32(kDt / F32(20.0))
    p = PbfParams()
    p.h = kH
    p.cell = F32(2.0)
    p.rho0 = F32(1.015)
    p.mass = F32(1.0)
    p.dt = F32(1.0)
    p.gravity[0] = 0.0
    p.gravity[1] = F32(F32(F32(1000.0) * kPBF_dt) * kPBF_dt)  # kGravityStep, PBF.cu:19
    p.iters = iters
    p.eps = F32(0.005)
    p.scorr_k = F32(0.005)
    p.scorr_dq = F32(F32(0.2) * kH)
    p.omega = F32(1.25)
    p.c_min = F32(-0.002)
    p.xsph_c = F32(0.035)
    p.vort_eps = 0.0
    p.v_max = F32(1.0)
    p.v_min = F32(0.00005)
    p.wall_margin = F32(1e-3)
    p.poly6_coeff = F32(F32(1.0) / F32(F32(64.0) * kPi))
    p.spiky_coeff = F32(F32(30.0) / F32(F32(32.0) * kPi))
    p.flags = PBF_SELF_GRAD | PBF_VEL_CLAMP
    return p


REFERENCE_BOX = (0.0, 0.0, 12 * 32.0, 6 * 32.0)  # kSceneDimX x kSceneDimY chunks of kChunkDim


def reference_pbf_block(nx: int = 48, ny: int = 40, spacing: float = 1.05, seed: int = 11,
                        origin=(100.0, 60.0), disp=0.05, box=REFERENCE_BOX):
    """A jittered block of atoms with small random displacements (reference units)."""
    g = rng(seed)
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    pos = np.stack([origin[0] + ix.ravel() * spacing, origin[1] + iy.ravel() * spacing], 1)
    pos += g.uniform(-0.05, 0.05, pos.shape)
    vel = g.uniform(-disp, disp, pos.shape)
    return pos.astype(F32), vel.astype(F32), [box]


def reference_border_band(chunk=(5, 2), speed: float = 1.0, seed: int = 31, box=REFERENCE_BOX):
    """Atoms converging on one 32 x 32 chunk of the reference's world from the 2 x 2 cells that border it in its
    eight neighbour chunks (reference units, velocities per substep): 8 atoms per cell, placed so that their
    first prediction x + v + g lies in that cell, every atom moving towards the chunk's centre at `speed`.
    After one substep 258 of them queue for the centre chunk, most of the reference's 320 migration slots
    (kMaxMigrants, constants.h:51), while no border cell holds more atoms than the 8 halo slots the reference
    exports per cell (kCellSlots, constants.h:47; a denser border cell loses neighbours across the chunk
    border in the reference, haloKernel PBF.cu:66-137)."""
    g = rng(seed)
    g_step = reference_pbf_params().gravity[1]
    x0, y0 = chunk[0] * 32.0, chunk[1] * 32.0
    cells = []
    for k in range(16):
        cells += [(x0 - 2.0, y0 + 2 * k, True), (x0 + 32.0, y0 + 2 * k, True),
                  (x0 + 2 * k, y0 - 2.0, False), (x0 + 2 * k, y0 + 32.0, False)]
    cells += [(x0 - 2.0, y0 - 2.0, True), (x0 + 32.0, y0 - 2.0, True), (x0 - 2.0, y0 + 32.0, True),
              (x0 + 32.0, y0 + 32.0, True)]
    across = [(ox, oy) for ox in (0.5, 1.5) for oy in (0.25, 0.75, 1.25, 1.75)]
    along = [(ox, oy) for ox in (0.25, 0.75, 1.25, 1.75) for oy in (0.5, 1.5)]
    pts = [(cx + ox, cy + oy) for cx, cy, side in cells for ox, oy in (across if side else along)]
    xs1 = np.array(pts) + g.uniform(-0.05, 0.05, (len(pts), 2))  # first predictions
    d = np.array([x0 + 16.0, y0 + 16.0]) - xs1
    vel = speed * d / np.linalg.norm(d, axis=1, keepdims=True) + g.uniform(-0.02, 0.02, xs1.shape)
    pos = xs1 - vel
    pos[:, 1] -= g_step
    return pos.astype(F32), vel.astype(F32), [box]


def reference_render_view(seed: int = 41, chunks_x: int = 12, chunks_y: int = 6, capacity: int = 1536,
                          visible=(3, 2), stack: int = 6):
    """A chunk-major view (the reference's View: chunks_x x chunks_y chunks of `capacity` slots, absolute
    coordinates, reference units) whose image the reference's own drawKernel (cuda-render.cu:259-310) draws
    deterministically: every pixel is written by one thread only. In each of the first visible[0] x visible[1]
    chunks, atoms 0..195 sit on a 14 x 14 lattice 2 units (10 pixels at scale 5) apart, 28 more on the chunk's
    left and bottom edges (their splats cover the black chunk lines), and atom a + 256 k (k < stack) on top of
    atom a, a little offset: drawKernel's thread a draws those in order, so stacked splats blend sequentially.
    Splats of different lattice points never overlap; slots 224..255 of every 256 hold atoms outside the
    image, which draw nothing. Chunk counts are seeded; the other chunks are empty.
    Returns (pos [chunks, capacity, 2] float32, counts [chunks] int32)."""
    g = rng(seed)
    pos = np.full((chunks_x * chunks_y, capacity, 2), -50.0, F32)
    counts = np.zeros(chunks_x * chunks_y, np.int32)
    base = [(3.0 + 2 * i, 3.0 + 2 * j) for j in range(14) for i in range(14)]
    base += [(0.2, 3.0 + 2 * j) for j in range(14)] + [(3.0 + 2 * i, 0.2) for i in range(14)]
    base = np.array(base)  # 224 points, chunk-local
    for cy in range(visible[1]):
        for cx in range(visible[0]):
            c = cx + cy * chunks_x
            org = np.array([cx * 32.0, cy * 32.0])
            for k in range(stack):
                jit = g.uniform(-0.1, 0.1, base.shape) if k == 0 else g.uniform(-0.3, 0.3, base.shape)
                pos[c, 256 * k:256 * k + len(base)] = org + base + jit
            counts[c] = int(g.integers(200, min(capacity, 256 * stack) + 1))
    return pos, counts


def reference_million(seed: int = 12, side: int = 1024):
    """1,048,576 atoms on a 1024 x 1024 lattice (spacing 1, the atom diameter) filling a 32 x 32-chunk world
    of the reference (1024 x 1024 units, 1024 atoms per chunk of capacity 1536), small random
    displacements; reference units. The same scene drives the engine and the reference's kernels."""
    g = rng(seed)
    ix, iy = np.meshgrid(np.arange(side), np.arange(side), indexing="xy")
    pos = np.stack([ix.ravel() + 0.5, iy.ravel() + 0.5], 1)
    pos += g.uniform(-0.05, 0.05, pos.shape)
    vel = g.uniform(-0.02, 0.02, pos.shape)
    return pos.astype(F32), vel.astype(F32), [(0.0, 0.0, float(side), float(side))]


def lattice_mass(h: float, spacing: float, rho0: float = 1.0) -> float:
    """Particle mass that makes the 2D poly6 density of a square lattice equal rho0."""
    c6 = 4.0 / (math.pi * h ** 8)
    r = int(math.ceil(h / spacing))
    s = 0.0
    for i in range(-r, r + 1):
        for j in range(-r, r + 1):
            q = h * h - (i * spacing) ** 2 - (j * spacing) ** 2
            if q >= 0:
                s += c6 * q ** 3
    return rho0 / s


def dam_params(iters: int = 4, h: float = 0.02, spacing: float = 0.01) -> PbfParams:
    """Plain PBF dam break: h=0.02, rest density 1, gravity -9.8, dt=1/120, epsilon 100, XSPH c=0.01.
    The XSPH coefficient is the mass/density-normalised one: the engine applies
    v += c_abs sum_j (v_j - v_i) W_ij, so c_abs = c m / rho0."""
    m = lattice_mass(h, spacing)
    p = PbfParams()
    p.h = h
    p.cell = 0.0
    p.rho0 = 1.0
    p.mass = m
    p.dt = 1.0 / 120.0
    p.gravity[0] = 0.0
    p.gravity[1] = -9.8
    p.iters = iters
    p.eps = 100.0
    p.scorr_k = 0.0
    p.scorr_dq = 0.2 * h
    p.omega = 1.0
    p.c_min = 0.0
    p.xsph_c = 0.01 * m / 1.0
    p.vort_eps = 0.0
    p.v_max = 0.0
    p.v_min = 0.0
    p.wall_margin = 1e-6
    p.poly6_coeff = 0.0
    p.spiky_coeff = 0.0
    p.flags = 0
    return p


def dam_break(n_side: int = 128, spacing: float = 0.01, box: float = 2.56, seed: int = 0, h: float = 0.02):
    """16,384 particles on a 128x128 lattice (spacing 0.5h) in the lower-left quarter of a square box,
    jittered by U(+-0.01h), at rest. The box side is 2.56 so that the 1.28-wide block is exactly its
    lower-left quarter."""
    g = rng(seed)
    ix, iy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy")
    pos = np.stack([(ix.ravel() + 0.5) * spacing, (iy.ravel() + 0.5) * spacing], 1)
    pos += g.uniform(-0.01 * h, 0.01 * h, pos.shape)
    vel = np.zeros_like(pos)
    return pos.astype(F32), vel.astype(F32), [(0.0, 0.0, box, box)]


def million(seed: int = 2, spacing: float = 0.01, h: float = 0.02):
    """1,048,576 particles in a 20.48 x 20.48 domain (4 x 4 chunks of 5.12): a 960 x 1024 lattice block
    (983,040 particles, spacing 0.5h) in the lower-left corner plus a 256 x 256 splash block
    (65,536 particles) higher up with random directions and |v| ~ U(0, 2)."""
    g = rng(seed)
    side = 20.48
    ix, iy = np.meshgrid(np.arange(960), np.arange(1024), indexing="xy")
    block = np.stack([(ix.ravel() + 0.5) * spacing, (iy.ravel() + 0.5) * spacing], 1)
    sx, sy = np.meshgrid(np.arange(256), np.arange(256), indexing="xy")
    splash = np.stack([12.0 + (sx.ravel() + 0.5) * spacing, 12.0 + (sy.ravel() + 0.5) * spacing], 1)
    pos = np.concatenate([block, splash])
    pos += g.uniform(-0.01 * h, 0.01 * h, pos.shape)
    vel = np.zeros_like(pos)
    ang = g.uniform(0.0, 2.0 * math.pi, splash.shape[0])
    sp = g.uniform(0.0, 2.0, splash.shape[0])
    vel[block.shape[0]:, 0] = sp * np.cos(ang)
    vel[block.shape[0]:, 1] = sp * np.sin(ang)
    return pos.astype(F32), vel.astype(F32), [(0.0, 0.0, side, side)]


MILLION_DT = 1.0 / 2000.0  # the 10 m deep block needs an effective sound speed K dx / dt well above sqrt(g H)


def million_workload(iters: int = 4):
    """The 1M-particle PBF workload: million() with the dam-break physics at dt = 1/2000 (the plain 4-iteration
    form diverges at 1/240 and above on this 10 m deep block). Returns (params, pos, vel, boxes)."""
    p = dam_params(iters=iters)
    p.dt = MILLION_DT
    pos, vel, boxes = million()
    return p, pos, vel, boxes


BATCHED_DT = 1.0 / 480.0  # the dam-break physics is stable at 1/480, not at 1/120 (4 Jacobi iterations)


def batched_workload(iters: int = 4, n_scenes: int = 256):
    """256 independent dam-break scenes (batched_scenes, seed 3, 2,048-65,536 particles each) with the
    dam-break physics at dt = 1/480. Returns (params, pos, vel, dom, boxes)."""
    p = dam_params(iters=iters)
    p.dt = BATCHED_DT
    pos, vel, dom, boxes = batched_scenes(n_scenes=n_scenes, seed=3, lo=2048, hi=65536)
    return p, pos, vel, dom, boxes


def batched_scenes(n_scenes: int = 256, seed: int = 3, lo: int = 2048, hi: int = 65536, spacing: float = 0.01):
    """Independent dam-break scenes: particle counts log-uniform in [lo, hi], box aspect U(0.5, 2). Each
    scene's block fills the lower-left quarter of its box at spacing 0.5h. Returns (pos, vel, dom, boxes);
    scenes are laid side by side (disjoint boxes) but never interact."""
    g = rng(seed)
    counts = np.exp(g.uniform(math.log(lo), math.log(hi), n_scenes)).astype(np.int64)
    aspects = g.uniform(0.5, 2.0, n_scenes)
    pos_l, vel_l, dom_l, boxes = [], [], [], []
    x0 = 0.0
    for s in range(n_scenes):
        n = int(counts[s])
        a = float(aspects[s])  # width / height of the block (and of the box)
        bw = max(1, int(round(math.sqrt(n * a))))
        bh = max(1, int(math.ceil(n / bw)))
        ix, iy = np.meshgrid(np.arange(bw), np.arange(bh), indexing="xy")
        p = np.stack([(ix.ravel() + 0.5) * spacing, (iy.ravel() + 0.5) * spacing], 1)[:n]
        p += g.uniform(-0.0002, 0.0002, p.shape)
        W, H = 2.0 * bw * spacing, 2.0 * bh * spacing
        p[:, 0] += x0
        boxes.append((x0, 0.0, W, H))
        pos_l.append(p)
        vel_l.append(np.zeros_like(p))
        dom_l.append(np.full(n, s, np.int32))
        x0 += W + 1.0
    return (np.concatenate(pos_l).astype(F32), np.concatenate(vel_l).astype(F32), np.concatenate(dom_l),
            boxes)


# ===================================================================================================== MPM
def reference_mpm_params() -> MpmParams:
    """The reference's MLS-MPM constants (constants.h:72-88, MPM.cu), FP32."""
    p = MpmParams()
    kDt = F32(0.032)
    p.dx = 2.0
    p.grid_offset = 2.0
    p.nx = 12 * 32 // 2 + 4
    p.ny = 6 * 32 // 2 + 4
    p.dt = F32(kDt / F32(20))
    p.gravity[0] = 0.0
    p.gravity[1] = 700.0
    p.mass = 1.0
    p.vol0 = 1.2
    p.bc_type = MPM_BC_SLIP
    p.bc_width = 2
    p.clamp_lo[0], p.clamp_lo[1] = 0.0, 0.0
    p.clamp_hi[0], p.clamp_hi[1] = 384.0, 192.0
    p.material = MPM_MAT_FLUID
    p.k_bulk = 8.2e4
    p.gamma = 3.2
    p.p_min = F32(-0.0) * F32(8.2e4)
    p.p_max = F32(10.0) * F32(8.2e4)
    p.J_min = 0.1
    p.J_max = 10.0
    p.E = 0.0
    p.nu = 0.0
    p.theta_c = 0.0
    p.theta_s = 0.0
    p.hardening = 0.0
    p.sort_interval = 0
    p.flags = MPM_FLAG_FLUID_F
    return p


def reference_mpm_block(nx: int = 60, ny: int = 40, spacing: float = 1.26, seed: int = 21,
                        origin=(60.0, 40.0)):
    g = rng(seed)
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    pos = np.stack([origin[0] + ix.ravel() * spacing, origin[1] + iy.ravel() * spacing], 1)
    pos += g.uniform(-0.1, 0.1, pos.shape)
    vel = g.uniform(-20.0, 20.0, pos.shape)
    n = pos.shape[0]
    Cm = g.uniform(-0.5, 0.5, (n, 4))
    F = np.tile(np.array([1, 0, 0, 1], F32), (n, 1)) + g.uniform(-0.01, 0.01, (n, 4))
    J = g.uniform(0.95, 1.05, n)
    return pos.astype(F32), vel.astype(F32), Cm.astype(F32), F.astype(F32), J.astype(F32)


def elastic_params(n: int = 65536, grid: int = 128) -> MpmParams:
    """Plain MLS-MPM: 128^2 grid over the unit box, fixed-corotated E=1e3, nu=0.2, particle mass 1/65536,
    dt=1e-4, gravity -9.8, sticky walls 3 nodes wide."""
    dx = 1.0 / grid
    p = MpmParams()
    p.dx = dx
    p.grid_offset = 0.0
    p.nx = grid
    p.ny = grid
    p.dt = 1e-4
    p.gravity[0] = 0.0
    p.gravity[1] = -9.8
    p.mass = 1.0 / 65536.0
    p.vol0 = 2 * 0.25 * 0.25 / n
    p.bc_type = MPM_BC_STICKY
    p.bc_width = 2
    p.clamp_lo[0] = p.clamp_lo[1] = 2 * dx
    p.clamp_hi[0] = p.clamp_hi[1] = 1.0 - 3 * dx
    p.material = MPM_MAT_COROTATED
    p.k_bulk = 0.0
    p.gamma = 1.0
    p.p_min = -1e30
    p.p_max = 1e30
    p.J_min = 0.1
    p.J_max = 10.0
    p.E = 1e3
    p.nu = 0.2
    p.theta_c = 2.5e-2
    p.theta_s = 4.5e-3
    p.hardening = 10.0
    p.sort_interval = 0
    p.flags = 0
    return p


def two_squares(n: int = 65536, seed: int = 1):
    """65,536 particles uniform in two 0.25 x 0.25 squares (4 per cell on a 128^2 grid would need 0.0625
    area per 4096 particles; here each square holds 32,768, i.e. 32 per cell)."""
    g = rng(seed)
    h = n // 2
    a = g.uniform(0.0, 0.25, (h, 2)) + np.array([0.2, 0.2])
    b = g.uniform(0.0, 0.25, (n - h, 2)) + np.array([0.55, 0.45])
    pos = np.concatenate([a, b]).astype(F32)
    vel = np.zeros_like(pos)
    vel[:h, 0] = 0.5
    vel[h:, 0] = -0.5
    return pos, vel


def elastic_workload(sort_interval: int = 16):
    """The plain MLS-MPM workload: 65,536 fixed-corotated particles in two squares on a 128^2 grid
    (elastic_params, two_squares), 32 particles per cell, re-sorted by cell every sort_interval steps so that
    the particles of a cell are consecutive. Returns (params, pos, vel)."""
    p = elastic_params()
    p.sort_interval = sort_interval
    pos, vel = two_squares()
    return p, pos, vel


def mixed_params(n: int, grid: int = 1024) -> MpmParams:
    """Mixed materials on a 1024^2 grid: water (J-based EOS, bulk modulus 10), snow (theta_c=2.5e-2,
    theta_s=4.5e-3, hardening 10) and jelly (E=5e3, nu=0.2); dt=5e-5."""
    p = elastic_params(n, grid)
    p.dt = 5e-5
    p.E = 5e3
    p.nu = 0.2
    p.k_bulk = 10.0
    p.gamma = 1.0
    p.p_min = -1e30
    p.p_max = 1e30
    p.flags = MPM_FLAG_PER_PARTICLE_MATERIAL
    # density 1000: the jelly's wave speed sqrt(E / rho) is then 2.2 m/s and dt c / dx = 0.12 on the 1024^2
    # grid (at density 3.3, 1 / n per particle, it is 2.0 and the step diverges)
    p.vol0 = 0.3 / n
    p.mass = 1000.0 * p.vol0
    # re-sorted by base node every 32 steps: mean step over 64 steps 0.172 / 0.163 / 0.159 / 0.158 ms at
    # intervals 8 / 16 / 32 / 64 (GB300, 4M particles), the runs of particles on one base node staying long
    p.sort_interval = 32
    return p


def mixed_discs(n: int = 4194304, seed: int = 4, discs_per_material: int = 3, area: float = 0.3,
                materials=(MPM_MAT_FLUID, MPM_MAT_SNOW, MPM_MAT_COROTATED)):
    """n particles, an equal share of each material (default: water, snow and jelly), in seeded random discs
    of equal radius."""
    g = rng(seed)
    k_m = len(materials)
    nd = k_m * discs_per_material
    r = math.sqrt(area / (nd * math.pi))
    per_mat = [n // k_m] * (k_m - 1) + [n - (k_m - 1) * (n // k_m)]
    pos_l, mat_l = [], []
    for m, cnt in zip(materials, per_mat):
        cs = g.uniform(0.15 + r, 0.85 - r, (discs_per_material, 2))
        split = [cnt // discs_per_material] * discs_per_material
        split[-1] += cnt - sum(split)
        for c, k in zip(cs, split):
            rad = r * np.sqrt(g.uniform(0, 1, k))
            th = g.uniform(0, 2 * math.pi, k)
            pos_l.append(np.stack([c[0] + rad * np.cos(th), c[1] + rad * np.sin(th)], 1))
            mat_l.append(np.full(k, m, np.int32))
    pos = np.concatenate(pos_l).astype(F32)
    mat = np.concatenate(mat_l)
    # spatially coherent initial order (row-major by grid cell), which keeps P2G tiles small
    cell = (np.floor(pos[:, 1] * 1024).astype(np.int64) * 1024 + np.floor(pos[:, 0] * 1024).astype(np.int64))
    order = np.argsort(cell, kind="stable")
    return pos[order], mat[order]


def mixed_batch(n_scenes: int = 32, seed: int = 6, lo: int = 65536, hi: int = 524288, total_ref: int = 4194304):
    """Independent mixed-material scenes for one batched engine: particle counts log-uniform in [lo, hi],
    each scene water, snow and jelly discs (mixed_discs) covering 0.3 of its square box. Every scene has the
    particle density of the total_ref-particle scene on the 1024^2 grid (mixed_params(total_ref)), so they
    share dx, dt, mass and vol0; scene q's grid is g_q x g_q nodes, g_q = 1024 sqrt(n_q / total_ref) rounded
    up to a multiple of 8 (128 nodes for 64k particles, 368 for 512k).
    Returns (params, scenes, pos, mat, scene_id): scenes as (nx, ny, clamp_lo, clamp_hi) tuples, positions
    in each scene's own coordinates, scene-major."""
    g = rng(seed)
    counts = np.exp(g.uniform(math.log(lo), math.log(hi), n_scenes)).astype(np.int64)
    p = mixed_params(total_ref)
    dx = p.dx
    scenes, pos_l, mat_l, sid_l = [], [], [], []
    for q in range(n_scenes):
        n = int(counts[q])
        side = int(math.ceil(1024.0 * math.sqrt(n / total_ref) / 8.0)) * 8
        L = side * dx
        pos, mat = mixed_discs(n, seed=1000 + seed * 64 + q)
        scenes.append((side, side, (2 * dx, 2 * dx), (L - 3 * dx, L - 3 * dx)))
        pos_l.append(pos * F32(L))
        mat_l.append(mat)
        sid_l.append(np.full(n, q, np.int32))
    return p, scenes, np.concatenate(pos_l).astype(F32), np.concatenate(mat_l), np.concatenate(sid_l)
