"""Benchmark: PBF particle-steps/s at 1,048,576 particles (plain 4-iteration Jacobi form) on one GB300.

A step is one PBF solver step (the reference's substep: predict + sort, 4 x (lambda, delta p), velocity +
XSPH) over the 1M-particle scene (a 960 x 1024 lattice block plus a 65,536-particle splash, 20.48 x 20.48
domain, h = 0.02, dt = 1/2000: the 10 m deep block needs an effective sound speed K dx / dt well above
sqrt(g H), and the plain 4-iteration form diverges at 1/240 and above). Inputs are resident in HBM when the
timed region starts; L2 is flushed (a 256 MiB memset) before every timed step, since the working set
(~60 MB) would otherwise stay in the 129 MB L2 across steps.

learned: the network-warm-started 2-iteration step against the plain forms on the same scene (its network
       trained on the GPU first, untimed), with the density error each reaches.

value: particle-steps/s through the graph-launched step (gpe_pbf_step), CUDA events on the launch stream.
e2e:   the same metric through the C ABI with host buffers: per step set_state from pinned host memory,
       one step, get_state back to pinned host memory, all inside the timed region; three engines on three
       streams take turns so that one step's copies overlap the others' compute (the one-engine,
       synchronous figure is reported beside it).
roofline: the dominant kernel (largest share of step time) timed per launch in a stage-by-stage pass with
       CUDA events, against its algorithmic bytes per particle.
cpu_baseline: the oracle's OpenMP FP64 restatement of the same step on a bounded sample, host cores.

`--impl reference` times the reference's path on the host cores: the reference has no CPU implementation
of its solver, so the oracle port stands in for it (kind "port").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "gpu-physics-engine_gb300"))
sys.path.insert(0, str(ROOT))

HBM_FALLBACK = 6800.0
ALG_BYTES = {  # algorithmic bytes per particle per launch (FP32 SoA, each field read/written once)
    "predict_sort": 36.0,  # read x, v; write x, x*, perm
    "lambda": 12.0,        # read x*; write lambda
    "delta_p": 20.0,       # read x*, lambda; write x*
    "xsph": 24.0,          # read x, x*; write v
}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the 1M-particle step's neighbour
# kernels from ncu captures of this workload's first timed step (cold caches: ncu flushes them before each
# replay). lambda: the mean over a step's four launches, the mask-recording pass (22.1 MB) and three masked
# passes (39.1 MB each, which also read the 16 MB candidate-mask array and the cell starts that stay in L2
# in a live step)
NCU_TRAFFIC = {"lambda": 34.87e6, "delta_p": 43.5e6, "xsph": 39.27e6}
# warp instructions per launch (smsp__inst_executed.sum) of the same kernels from the same captures; lambda:
# the mean over a step's four launches (the mask-recording lambda executes 45.8 M, a masked one 20.8 M). The
# neighbour kernels are bound by instruction issue, and the issue roofline is these instructions over the
# live launch time against 4 schedulers x SMs x the sampled SM clock.
NCU_WARP_INST = {"lambda": 27.05e6, "delta_p": 20.21e6, "xsph": 15.71e6}

# engines whose steps alternate in the end-to-end measurement (measured when every step restarted from the
# initial state: 1 engine 0.608 ms per step with synchronous copies, 2 engines 0.411, 3 engines 0.386)
E2E_ENGINES = 3


def peaks():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 6:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, val in zip(names, f[2:6]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("GPE_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, local_s: float, ws: int) -> float:
    """Whole-job throughput of ws replicas that each processed units_per_rank units in local_s seconds: the
    units of all ranks over the slowest rank's time (every rank runs the same scene; no data crosses ranks)."""
    return ws * units_per_rank / allmax(local_s, ws)


def workload(iters: int = 4):
    from gpe import scenes

    p, pos, vel, boxes = scenes.million_workload(iters=iters)
    cfg = {"workload": "pbf_1m_plain_k4", "particles": int(len(pos)), "iters": iters, "h": 0.02,
           "dt": "1/2000", "domain": "20.48 x 20.48 (4 x 4 chunks of 5.12)", "cells": 1024 * 1024,
           "scene": "960x1024 lattice block + 256x256 splash |v|~U(0,2), seed 2",
           "l2": "flushed before every timed step (256 MiB memset)"}
    return p, pos, vel, boxes, cfg


def learned_leg(args, stream, flush_l2):
    """The learned warm start against the plain form on the same scene: the network is trained first (pairs
    from 41 plain 20-iteration steps, every 20th particle, 30 epochs on the GPU, best of three seeds on a
    held-out stretch of the scene; untimed), then the
    network-warm-started 2-iteration step (and the 1-iteration one, the network's multiplier alone) and the
    plain forms are timed like the headline."""
    import torch

    import gpe

    sh = stream.cuda_stream
    p20, pos, vel, boxes, _ = workload(iters=20)
    n = len(pos)
    e = gpe.Pbf(p20, boxes, capacity=n)
    e.set_state(pos, vel, stream=sh)
    col = gpe.Mlp(max_pairs=2_200_000, seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    col.collect(e, n_steps=41, stride=20, seed=3, stream=sh)
    t_col = time.perf_counter() - t0
    X, T, _ = col.pairs()
    col.close()
    # the state after the collection steps: a later stretch of the scene, on which the candidates are judged
    vx, vv, _ = e.get_state()
    e.close()

    def held_out_error(net):
        p2, _, _, _, _ = workload(iters=2)
        eng = gpe.Pbf(p2, boxes, capacity=n)
        eng.set_state(vx, vv, stream=sh)
        eng.set_warm_start(gpe.WARM_MLP, net)
        eng.step(10, stream=sh)
        dmax, _ = eng.density_error(stream=sh)
        eng.close()
        return dmax

    # three networks from three seeds on the same pairs; the one with the smallest max density error over 10
    # warm-started steps from the held-out state is kept (the training order varies from run to run with the
    # atomic appends of the pair collection, and so does the worst particle's error)
    t0 = time.perf_counter()
    cands = []
    for seed in (1, 2, 3):
        cand = gpe.Mlp(max_pairs=len(T), seed=seed)
        cand.set_pairs(X, T)
        tl_c, vl_c = cand.train(gpe.make_train_params(epochs=30, batch=8192, lr=2e-3, val_fraction=0.1, seed=seed,
                                                      lr_schedule=1), stream=sh)
        cands.append((held_out_error(cand), seed, tl_c, vl_c, cand))
    t_tr = time.perf_counter() - t0
    cands.sort(key=lambda c: c[0])
    held, best_seed, tl, vl, net = cands[0]
    for c in cands[1:]:
        c[4].close()
    pairs = len(T)

    def timed(iters, warm):
        p, _, _, _, _ = workload(iters=iters)
        eng = gpe.Pbf(p, boxes, capacity=n)
        eng.set_state(pos, vel, stream=sh)
        if warm:
            eng.set_warm_start(gpe.WARM_MLP, net)
        for _ in range(args.warmup):  # with the network, the first of these starts the multiplier memory
            eng.step(1, stream=sh)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in ev:
            flush_l2()
            a.record(stream)
            eng.step(1, stream=sh)
            b.record(stream)
        torch.cuda.synchronize()
        s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
        dmax, dmean = eng.density_error(stream=sh)
        st = eng.status()
        eng.close()
        return {"value": n * args.steps / s, "ms_per_step": 1e3 * s / args.steps, "iters": iters,
                "density_error": {"max": dmax, "mean": dmean}, "status": st}

    learned = timed(2, True)
    learned_k1 = timed(1, True)  # the network's multiplier alone: one delta p pass, no plain iteration
    plain2 = timed(2, False)
    # the cheapest plain form that reaches the learned form's density error, for the equal-error comparison
    plain_k = {}
    for k in (6, 8, 12):
        plain_k[f"k{k}"] = timed(k, False)
    reach = [v for v in plain_k.values() if v["density_error"]["max"] <= max(learned["density_error"]["max"], 0.01)]
    cheapest = min(reach, key=lambda v: v["ms_per_step"]) if reach else None
    learned.update({"network_k1": learned_k1, "plain_k2": plain2, "plain_more_iters": plain_k,
                    "speedup_vs_cheapest_plain_at_equal_error": (learned["value"] / cheapest["value"]) if cheapest
                    else None,
                    "train": {"pairs": pairs, "train_loss": tl, "val_loss": vl, "collect_s": t_col, "train_s": t_tr,
                              "seed": best_seed,
                              "held_out_max_density_error": {f"seed{c[1]}": c[0] for c in cands},
                              "how": "pairs from 41 plain 20-iteration steps (every 20th particle); three networks "
                                     "(seeds 1-3), 30 epochs each, batch 8192, AdamW lr 2e-3 with cosine decay, "
                                     "standardised MSE; the one with the smallest max density error over 10 "
                                     "warm-started steps from the state after collection is kept"}})
    return learned


def cpu_baseline(p, pos, vel, boxes, budget_s=12.0, max_steps=30):
    from oracle import pyoracle

    o = pyoracle.PbfOracle(p, boxes)
    o.step(pos, vel, None, 1)  # warm-up (page-in, thread pool)
    x, v = pos, vel
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < budget_s:
        r = o.step(x, v, None, 1)
        x, v = r["x"], r["v"]
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": len(pos) * steps / dt, "unit": "particle-steps/s", "cores": pyoracle.num_threads(),
            "kind": "port",
            "sample": f"{steps} full steps of the {len(pos)}-particle workload (FP64 oracle, OpenMP)"}


def reference_cuda_leg(args, stream, flush_l2):
    """The reference's own PBF kernels (PBF.cu built for sm_103a, a 32 x 32-chunk world) against the engine on
    the same 1M-atom scene with the reference's constants (2 Jacobi iterations, dt = 1 units). Both timed per
    substep with CUDA events after an L2 flush; the reference's substep (10 nodes, PBF.cu:921-955) is
    captured once into a CUDA graph as the reference does."""
    import torch

    import gpe
    from gpe import scenes

    cubin = ROOT / "oracle" / "_ref" / "PBF_ref_32x32_m320.cubin"
    if not cubin.exists():
        return {"unavailable": "reference kernels not built (oracle/build_ref.py needs the reference sources)"}
    from oracle import refrun

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_million()
    n = len(pos)
    sh = stream.cuda_stream

    def timed(run_one):
        for _ in range(args.warmup):
            run_one()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for a, b in ev:
            flush_l2()
            a.record(stream)
            run_one()
            b.record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / 1e3

    ref = refrun.RefPBF((32, 32), 320, cubin=cubin)
    ref.seed(pos, vel, float(p.gravity[1]))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        ref.substep(iters=p.iters, full=True, stream=sh)

    def replay():
        with torch.cuda.stream(stream):  # replay on the stream the events are recorded on
            graph.replay()

    ref_s = timed(replay)
    atoms_kept = int(ref.num_atoms.sum().item())
    del graph, ref
    e = gpe.Pbf(p, boxes, capacity=n)
    e.set_state(pos, vel, stream=sh)
    eng_s = timed(lambda: e.step(1, stream=sh))
    e.close()
    out = {"workload": "pbf_1m_reference_units_k2", "particles": n, "unit": "particle-steps/s",
           "reference_value": n * args.steps / ref_s, "engine_value": n * args.steps / eng_s,
           "speedup": ref_s / eng_s, "reference_ms_per_step": 1e3 * ref_s / args.steps,
           "engine_ms_per_step": 1e3 * eng_s / args.steps, "reference_atoms_after": atoms_kept,
           "how": "reference PBF.cu kernels (sm_103a cubin, 32x32 chunks) in a CUDA graph vs gpe_pbf_step, "
                  "same scene and constants, L2 flushed before each timed substep"}
    out["mpm"] = reference_mpm_leg(timed, stream, args.steps)
    out["small"] = reference_small_leg(timed, stream, args.steps)
    return out


def reference_small_leg(timed, stream, steps):
    """The small configurations against the reference's own kernels, reference units and constants: PBF with
    16,384 atoms (a 128 x 128 block) in the reference's 12 x 6-chunk world (K = 2), and MLS-MPM with 65,536
    J-EOS fluid particles (a 256 x 256 block) on its 196 x 100-node grid, the reference's MPM substep at its
    36-block launch shape and at 8 blocks per SM. Per substep, graph-launched, L2 flushed before each."""
    import torch

    import gpe
    from gpe import scenes
    from oracle import refrun

    pbf_cubin = ROOT / "oracle" / "_ref" / "PBF_ref_12x6_m320.cubin"
    mpm_cubin = ROOT / "oracle" / "_ref" / "MPM_ref_12x6_n400000.cubin"
    if not (pbf_cubin.exists() and mpm_cubin.exists()):
        return {"unavailable": "reference kernels not built (oracle/build_ref.py needs the reference sources)"}
    sh = stream.cuda_stream
    out = {}

    def graph_of(fn):
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            fn()

        def replay():
            with torch.cuda.stream(stream):
                graph.replay()

        return graph, replay

    g = np.random.default_rng(5)
    ix, iy = np.meshgrid(np.arange(128), np.arange(128), indexing="xy")
    x = np.stack([20.0 + ix.ravel(), 20.0 + iy.ravel()], 1) + g.uniform(-0.05, 0.05, (128 * 128, 2))
    v = g.uniform(-0.02, 0.02, x.shape)
    x, v = x.astype(np.float32), v.astype(np.float32)
    p = scenes.reference_pbf_params(iters=2)
    ref = refrun.RefPBF((12, 6), 320, cubin=pbf_cubin)
    ref.seed(x, v, float(p.gravity[1]))
    graph, replay = graph_of(lambda: ref.substep(iters=p.iters, full=True, stream=sh))
    ref_ms = 1e3 * timed(replay) / steps
    del graph, ref
    e = gpe.Pbf(p, [scenes.REFERENCE_BOX], capacity=len(x))
    e.set_state(x, v, stream=sh)
    eng_ms = 1e3 * timed(lambda: e.step(1, stream=sh)) / steps
    e.close()
    out["pbf_16k"] = {"reference_ms_per_step": ref_ms, "engine_ms_per_step": eng_ms, "speedup": ref_ms / eng_ms}

    ix, iy = np.meshgrid(np.arange(256), np.arange(256), indexing="xy")
    xm = np.stack([40.0 + ix.ravel() * 0.7, 5.0 + iy.ravel() * 0.7], 1) + g.uniform(-0.05, 0.05, (65536, 2))
    vm = g.uniform(-5.0, 5.0, xm.shape)
    Cm = np.zeros((65536, 4))
    F = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), (65536, 1))
    J = np.ones(65536)
    xm, vm, Cm, F, J = (a.astype(np.float32) for a in (xm, vm, Cm, F, J))
    ref = refrun.RefMPM(400 * 1000, (12, 6), cubin=mpm_cubin)
    res = {}
    for label, blocks in (("36_blocks", 36), ("full_gpu", 8 * torch.cuda.get_device_properties(0)
                                                  .multi_processor_count)):
        ref.seed(xm, vm, Cm, F, J)
        graph, replay = graph_of(lambda: ref.substep(0, stream=sh, blocks=blocks))
        res[label] = 1e3 * timed(replay) / steps
        del graph
    del ref
    em = gpe.Mpm(scenes.reference_mpm_params(), capacity=65536)
    em.set_state(xm, vm, Cm, F, J, stream=sh)
    eng_ms = 1e3 * timed(lambda: em.step(1, stream=sh)) / steps
    em.close()
    out["mpm_65k"] = {"reference_ms_per_step_36_blocks": res["36_blocks"],
                      "reference_ms_per_step_full_gpu": res["full_gpu"], "engine_ms_per_step": eng_ms,
                      "speedup_vs_reference_launch_shape": res["36_blocks"] / eng_ms,
                      "speedup_vs_reference_full_gpu": res["full_gpu"] / eng_ms}
    return out


def reference_mpm_leg(timed, stream, steps):
    """The reference's own MLS-MPM kernels (MPM.cu built for sm_103a, a 64 x 64-chunk world, 1028^2 grid
    nodes) against the engine on the same 4,194,304-particle block with the reference's constants (J-EOS
    fluid, dt = 0.032 / 20): the reference substep (clear, P2G, grid, G2P) captured into a CUDA graph at the
    reference's launch shape (36 blocks of 256 threads) and at a full-GPU shape (8 blocks per SM), and
    gpe_mpm_step."""
    import torch

    import gpe
    from gpe import scenes

    cubin = ROOT / "oracle" / "_ref" / "MPM_ref_64x64_n4194304.cubin"
    if not cubin.exists():
        return {"unavailable": "reference kernels not built (oracle/build_ref.py needs the reference sources)"}
    from oracle import refrun

    side = 2048
    g = np.random.default_rng(31)
    ix, iy = np.meshgrid(np.arange(side), np.arange(side), indexing="xy")
    x = np.stack([100.0 + ix.ravel() * 0.6, 100.0 + iy.ravel() * 0.6], 1) + g.uniform(-0.05, 0.05, (side * side, 2))
    n = len(x)
    v = g.uniform(-5.0, 5.0, (n, 2))
    Cm = np.zeros((n, 4))
    F = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), (n, 1))
    J = np.ones(n)
    x, v, Cm, F, J = (a.astype(np.float32) for a in (x, v, Cm, F, J))
    sh = stream.cuda_stream
    ref = refrun.RefMPM(n, (64, 64), cubin=cubin)
    res = {}
    for label, blocks in (("reference_launch_shape", 36), ("full_gpu", 8 * torch.cuda.get_device_properties(0)
                                                             .multi_processor_count)):
        ref.seed(x, v, Cm, F, J)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            ref.substep(0, stream=sh, blocks=blocks)

        def replay():
            with torch.cuda.stream(stream):
                graph.replay()

        res[label] = 1e3 * timed(replay) / steps
        del graph
    del ref
    p = scenes.reference_mpm_params()
    p.nx = p.ny = 64 * 32 // 2 + 4
    p.clamp_hi[0] = p.clamp_hi[1] = 64.0 * 32.0
    e = gpe.Mpm(p, capacity=n)
    e.set_state(x, v, Cm, F, J, stream=sh)
    eng_s = timed(lambda: e.step(1, stream=sh))
    st = e.status()
    e.close()
    return {"workload": "mpm_4m_reference_units", "particles": n, "grid_nodes": p.nx * p.ny,
            "reference_ms_per_step_36_blocks": res["reference_launch_shape"],
            "reference_ms_per_step_full_gpu": res["full_gpu"], "engine_ms_per_step": 1e3 * eng_s / steps,
            "speedup_vs_reference_launch_shape": res["reference_launch_shape"] / (1e3 * eng_s / steps),
            "speedup_vs_reference_full_gpu": res["full_gpu"] / (1e3 * eng_s / steps), "engine_status": st}


def render_leg(args, stream, flush_l2, eng):
    """The headless splat rasteriser on the 1M-particle state: published into a 4 x 4-chunk view and drawn
    into a 2048 x 2048 RGBA8 image (100 pixels per metre), timed per frame (publish + draw) like the
    headline. Algorithmic bytes per frame: particles read by the publish (16 B) and written to the view
    (16 B), view positions read by the splat pass (8 B); per pixel the centre counts zeroed and read (4 + 4 B)
    and the image written (4 B). The one atomic per particle lands on the 16 MB count image in L2."""
    import torch

    import gpe

    sh = stream.cuda_stream
    n = eng.n
    cx = cy = 4
    dim, cap = 5.12, 1 << 18  # a chunk of 5.12 m holds 512 x 512 atoms at 0.01 m spacing
    vp = torch.empty((cx * cy * cap, 2), dtype=torch.float32, device="cuda")
    vv = torch.empty_like(vp)
    vc = torch.zeros(cx * cy, dtype=torch.int32, device="cuda")
    view = gpe.View(vp.data_ptr(), vv.data_ptr(), vc.data_ptr(), cx, cy, dim, cap)
    W = H = 2048
    img = torch.empty((H, 4 * W), dtype=torch.uint8, device="cuda")
    cov = torch.empty((H, W), dtype=torch.int32, device="cuda")
    r = gpe.Raster(img.data_ptr(), 4 * W, W, H, 100.0, dim, cov.data_ptr())

    def frame():
        eng.publish(view, stream=sh)
        gpe.render_frame(r, view, stream=sh)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in ev:
        flush_l2()
        a.record(stream)
        frame()
        b.record(stream)
    torch.cuda.synchronize()
    s = sum(a.elapsed_time(b) for a, b in ev) / 1e3 / args.steps
    bytes_frame = 40.0 * n + (4 + 4 + 4) * W * H
    peak, _ = peaks()
    return {"workload": "render_1m_2048x2048", "particles": n, "pixels": W * H, "ms_per_frame": 1e3 * s,
            "pixels_per_s": W * H / s, "particles_per_s": n / s, "alg_bytes_per_frame": bytes_frame,
            "effective_gbs": bytes_frame / s / 1e9, "hbm_frac": bytes_frame / s / 1e9 / peak}


def batched_leg(args, stream, flush_l2):
    """Batched PBF: 256 independent dam-break scenes, particle counts log-uniform in [2048, 65536] (seed 3),
    box aspect U(0.5, 2), C0 physics at dt = 1/480, 4 iterations, all scenes in one engine; timed with the
    default tuning, with the autotuner's choice (cell size, block size, persistent solve) and with the two
    persistent forms at the chosen cell size, block size and mask skin."""
    import torch

    import gpe
    from gpe import scenes

    sh = stream.cuda_stream
    p, pos, vel, dom, boxes = scenes.batched_workload(iters=4)
    n = len(pos)
    e = gpe.Pbf(p, boxes, capacity=n)

    def timed():
        e.set_state(pos, vel, dom, stream=sh)
        for _ in range(args.warmup):
            e.step(1, stream=sh)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in ev:
            flush_l2()
            a.record(stream)
            e.step(1, stream=sh)
            b.record(stream)
        torch.cuda.synchronize()
        s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
        return {"value": n * args.steps / s, "ms_per_step": 1e3 * s / args.steps, "status": e.status()}

    default = timed()
    if args.no_autotune:  # (for profiler launch lists) the default tuning stands in for the tuner's choice
        best, trial_ms, tune_s = e.tuning(), -1.0, 0.0
        tuned = default
    else:
        e.set_state(pos, vel, dom, stream=sh)
        t0 = time.perf_counter()
        best, trial_ms = e.autotune(trial_steps=4, stream=sh)
        tune_s = time.perf_counter() - t0
        tuned = timed()
    # the persistent forms at the tuned cell, block and skin: all passes of a step in one cooperative launch
    # (after the sort's launches), and the whole step in one
    persistent = {}
    for mode, name in ((1, "solve"), (2, "whole_step")):
        e.set_tuning(cell=best.cell, block=best.block, persistent=mode, skin=best.skin)
        persistent[name] = timed()
    e.close()
    return {"workload": "pbf_batched_256_scenes", "scenes": 256, "particles": n, "unit": "particle-steps/s",
            "default": default, "tuned": tuned, "persistent": persistent,
            "tuning": {"cell_over_h": best.cell / p.h, "block": best.block, "persistent": int(best.persistent),
                       "skin": round(best.skin, 3),
                       "trial_ms_per_step": trial_ms, "autotune_s": tune_s}}


def mpm_warmup(steps, sort_interval):
    """Untimed steps before an MLS-MPM engine is timed. The engine keeps one CUDA graph per grid rotation
    (3), state buffer (2, swapped by each re-sort) and sort / no sort; stepping one at a time, all of them
    are captured within six re-sort intervals, so warming up over those keeps graph capture out of the
    timed steps."""
    return max(steps, 6 * sort_interval) if sort_interval > 0 else steps


def mpm_leg(args, stream, flush_l2):
    """MLS-MPM, timed like the headline (graph-launched steps, L2 flushed before each):
    mixed: 4,194,304 particles (a third each of water, snow and jelly in seeded discs) on a 1024^2 grid,
           dt = 5e-5, spatial re-sort every 32 steps; algorithmic bytes 136 per particle (x, v, C, F, J,
           material and plastic state read and written once) plus 64 per grid node;
    library: the same grid and particle count with a fifth each of water, jelly, snow, Neo-Hookean and
           Drucker-Prager sand (two discs each);
    elastic: 65,536 fixed-corotated particles in two squares on a 128^2 grid (32 per cell), dt = 1e-4,
           re-sorted every 16 steps (launch-bound);
    batched_32: 32 mixed scenes of 64k-512k particles in one engine (batched_mpm).
    Each scene is timed over at least one re-sort interval of steps (so the re-sort's cost enters the mean at
    its own frequency) and at least --steps steps."""
    import torch

    import gpe
    from gpe import scenes

    sh = stream.cuda_stream
    peak, _ = peaks()

    def timed(p, pos, vel, mat, alg_bytes, scene_list=None, sid=None):
        n = len(pos)
        e = gpe.Mpm(p, capacity=n, scenes=scene_list)
        e.set_state(pos, vel, material=mat, stream=sh, scene_id=sid)
        for _ in range(mpm_warmup(args.warmup, p.sort_interval)):
            e.step(1, stream=sh)
        torch.cuda.synchronize()
        steps = max(args.steps, p.sort_interval)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in ev:
            flush_l2()
            a.record(stream)
            e.step(1, stream=sh)
            b.record(stream)
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in ev]
        s = sum(ms) / 1e3
        st = e.status()
        launches = e.launches_per_step()
        e.close()
        gbs = alg_bytes * steps / s / 1e9
        return {"particles": n, "value": n * steps / s, "unit": "particle-steps/s", "steps": steps,
                "sort_interval": p.sort_interval, "ms_per_step": 1e3 * s / steps, "alg_bytes_per_step": alg_bytes,
                "effective_gbs": gbs, "hbm_frac": gbs / peak, "launches_per_step": launches, "status": st,
                # the step that re-sorts is the slowest; the median is a step between re-sorts
                "ms_step_median": float(np.median(ms)), "ms_step_max": max(ms)}

    out = {}
    n = 4194304
    p = scenes.mixed_params(n)
    pos, mat = scenes.mixed_discs(n)
    out["mixed_4m"] = timed(p, pos, np.zeros_like(pos), mat, 136.0 * n + 64.0 * p.nx * p.ny)
    # the whole constitutive library in one scene: water, jelly (corotated), snow, Neo-Hookean and sand
    lib = (gpe.MPM_MAT_FLUID, gpe.MPM_MAT_COROTATED, gpe.MPM_MAT_SNOW, gpe.MPM_MAT_NEOHOOKEAN, gpe.MPM_MAT_SAND)
    pos, mat = scenes.mixed_discs(n, seed=5, discs_per_material=2, materials=lib)
    out["library_4m"] = timed(p, pos, np.zeros_like(pos), mat, 136.0 * n + 64.0 * p.nx * p.ny)
    pe, pos, vel = scenes.elastic_workload()
    out["elastic_65k"] = timed(pe, pos, vel, None, 120.0 * len(pos) + 64.0 * pe.nx * pe.ny)
    out["batched_32"] = batched_mpm(timed, sh, stream)
    return out


def batched_mpm(timed, sh, stream):
    """32 mixed-material scenes of 64k-512k particles (log-uniform, seed 6), each on its own square grid at
    the 4M scene's particle density, in one engine (one set of launches per step over all scenes); beside
    it the same scenes as 32 engines stepped one after the other on the stream."""
    import torch

    import gpe
    from gpe import scenes

    p, sc, pos, mat, sid = scenes.mixed_batch()
    table = [gpe.make_mpm_scene(*s) for s in sc]
    nodes = sum(s[0] * s[1] for s in sc)
    n = len(pos)
    r = timed(p, pos, np.zeros_like(pos), mat, 136.0 * n + 64.0 * nodes, scene_list=table, sid=sid)
    r.update({"scenes": len(sc), "nodes": nodes})
    solo = []
    for q, s in enumerate(sc):
        ps = p.copy()
        ps.nx, ps.ny = s[0], s[1]
        ps.clamp_lo[0], ps.clamp_lo[1] = s[2]
        ps.clamp_hi[0], ps.clamp_hi[1] = s[3]
        sel = sid == q
        e = gpe.Mpm(ps, capacity=int(sel.sum()))
        e.set_state(pos[sel], np.zeros_like(pos[sel]), material=mat[sel], stream=sh)
        solo.append(e)
    for _ in range(mpm_warmup(3, p.sort_interval)):
        for e in solo:
            e.step(1, stream=sh)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(10, p.sort_interval)  # one re-sort interval, as the batched engine is timed
    a.record(stream)
    for _ in range(reps):
        for e in solo:
            e.step(1, stream=sh)
    b.record(stream)
    torch.cuda.synchronize()
    r["solo_engines_ms_per_step"] = a.elapsed_time(b) / reps
    for e in solo:
        e.close()
    return r


def run_reference(args, rank, ws):
    if rank != 0:
        return
    p, pos, vel, boxes, cfg = workload()
    from oracle import pyoracle

    o = pyoracle.PbfOracle(p, boxes)
    x, v = pos, vel
    for _ in range(args.warmup):
        r = o.step(x, v, None, 1)
        x, v = r["x"], r["v"]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = o.step(x, v, None, 1)
        x, v = r["x"], r["v"]
    dt = time.perf_counter() - t0
    val = len(pos) * args.steps / dt
    line = {"metric": "pbf_particle_steps_per_s_1m", "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": pyoracle.num_threads(),
                             "kind": "port",
                             "sample": f"{args.steps} full steps of the {len(pos)}-particle workload; the "
                                       "reference has no CPU solver, so its FP64 restatement stands in"},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpe(args, rank, ws):
    import torch

    import gpe

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    p, pos, vel, boxes, cfg = workload()
    n = len(pos)
    eng = gpe.Pbf(p, boxes, capacity=n)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    # pinned host buffers for the end-to-end leg
    h_pos = torch.from_numpy(pos).pin_memory()
    h_vel = torch.from_numpy(vel).pin_memory()
    o_pos = torch.empty((n, 2), dtype=torch.float32).pin_memory()
    o_vel = torch.empty((n, 2), dtype=torch.float32).pin_memory()

    eng.set_state(pos, vel, stream=sh)
    # the engine's autotuner picks cell size, block size, persistent solve and mask skin for this scene (it
    # restores the state afterwards); untimed. Its trials run consecutive steps without an L2 flush, as a
    # simulation loop does; the timed steps below flush L2 before each step, and under that protocol its
    # choice can trail another candidate by about 1% (skin 0.1 h against 0.075 h at 1M particles).
    # --no-autotune keeps the engine's default tuning (for profiler launch lists, which would otherwise fill
    # with the tuner's trials)
    if args.no_autotune:
        best = eng.tuning()
    else:
        best, _ = eng.autotune(trial_steps=3, stream=sh)
    cfg["tuning"] = {"cell_over_h": round(best.cell / p.h, 3), "block": best.block,
                     "persistent": int(best.persistent), "skin": round(best.skin, 3)}
    for _ in range(args.warmup):
        eng.step(1, stream=sh)
    torch.cuda.synchronize()

    # ---- timed region: graph-launched steps ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        for a, b in ev:
            flush_l2()
            a.record(stream)
            eng.step(1, stream=sh)
            b.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1e3
    value = replica_value(n * args.steps, total_s, ws)
    dmax, dmean = eng.density_error(stream=sh)
    launches = eng.launches_per_step()

    # ---- stage-by-stage pass for the per-kernel roofline ----
    stage_ms = {k: [] for k in ALG_BYTES}
    # the sort stage's launches: the step's, less one λ and one Δp per iteration and the XSPH pass, plus the
    # predict + histogram kernel that the stage API runs (inside a run of steps the previous XSPH does its work)
    stage_launches = {"predict_sort": launches - 2 * p.iters - 1 + (1 if p.vort_eps == 0.0 else 0), "lambda": 1,
                      "delta_p": 1, "xsph": 1}
    for _ in range(args.steps):
        flush_l2()
        seq = [("predict_sort", gpe.PBF_STAGE_PREDICT_SORT)]
        for _ in range(p.iters):
            seq += [("lambda", gpe.PBF_STAGE_LAMBDA), ("delta_p", gpe.PBF_STAGE_DELTA_P)]
        seq += [("xsph", gpe.PBF_STAGE_XSPH)]
        evs = []
        for name, st in seq:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.stage(st, stream=sh)
            b.record(stream)
            evs.append((name, a, b))
        eng.stage(gpe.PBF_STAGE_FINISH, stream=sh)
        torch.cuda.synchronize()
        for name, a, b in evs:
            stage_ms[name].append(a.elapsed_time(b))
    share = {k: sum(v) for k, v in stage_ms.items()}
    tot = sum(share.values())
    dom_name = max(share, key=lambda k: share[k])
    per_launch_ms = statistics.mean(stage_ms[dom_name]) / stage_launches[dom_name]
    peak, peak_kind = peaks()
    achieved = ALG_BYTES[dom_name] * n / (per_launch_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": {"lambda": "k_lambda", "delta_p": "k_delta_p", "xsph": "k_xsph",
                                           "predict_sort": "sort group"}[dom_name],
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": NCU_TRAFFIC.get(dom_name),
                "alg_bytes_per_launch": ALG_BYTES[dom_name] * n, "launch_ms": per_launch_ms,
                "share": {k: v / tot for k, v in share.items()},
                "stage_ms_per_step": {k: statistics.mean(v) for k, v in stage_ms.items()},
                # every stage's algorithmic bytes (per pass; the sort stage's for its whole group of launches)
                # over its time, and that against the peak
                "stage_gbs": {k: ALG_BYTES[k] * n / (statistics.mean(v) / 1e3) / 1e9 for k, v in stage_ms.items()},
                "stage_frac": {k: ALG_BYTES[k] * n / (statistics.mean(v) / 1e3) / 1e9 / peak
                               for k, v in stage_ms.items()}}
    if dom_name in NCU_WARP_INST:
        sm_mhz = clk.summary().get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        issue_peak = 4.0 * sms * sm_mhz * 1e6
        issue = NCU_WARP_INST[dom_name] / (per_launch_ms / 1e3)
        roofline["issue"] = {"warp_inst_per_launch": NCU_WARP_INST[dom_name], "achieved": issue, "peak": issue_peak,
                             "unit": "warp-instructions/s", "frac": issue / issue_peak,
                             "how": "ncu smsp__inst_executed.sum per launch over the live launch time; peak = 4 "
                                    "schedulers x SMs x the median SM clock sampled in the timed region"}

    # ---- end to end through the C ABI with host buffers ----
    # The host holds the simulation state: every step copies in the state the host received from the
    # previous step and copies out the new one, as a caller that keeps its particles in host memory does.
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    eng.get_state(o_pos.numpy(), o_vel.numpy(), stream=sh)  # the state after the timed steps (untimed)
    for a, b in e2e_ev:
        flush_l2()
        a.record(stream)
        eng.set_state(o_pos.numpy(), o_vel.numpy(), stream=sh)
        eng.step(1, stream=sh)
        eng.get_state(o_pos.numpy(), o_vel.numpy(), stream=sh)
        b.record(stream)
    torch.cuda.synchronize()
    e2e_s = sum(a.elapsed_time(b) for a, b in e2e_ev) / 1e3
    e2e_seq = {"value": replica_value(n * args.steps, e2e_s, ws), "unit": "particle-steps/s",
               "how": "one engine on one stream: copy in the host's state, step, copy the new state out "
                      "(synchronous), per step"}

    # E2E_ENGINES engines on as many streams, step s on engine s % E2E_ENGINES with page-locked buffers
    # (GPE_MEM_PINNED: the copies are asynchronous), so one step's copies overlap the other engines' steps;
    # every step still copies its 16 MB in and its 16 MB out inside the timed region. Each engine continues
    # its own simulation from its host buffer (copy in the host's state, step, copy the new state back into
    # that buffer). No L2 flush: the engines' working sets (about 130 MB each) alternate through the 129 MB L2.
    engines = [eng] + [gpe.Pbf(p, boxes, capacity=n) for _ in range(E2E_ENGINES - 1)]
    for e_ in engines[1:]:
        e_.set_tuning(cell=best.cell, block=best.block, persistent=int(best.persistent), skin=best.skin)
    streams = [stream] + [torch.cuda.Stream() for _ in range(E2E_ENGINES - 1)]
    outs = [(o_pos, o_vel)] + [(torch.empty((n, 2), dtype=torch.float32).pin_memory(),
                                torch.empty((n, 2), dtype=torch.float32).pin_memory())
                               for _ in range(E2E_ENGINES - 1)]
    for q in range(E2E_ENGINES):  # untimed: each engine's graph, and warm-up steps through the host buffers
        engines[q].set_state(h_pos, h_vel, stream=streams[q].cuda_stream)
        engines[q].step(1, stream=streams[q].cuda_stream)
        engines[q].get_state(outs[q][0], outs[q][1], stream=streams[q].cuda_stream)
        for _ in range(args.warmup):
            engines[q].set_state(outs[q][0], outs[q][1], stream=streams[q].cuda_stream)
            engines[q].step(1, stream=streams[q].cuda_stream)
            engines[q].get_state(outs[q][0], outs[q][1], stream=streams[q].cuda_stream)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(streams[0])
    for st_ in streams[1:]:
        st_.wait_event(t0)
    h0 = time.perf_counter()
    for s_ in range(args.steps):
        q = s_ % E2E_ENGINES
        st_ = streams[q].cuda_stream
        engines[q].set_state(outs[q][0], outs[q][1], stream=st_)
        engines[q].step(1, stream=st_)
        engines[q].get_state(outs[q][0], outs[q][1], stream=st_)
    host_s = time.perf_counter() - h0  # the host's time to issue the steps (the calls return before the GPU)
    for st_ in streams[1:]:
        j_ = torch.cuda.Event()
        j_.record(st_)
        streams[0].wait_event(j_)
    t1.record(streams[0])
    torch.cuda.synchronize()
    e2e_pipe_s = t0.elapsed_time(t1) / 1e3
    for e_ in engines[1:]:
        e_.close()
    e2e = {"value": replica_value(n * args.steps, e2e_pipe_s, ws), "unit": "particle-steps/s",
           "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n,
           "how": f"{E2E_ENGINES} engines on {E2E_ENGINES} streams, page-locked host buffers, asynchronous "
                  "copies: one step's copies overlap the other engines' steps; each engine continues its "
                  "simulation from the state in its host buffer; no L2 flush: between two steps of one engine "
                  "the other engines' steps stream about 260 MB through the 129 MB L2",
           "host_issue_ms_per_step": 1e3 * host_s / args.steps, "sequential": e2e_seq}

    if rank != 0:
        return
    base = None
    if ws == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(p, pos, vel, boxes)
    render = None
    if ws == 1 and not args.no_render:
        try:
            render = render_leg(args, stream, flush_l2, eng)
        except Exception as exc:  # reported, never fatal to the headline number
            render = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
    eng.close()
    learned = None
    if ws == 1 and not args.no_learned:
        try:
            learned = learned_leg(args, stream, flush_l2)
            plain4 = n * args.steps / total_s
            learned["speedup_vs_plain_k4"] = learned["value"] / plain4
            # the network's multiplier with one delta p pass against the plain 4-iteration form, and whether
            # it reaches that form's own max density error
            k1 = learned["network_k1"]
            learned["network_k1"]["speedup_vs_plain_k4"] = k1["value"] / plain4
            learned["network_k1"]["error_le_plain_k4"] = k1["density_error"]["max"] <= dmax
            learned["target"] = {"density_error_max_le_1pct": learned["density_error"]["max"] <= 0.01,
                                 "speedup_ge_2x": learned["speedup_vs_plain_k4"] >= 2.0}
        except Exception as exc:  # reported, never fatal to the headline number
            learned = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
    batched = None
    if ws == 1 and not args.no_batched:
        try:
            batched = batched_leg(args, stream, flush_l2)
        except Exception as exc:  # reported, never fatal to the headline number
            batched = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
    mpm = None
    if ws == 1 and not args.no_mpm:
        try:
            mpm = mpm_leg(args, stream, flush_l2)
        except Exception as exc:  # reported, never fatal to the headline number
            mpm = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
    ref_cuda = None
    if ws == 1 and not args.no_reference_cuda:
        try:
            ref_cuda = reference_cuda_leg(args, stream, flush_l2)
        except Exception as exc:  # reported, never fatal to the headline number
            ref_cuda = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}
    ms = 1e3 * ws * n / value  # the slowest rank's time per step
    line = {"metric": "pbf_particle_steps_per_s_1m", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg, "e2e": e2e, "roofline": roofline, "cpu_baseline": base,
            "gpu_launches": launches * args.steps, "launches_per_step": launches,
            "hbm_effective_gbs": 212.0 * value / ws / 1e9,
            "density_error": {"max": dmax, "mean": dmean}, "clocks": clk.summary(),
            "learned": learned, "batched": batched, "mpm": mpm, "render": render, "reference_cuda": ref_cuda}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpe", choices=["gpe", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-cuda", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-mpm", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, ws = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
    else:
        run_gpe(args, rank, ws)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
