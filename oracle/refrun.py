"""Runs the reference's own PBF and MLS-MPM kernels (libs/cuda-engine/source/PBF.cu, MPM.cu), built headless
as cubins by oracle/build_ref.py, through the CUDA driver API. TEST INFRASTRUCTURE: the parity tests and the
reference-CUDA timing leg of bench.py use it as the checker; the engine never calls it.

The reference builds its tick as a CUDA graph (PBF.cu:901-961, MPM.cu:326-374); this runner issues the same
kernels with the same launch shapes and arguments in the same order, restated from those two functions.
Device buffers are torch tensors laid out like the reference's arenas (cuda-engine.cpp:102-171).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"

_cu = None


def cu() -> C.CDLL:
    global _cu
    if _cu is None:
        L = C.CDLL("libcuda.so.1")
        L.cuInit(0)
        _cu = L
    return _cu


def _chk(rc: int, what: str) -> None:
    if rc != 0:
        name = C.c_char_p()
        cu().cuGetErrorName(rc, C.byref(name))
        raise RuntimeError(f"{what}: CUDA driver error {rc} {name.value}")


class Float2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class Int2(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32)]


class View(C.Structure):  # cuda-engine.h:51-57
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("num_atoms", C.c_void_p), ("slot", C.c_int32)]


class Module:
    """A loaded cubin with its __global__ functions looked up by their source names."""

    def __init__(self, path: Path):
        import torch

        torch.zeros(1, device="cuda")  # make the runtime's primary context current on this thread
        self.mod = C.c_void_p()
        _chk(cu().cuModuleLoad(C.byref(self.mod), str(path).encode()), f"cuModuleLoad({path})")
        cnt = C.c_uint()
        _chk(cu().cuModuleGetFunctionCount(C.byref(cnt), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * cnt.value)()
        _chk(cu().cuModuleEnumerateFunctions(funcs, cnt, self.mod), "cuModuleEnumerateFunctions")
        self.by_name = {}
        for f in funcs:
            nm = C.c_char_p()
            _chk(cu().cuFuncGetName(C.byref(nm), C.c_void_p(f)), "cuFuncGetName")
            self.by_name[nm.value.decode()] = C.c_void_p(f)

    def fn(self, name: str) -> C.c_void_p:
        tag = f"{len(name)}{name}"  # Itanium mangling of a free function: _Z<len><name><params>
        hits = [f for n, f in self.by_name.items() if n.startswith("_Z" + tag)]
        if len(hits) != 1:
            raise KeyError(f"kernel {name}: {len(hits)} matches")
        return hits[0]

    def set_global(self, name: str, struct) -> None:
        dptr, size = C.c_void_p(), C.c_size_t()
        _chk(cu().cuModuleGetGlobal_v2(C.byref(dptr), C.byref(size), self.mod, name.encode()),
             f"cuModuleGetGlobal({name})")
        assert size.value == C.sizeof(struct), (name, size.value, C.sizeof(struct))
        _chk(cu().cuMemcpyHtoD_v2(dptr, C.byref(struct), C.c_size_t(C.sizeof(struct))), f"upload {name}")


def launch(f, grid, block, args, stream=0, smem=0) -> None:
    holders = []
    for a in args:
        holders.append(a if isinstance(a, C._SimpleCData) or isinstance(a, C.Structure) else C.c_void_p(a))
    argv = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
    g = tuple(grid) + (1,) * (3 - len(grid))
    b = tuple(block) + (1,) * (3 - len(block))
    _chk(cu().cuLaunchKernel(f, g[0], g[1], g[2], b[0], b[1], b[2], smem, C.c_void_p(stream), argv, None),
         "cuLaunchKernel")


def _p(t) -> int:
    return t.data_ptr()


# ===================================================================================================== PBF
class RefPBF:
    """The reference PBF solver for a kSceneDimX x kSceneDimY chunk world (constants fixed at build time)."""

    MAX_ATOMS, GRID, SLOTS, CHUNK = 1536, 16, 8, 32.0
    HALO_CELLS = 4 * 16 + 4
    HALO_ATOMS = HALO_CELLS * 8

    def __init__(self, scene=(12, 6), migrants=320, cubin=None):
        import torch

        self.sx, self.sy = scene
        self.mig = migrants
        path = cubin or REF_DIR / f"PBF_ref_{self.sx}x{self.sy}_m{migrants}.cubin"
        self.m = Module(path)
        self.k = {n: self.m.fn(n) for n in ("haloKernel", "lambdaKernel", "posCorrectionKernel", "velocityKernel",
                                             "XSPHKernel", "migrationKernel", "prepNextSubstepKernel",
                                             "PBFOutputKernel")}
        nc = self.sx * self.sy
        ext = (self.sx + 2) * (self.sy + 2)
        dev = "cuda"
        z = lambda *shape, dt=torch.float32: torch.zeros(*shape, dtype=dt, device=dev)  # noqa: E731
        self.offsets = z(nc * 256, dt=torch.int32)
        self.pos = [z(nc * self.MAX_ATOMS, 2), z(nc * self.MAX_ATOMS, 2)]
        self.vel = z(nc * self.MAX_ATOMS, 2)
        self.lam = z(nc * self.MAX_ATOMS)
        self.num_atoms = z(nc, dt=torch.int32)
        self.mig_pos = z(ext * migrants, 2)
        self.mig_vel = z(ext * migrants, 2)
        self.mig_count = z(ext, dt=torch.int32)
        self.halo_offsets = z(nc * self.HALO_CELLS, dt=torch.int32)
        self.halo_pos = [z(nc * self.HALO_ATOMS, 2), z(nc * self.HALO_ATOMS, 2)]
        self.halo_vel = z(nc * self.HALO_ATOMS, 2)
        self.halo_lambda = z(nc * self.HALO_ATOMS)
        self.out_pos = z(nc * self.MAX_ATOMS, 2)
        self.out_vel = z(nc * self.MAX_ATOMS, 2)
        self.out_num = z(nc, dt=torch.int32)
        self.m.set_global("c_torus", Int2(0, 0))
        self.m.set_global("c_output", View(_p(self.out_pos), _p(self.out_vel), _p(self.out_num), 1))

    # ----- seeding: the state the reference holds after prepNextSubstepKernel (PBF.cu:806-833) -----
    def seed(self, x: np.ndarray, v: np.ndarray, g_step: float):
        """x, v absolute (dt = 1 units). Places each atom in the chunk of its prediction x* = x + v + g, sorted
        by local cell (stable). Returns (chunk, slot) of every input atom."""
        import torch

        x = np.asarray(x, np.float32)
        v = np.asarray(v, np.float32)
        xs = (x + v).astype(np.float32)
        xs[:, 1] = (xs[:, 1] + np.float32(g_step)).astype(np.float32)
        cx = np.clip(np.floor(xs[:, 0] / self.CHUNK).astype(np.int64), 0, self.sx - 1)
        cy = np.clip(np.floor(xs[:, 1] / self.CHUNK).astype(np.int64), 0, self.sy - 1)
        chunk = cx + cy * self.sx
        org = np.stack([cx, cy], 1).astype(np.float32) * np.float32(self.CHUNK)
        xl = (x - org).astype(np.float32)
        xsl = (xs - org).astype(np.float32)
        gx = np.clip(np.floor(xsl[:, 0]).astype(np.int64) // 2, 0, 15)
        gy = np.clip(np.floor(xsl[:, 1]).astype(np.int64) // 2, 0, 15)
        cell = gx + 16 * gy
        order = np.lexsort((np.arange(len(x)), cell, chunk))
        nc = self.sx * self.sy
        counts = np.bincount(chunk, minlength=nc)
        if counts.max() > self.MAX_ATOMS:
            raise ValueError("a chunk exceeds kMaxAtoms")
        first = np.concatenate([[0], np.cumsum(counts)[:-1]])
        slot = np.empty(len(x), np.int64)
        slot[order] = np.arange(len(x)) - first[chunk[order]]
        idx = chunk * self.MAX_ATOMS + slot
        P0 = np.zeros((nc * self.MAX_ATOMS, 2), np.float32)
        P1 = np.zeros_like(P0)
        P0[idx] = xl
        P1[idx] = xsl
        offs = np.zeros((nc, 256), np.uint32)
        cc = np.zeros((nc, 256), np.int64)
        np.add.at(cc, (chunk, cell), 1)
        ends = np.cumsum(cc, 1)
        starts = ends - cc
        offs[:] = ((ends << 16) | starts).astype(np.uint32)
        self.pos[0].copy_(torch.from_numpy(P0))
        self.pos[1].copy_(torch.from_numpy(P1))
        self.vel.zero_()
        self.offsets.copy_(torch.from_numpy(offs.view(np.int32).ravel()))
        self.num_atoms.copy_(torch.from_numpy(counts.astype(np.int32)))
        self.halo_offsets.zero_()
        self.mig_count.zero_()
        self.chunk, self.slot, self.idx = chunk, slot, idx
        return chunk, slot

    # ----- one substep as in PBF.cu:921-955 -----
    def substep(self, iters=2, full=True, stream=0):
        sx, sy = self.sx, self.sy
        k = self.k
        slot = 0
        launch(k["haloKernel"], ((sx + 1) // 2, sy), (128, 2),
               [_p(self.offsets), _p(self.pos[1]), _p(self.halo_offsets), _p(self.halo_pos[slot]),
                _p(self.num_atoms)], stream)
        for _ in range(iters):
            launch(k["lambdaKernel"], (sx, sy), (512,),
                   [_p(self.offsets), _p(self.pos[1]), _p(self.lam), _p(self.halo_offsets), _p(self.halo_pos[slot]),
                    _p(self.halo_lambda), _p(self.num_atoms)], stream)
            launch(k["posCorrectionKernel"], (sx, sy), (512,),
                   [_p(self.offsets), _p(self.pos[1]), _p(self.lam), _p(self.halo_offsets),
                    _p(self.halo_pos[slot]), _p(self.halo_pos[slot ^ 1]), _p(self.halo_lambda),
                    _p(self.num_atoms)], stream)
            slot ^= 1
        launch(k["velocityKernel"], (sx, sy), (512,),
               [_p(self.offsets), _p(self.pos[0]), _p(self.pos[1]), _p(self.vel), _p(self.halo_vel),
                _p(self.num_atoms)], stream)
        launch(k["XSPHKernel"], (sx, sy), (1024,),
               [_p(self.offsets), _p(self.pos[1]), _p(self.vel), _p(self.halo_offsets), _p(self.halo_pos[slot]),
                _p(self.halo_vel), _p(self.num_atoms)], stream)
        if not full:
            return
        self.migrate(stream)
        self.prep(stream)

    def migrate(self, stream=0):
        """The migration half of a substep's tail (PBF.cu:947-950): halo offsets cleared, then atoms whose next
        prediction leaves their chunk queued for the destination chunk."""
        _chk(cu().cuMemsetD32Async(C.c_void_p(_p(self.halo_offsets)), 0, self.halo_offsets.numel(),
                                   C.c_void_p(stream)), "memset halo_offsets")
        launch(self.k["migrationKernel"], (self.sx, self.sy), (512,),
               [_p(self.pos[1]), _p(self.vel), _p(self.num_atoms), _p(self.mig_pos), _p(self.mig_vel),
                _p(self.mig_count)], stream)

    def prep(self, stream=0):
        """prepNextSubstepKernel (PBF.cu:951-954): queues drained, next prediction, per-chunk cell sort."""
        launch(self.k["prepNextSubstepKernel"], (self.sx, self.sy), (256,),
               [_p(self.offsets), _p(self.pos[0]), _p(self.pos[1]), _p(self.vel), _p(self.num_atoms),
                _p(self.mig_pos), _p(self.mig_vel), _p(self.mig_count)], stream)

    def read_sorted(self):
        """Every atom after prepNextSubstepKernel, chunk by chunk in the reference's (atomic-order) sorted
        order: (global cell index in the scene's row-major grid of 16 x 16-cell chunks, x, x*), absolute."""
        import torch

        torch.cuda.synchronize()
        num = self.num_atoms.cpu().numpy()
        offs = self.offsets.cpu().numpy().view(np.uint32).reshape(self.sx * self.sy, 256)
        P0 = self.pos[0].cpu().numpy().reshape(self.sx * self.sy, self.MAX_ATOMS, 2)
        P1 = self.pos[1].cpu().numpy().reshape(self.sx * self.sy, self.MAX_ATOMS, 2)
        cells, xs_, x_ = [], [], []
        ncx = self.sx * self.GRID
        for c in range(self.sx * self.sy):
            n = int(num[c])
            if n == 0:
                continue
            start = offs[c] & 0xFFFF
            end = offs[c] >> 16
            if int(end[-1]) != n:
                raise RuntimeError(f"chunk {c}: cell offsets end at {int(end[-1])}, not at its {n} atoms")
            local = np.repeat(np.arange(256), (end - start).astype(np.int64))
            gx = (c % self.sx) * self.GRID + local % self.GRID
            gy = (c // self.sx) * self.GRID + local // self.GRID
            org = np.array([(c % self.sx) * self.CHUNK, (c // self.sx) * self.CHUNK], np.float32)
            cells.append(gy * ncx + gx)
            x_.append(P0[c, :n] + org)
            xs_.append(P1[c, :n] + org)
        return (np.concatenate(cells).astype(np.uint32), np.concatenate(x_).astype(np.float32),
                np.concatenate(xs_).astype(np.float32))

    def output(self, stream=0):
        launch(self.k["PBFOutputKernel"], (self.sx, self.sy), (256,),
               [_p(self.pos[0]), _p(self.vel), _p(self.num_atoms)], stream)

    def read_seeded(self):
        """x*, v, lambda of the seeded atoms in input order (valid after substep(full=False)), absolute."""
        import torch

        torch.cuda.synchronize()
        P1 = self.pos[1].cpu().numpy()
        V = self.vel.cpu().numpy()
        L = self.lam.cpu().numpy()
        cx = (self.chunk % self.sx).astype(np.float32)
        cy = (self.chunk // self.sx).astype(np.float32)
        org = np.stack([cx, cy], 1) * np.float32(self.CHUNK)
        return (P1[self.idx] + org).astype(np.float32), V[self.idx], L[self.idx]


# ===================================================================================================== MPM
class RefMPM:
    def __init__(self, n_atoms=400 * 1000, scene=(12, 6), cubin=None):
        import torch

        self.sx, self.sy = scene
        self.cap = n_atoms
        path = cubin or REF_DIR / f"MPM_ref_{self.sx}x{self.sy}_n{n_atoms}.cubin"
        self.m = Module(path)
        self.k = {n: self.m.fn(n) for n in ("resetGridKernel", "P2GKernel", "gridKernel", "G2PKernel")}
        self.gx = self.sx * 32 // 2 + 4
        self.gy = self.sy * 32 // 2 + 4
        z = lambda *shape, dt=torch.float32: torch.zeros(*shape, dtype=dt, device="cuda")  # noqa: E731
        self.grid = [z(self.gx * self.gy, 4), z(self.gx * self.gy, 4)]
        self.pos = z(n_atoms, 2)
        self.vel = z(n_atoms, 2)
        self.C = z(n_atoms, 4)
        self.F = z(n_atoms, 4)
        self.J = z(n_atoms)
        self.num_points = z(2, dt=torch.int32)
        self.m.set_global("c_torus", Int2(0, 0))

    def seed(self, x, v, Cm, F, J):
        import torch

        n = len(x)
        for t, a in ((self.pos, x), (self.vel, v), (self.C, Cm), (self.F, F)):
            t[:n].copy_(torch.from_numpy(np.ascontiguousarray(a, np.float32)))
        self.J[:n].copy_(torch.from_numpy(np.ascontiguousarray(J, np.float32)))
        self.num_points.copy_(torch.tensor([n, n], dtype=torch.int32))
        self.n = n

    def substep(self, s=0, stream=0, blocks=36):
        """P2G -> grid -> G2P on grid[s & 1] after clearing it (MPM.cu:357-368). blocks: the reference launches
        36 blocks of 256 threads (constants.h); its kernels loop over particles and nodes with a grid stride,
        so any block count gives the same result."""
        BD, GD = (256,), (int(blocks),)
        g = self.grid[s & 1]
        launch(self.k["resetGridKernel"], GD, BD, [_p(g)], stream)
        launch(self.k["P2GKernel"], GD, BD,
               [_p(g), _p(self.pos), _p(self.vel), _p(self.C), _p(self.J), _p(self.num_points)], stream)
        launch(self.k["gridKernel"], GD, BD, [_p(g)], stream)
        launch(self.k["G2PKernel"], GD, BD,
               [_p(g), _p(self.pos), _p(self.vel), _p(self.C), _p(self.F), _p(self.J),
                C.c_size_t(self.sx * 32), C.c_size_t(self.sy * 32), _p(self.num_points)], stream)

    def read(self):
        import torch

        torch.cuda.synchronize()
        n = self.n
        return (self.pos[:n].cpu().numpy(), self.vel[:n].cpu().numpy(), self.C[:n].cpu().numpy(),
                self.F[:n].cpu().numpy(), self.J[:n].cpu().numpy())


# ===================================================================================================== render
class RefRender:
    """The reference's splat renderer (libs/render/source/cuda-render.cu: backgroundKernel and drawKernel, as
    launchFill issues them, :189-211) drawing a chunk-major view into a pitched RGBA8 device buffer instead of
    its D3D12 surface."""

    def __init__(self, cubin=None, scene=(12, 6)):
        self.sx, self.sy = scene
        self.m = Module(cubin or REF_DIR / f"render_ref_{self.sx}x{self.sy}.cubin")
        self.k = {n: self.m.fn(n) for n in ("backgroundKernel", "drawKernel")}

    def render(self, pos, counts, width, height, stream=0):
        import torch

        cap = pos.shape[1]
        d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1, 2)).cuda()
        d_vel = torch.zeros_like(d_pos)
        d_cnt = torch.from_numpy(np.ascontiguousarray(counts, np.int32)).cuda()
        pitch = 4 * width
        img = torch.zeros(height * pitch, dtype=torch.uint8, device="cuda")
        del cap
        sz = C.c_size_t
        launch(self.k["backgroundKernel"], ((width + 31) // 32, (height + 15) // 16), (32, 16),
               [_p(img), sz(pitch), sz(width), sz(height)], stream)
        launch(self.k["drawKernel"], (self.sx, self.sy), (256,),
               [_p(d_pos), _p(d_vel), _p(d_cnt), _p(img), sz(pitch), sz(width), sz(height)], stream)
        torch.cuda.synchronize()
        return img.cpu().numpy().reshape(height, width, 4)

