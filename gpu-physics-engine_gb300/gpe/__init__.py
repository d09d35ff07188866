"""ctypes binding of libgpe.so (include/gpe.h): the host-side handle API of the PBF and MLS-MPM engines.

The library is loaded from the package directory; importing this module fails loudly if it has not been
built (run gpu-physics-engine_gb300/build.py, or __graft_entry__.build()). There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "libgpe.so"

# ----- constants (include/gpe.h) -------------------------------------------------------------------------
OK, ERR_CUDA, ERR_DEVICE, ERR_NOT_READY, ERR_BAD_ARG, ERR_ALREADY, ERR_CAPACITY, ERR_NONFINITE, ERR_TIMEOUT = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)
MEM_HOST, MEM_DEVICE, MEM_PINNED = 0, 1, 2
STATUS_NONFINITE, STATUS_CAPACITY, STATUS_CELL_OVERFLOW, STATUS_TIMEOUT = 1, 2, 4, 8

PBF_SELF_GRAD, PBF_VEL_CLAMP, PBF_TRACK_IDS, PBF_PAIR_IDS, PBF_DYNAMIC_COUNT = 0x1, 0x2, 0x4, 0x8, 0x10
(PBF_STAGE_PREDICT_SORT, PBF_STAGE_LAMBDA, PBF_STAGE_DELTA_P, PBF_STAGE_XSPH, PBF_STAGE_VORTICITY,
 PBF_STAGE_FINISH, PBF_STAGE_DENSITY, PBF_STAGE_WARM_LAMBDA) = range(8)
(PBF_FIELD_POS, PBF_FIELD_VEL, PBF_FIELD_PRED, PBF_FIELD_LAMBDA, PBF_FIELD_KEY, PBF_FIELD_PERM,
 PBF_FIELD_CELL_START, PBF_FIELD_DOMAIN, PBF_FIELD_DENSITY, PBF_FIELD_ID, PBF_FIELD_OMEGA,
 PBF_FIELD_LAMBDA_PREV, PBF_FIELD_LAMBDA_SUM, PBF_FIELD_DISP) = range(14)
WARM_NONE, WARM_PREV, WARM_MLP = 0, 1, 2
MLP_FEATURES, MLP_HIDDEN, MLP_NUM_WEIGHTS, MLP_BLOB_FLOATS = 12, 64, 5057, 5083

MPM_MAT_FLUID, MPM_MAT_COROTATED, MPM_MAT_SNOW, MPM_MAT_NEOHOOKEAN, MPM_MAT_SAND = 0, 1, 2, 3, 4
MPM_BC_SLIP, MPM_BC_STICKY = 0, 1
MPM_FLAG_PER_PARTICLE_MATERIAL, MPM_FLAG_FLUID_F, MPM_FLAG_DYNAMIC_COUNT = 0x1, 0x2, 0x4
MPM_STAGE_CLEAR, MPM_STAGE_P2G, MPM_STAGE_GRID, MPM_STAGE_G2P, MPM_STAGE_SORT = range(5)


class PbfParams(C.Structure):
    _fields_ = [("h", C.c_float), ("cell", C.c_float), ("rho0", C.c_float), ("mass", C.c_float),
                ("dt", C.c_float), ("gravity", C.c_float * 2), ("iters", C.c_int32), ("eps", C.c_float),
                ("scorr_k", C.c_float), ("scorr_dq", C.c_float), ("omega", C.c_float), ("c_min", C.c_float),
                ("xsph_c", C.c_float), ("vort_eps", C.c_float), ("v_max", C.c_float), ("v_min", C.c_float),
                ("wall_margin", C.c_float), ("poly6_coeff", C.c_float), ("spiky_coeff", C.c_float),
                ("flags", C.c_uint32)]

    def copy(self) -> "PbfParams":
        o = PbfParams()
        C.pointer(o)[0] = self
        return o


class Domain(C.Structure):
    _fields_ = [("origin", C.c_float * 2), ("extent", C.c_float * 2)]


class MpmParams(C.Structure):
    _fields_ = [("dx", C.c_float), ("grid_offset", C.c_float), ("nx", C.c_int32), ("ny", C.c_int32),
                ("dt", C.c_float), ("gravity", C.c_float * 2), ("mass", C.c_float), ("vol0", C.c_float),
                ("bc_type", C.c_int32), ("bc_width", C.c_int32), ("clamp_lo", C.c_float * 2),
                ("clamp_hi", C.c_float * 2), ("material", C.c_int32), ("k_bulk", C.c_float),
                ("gamma", C.c_float), ("p_min", C.c_float), ("p_max", C.c_float), ("J_min", C.c_float),
                ("J_max", C.c_float), ("E", C.c_float), ("nu", C.c_float), ("theta_c", C.c_float),
                ("theta_s", C.c_float), ("hardening", C.c_float), ("sort_interval", C.c_int32),
                ("flags", C.c_uint32), ("sand_h", C.c_float * 4)]

    def copy(self) -> "MpmParams":
        o = MpmParams()
        C.pointer(o)[0] = self
        return o


class MpmScene(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("clamp_lo", C.c_float * 2), ("clamp_hi", C.c_float * 2)]


def make_mpm_scene(nx: int, ny: int, clamp_lo, clamp_hi) -> MpmScene:
    s = MpmScene()
    s.nx, s.ny = int(nx), int(ny)
    s.clamp_lo[0], s.clamp_lo[1] = clamp_lo
    s.clamp_hi[0], s.clamp_hi[1] = clamp_hi
    return s


class Hose(C.Structure):
    _fields_ = [("origin", C.c_float * 2), ("velocity", C.c_float * 2), ("nozzle_width", C.c_float),
                ("spacing", C.c_float), ("jitter", C.c_float), ("steps_per_call", C.c_int32)]


class View(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("counts", C.c_void_p), ("chunks_x", C.c_int32),
                ("chunks_y", C.c_int32), ("chunk_dim", C.c_float), ("chunk_capacity", C.c_int32)]


class Raster(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("pitch", C.c_int64), ("width", C.c_int32), ("height", C.c_int32),
                ("scale", C.c_float), ("chunk_dim", C.c_float), ("coverage", C.c_void_p)]


def render_frame(raster: "Raster", view, view_mem: int = MEM_HOST, stream=None) -> None:
    """Draws a published view into the raster's RGBA8 device image (gpe_render_frame)."""
    ptr = C.addressof(view) if view_mem == MEM_HOST else int(view)
    check(lib().gpe_render_frame(C.byref(raster), ptr, view_mem, stream), "gpe_render_frame")


class Tuning(C.Structure):
    _fields_ = [("cell", C.c_float), ("block", C.c_int32), ("persistent", C.c_int32), ("skin", C.c_float)]


class TrainParams(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("weight_decay", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("adam_eps", C.c_float), ("val_fraction", C.c_float),
                ("seed", C.c_uint64), ("lr_schedule", C.c_int32)]


def make_train_params(epochs=20, batch=8192, lr=2e-3, weight_decay=1e-4, beta1=0.9, beta2=0.999, adam_eps=1e-8,
                      val_fraction=0.1, seed=0, lr_schedule=0) -> TrainParams:
    """lr_schedule: 0 constant, 1 cosine decay to 0 over the call's optimiser steps."""
    return TrainParams(epochs, batch, lr, weight_decay, beta1, beta2, adam_eps, val_fraction, seed, lr_schedule)


def make_hose(origin, velocity, nozzle_width, spacing, jitter=0.0, steps_per_call=1) -> Hose:
    h = Hose()
    h.origin[0], h.origin[1] = origin
    h.velocity[0], h.velocity[1] = velocity
    h.nozzle_width, h.spacing, h.jitter, h.steps_per_call = nozzle_width, spacing, jitter, steps_per_call
    return h


def make_domains(boxes) -> "C.Array":
    arr = (Domain * len(boxes))()
    for i, (ox, oy, ex, ey) in enumerate(boxes):
        arr[i].origin[0], arr[i].origin[1] = ox, oy
        arr[i].extent[0], arr[i].extent[1] = ex, ey
    return arr


# ----- library loading -----------------------------------------------------------------------------------
_lib = None

PBF_EXPORTS = ["gpe_pbf_create", "gpe_pbf_destroy", "gpe_pbf_set_params", "gpe_pbf_get_params",
               "gpe_pbf_set_state", "gpe_pbf_get_state", "gpe_pbf_count", "gpe_pbf_num_cells", "gpe_pbf_step",
               "gpe_pbf_stage", "gpe_pbf_get_field", "gpe_pbf_set_field", "gpe_pbf_density_error",
               "gpe_pbf_status", "gpe_pbf_launches_per_step"]
MPM_EXPORTS = ["gpe_mpm_create", "gpe_mpm_destroy", "gpe_mpm_set_params", "gpe_mpm_set_state",
               "gpe_mpm_get_state", "gpe_mpm_count", "gpe_mpm_step", "gpe_mpm_stage", "gpe_mpm_get_grid",
               "gpe_mpm_status", "gpe_mpm_launches_per_step"]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"libgpe.so is not built ({LIB_PATH}); run gpu-physics-engine_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        vp, i32, i64, f32p = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_float)
        L.gpe_error_name.restype = C.c_char_p
        L.gpe_error_name.argtypes = [i32]
        L.gpe_last_error_message.restype = C.c_char_p
        L.gpe_last_cuda_error.restype = i32
        L.gpe_version.restype = i32
        sig = {
            "gpe_pbf_create": [C.POINTER(PbfParams), C.POINTER(Domain), i32, i64, C.POINTER(vp)],
            "gpe_pbf_destroy": [vp],
            "gpe_pbf_set_params": [vp, C.POINTER(PbfParams)],
            "gpe_pbf_get_params": [vp, C.POINTER(PbfParams)],
            "gpe_pbf_set_state": [vp, vp, vp, vp, i64, i32, vp],
            "gpe_pbf_get_state": [vp, vp, vp, vp, i64, i32, vp],
            "gpe_pbf_count": [vp, C.POINTER(i64)],
            "gpe_pbf_num_cells": [vp, C.POINTER(i64)],
            "gpe_pbf_step": [vp, i32, vp],
            "gpe_pbf_stage": [vp, i32, vp],
            "gpe_pbf_get_field": [vp, i32, vp, i64, i32, vp],
            "gpe_pbf_set_field": [vp, i32, vp, i64, i32, vp],
            "gpe_pbf_density_error": [vp, f32p, f32p, vp],
            "gpe_pbf_status": [vp, C.POINTER(C.c_uint32), vp],
            "gpe_pbf_launches_per_step": [vp, C.POINTER(i32)],
            "gpe_selftest_barrier_timeout": [C.POINTER(C.c_uint32)],
            "gpe_mpm_create": [C.POINTER(MpmParams), i64, C.POINTER(vp)],
            "gpe_mpm_create_scenes": [C.POINTER(MpmParams), C.POINTER(MpmScene), i32, i64, C.POINTER(vp)],
            "gpe_mpm_set_scene_ids": [vp, vp, i64, i32, vp],
            "gpe_mpm_destroy": [vp],
            "gpe_mpm_set_params": [vp, C.POINTER(MpmParams)],
            "gpe_mpm_set_state": [vp, vp, vp, vp, vp, vp, vp, i64, i32, vp],
            "gpe_mpm_get_state": [vp, vp, vp, vp, vp, vp, i64, i32, vp],
            "gpe_mpm_count": [vp, C.POINTER(i64)],
            "gpe_mpm_step": [vp, i32, vp],
            "gpe_mpm_stage": [vp, i32, vp],
            "gpe_mpm_get_grid": [vp, vp, i64, i32, vp],
            "gpe_mpm_status": [vp, C.POINTER(C.c_uint32), vp],
            "gpe_mpm_launches_per_step": [vp, C.POINTER(i32)],
            "gpe_pbf_set_warm_start": [vp, i32, vp],
            "gpe_render_frame": [C.POINTER(Raster), vp, i32, vp],
            "gpe_pbf_get_tuning": [vp, C.POINTER(Tuning)],
            "gpe_pbf_set_tuning": [vp, C.POINTER(Tuning)],
            "gpe_pbf_autotune": [vp, i32, C.POINTER(Tuning), C.POINTER(C.c_float), vp],
            "gpe_mlp_create": [i64, C.c_uint64, C.POINTER(vp)],
            "gpe_mlp_destroy": [vp],
            "gpe_mlp_get_blob": [vp, vp, i64],
            "gpe_mlp_set_blob": [vp, vp, i64],
            "gpe_mlp_collect": [vp, vp, i32, i32, C.c_uint64, vp],
            "gpe_mlp_num_pairs": [vp, C.POINTER(i64)],
            "gpe_mlp_get_pairs": [vp, vp, vp, vp, i64, i32, vp],
            "gpe_mlp_set_pairs": [vp, vp, vp, i64, i32, vp],
            "gpe_mlp_train": [vp, C.POINTER(TrainParams), C.POINTER(C.c_float), C.POINTER(C.c_float), vp],
            "gpe_mlp_infer": [vp, vp, vp, i64, i32, vp],
            "gpe_mlp_gradient": [vp, vp, vp, i64, vp, C.POINTER(C.c_float), i32, vp],
            "gpe_pbf_emit": [vp, C.POINTER(Hose), C.c_uint64, C.POINTER(i32), vp],
            "gpe_pbf_publish": [vp, vp, i32, vp],
            "gpe_pbf_enqueue": [vp, i32, vp],
            "gpe_mpm_emit": [vp, C.POINTER(Hose), C.c_uint64, C.POINTER(i32), vp],
            "gpe_mpm_publish": [vp, vp, i32, vp],
            "gpe_mpm_enqueue": [vp, i32, vp],
            "gpe_mpm_buffers": [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                C.POINTER(vp)],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = i32
        _lib = L
    return _lib


class GpeError(RuntimeError):
    def __init__(self, status: int, where: str):
        L = lib()
        msg = L.gpe_last_error_message().decode(errors="replace")
        super().__init__(f"{where}: {L.gpe_error_name(status).decode()} ({status}) {msg}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != OK:
        raise GpeError(status, where)


def _ptr(a) -> int | None:
    """Address of a numpy array (host) or a torch tensor / int device pointer."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


def _mem(a, pinned_ok: bool = False) -> int:
    """Memory kind of a buffer: numpy arrays and CPU tensors are host memory (page-locked CPU tensors are
    MEM_PINNED where the entry point takes it: the copy is then asynchronous), CUDA tensors and ints device."""
    if isinstance(a, np.ndarray):
        return MEM_HOST
    if hasattr(a, "is_cuda") and not a.is_cuda:
        return MEM_PINNED if (pinned_ok and a.is_pinned()) else MEM_HOST
    return MEM_DEVICE


def _f32(a, shape_last: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(-1, shape_last)


# ----- PBF ----------------------------------------------------------------------------------------------
_FIELD_DT = {PBF_FIELD_POS: (np.float32, 2), PBF_FIELD_VEL: (np.float32, 2), PBF_FIELD_PRED: (np.float32, 2),
             PBF_FIELD_LAMBDA: (np.float32, 1), PBF_FIELD_KEY: (np.uint32, 1), PBF_FIELD_PERM: (np.uint32, 1),
             PBF_FIELD_CELL_START: (np.uint32, 1), PBF_FIELD_DOMAIN: (np.int32, 1),
             PBF_FIELD_DENSITY: (np.float32, 1), PBF_FIELD_ID: (np.uint32, 1), PBF_FIELD_OMEGA: (np.float32, 1),
             PBF_FIELD_LAMBDA_PREV: (np.float32, 1), PBF_FIELD_LAMBDA_SUM: (np.float32, 1),
             PBF_FIELD_DISP: (np.float32, 2)}


class Pbf:
    """One PBF engine handle (gpe_pbf): a set of scenes with their particles resident on the GPU."""

    def __init__(self, params: PbfParams, boxes, capacity: int):
        self.params = params.copy()
        self.boxes = [tuple(map(float, b)) for b in boxes]
        self._doms = make_domains(self.boxes)
        h = C.c_void_p()
        check(lib().gpe_pbf_create(C.byref(self.params), self._doms, len(self.boxes), int(capacity), C.byref(h)),
              "gpe_pbf_create")
        self.h = h
        self.capacity = int(capacity)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gpe_pbf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: PbfParams) -> None:
        check(lib().gpe_pbf_set_params(self.h, C.byref(params)), "gpe_pbf_set_params")
        self.params = params.copy()

    def set_state(self, pos, vel=None, domain=None, stream=None) -> None:
        if isinstance(pos, np.ndarray):
            pos = _f32(pos, 2)
            vel = None if vel is None else _f32(vel, 2)
            domain = None if domain is None else np.ascontiguousarray(domain, dtype=np.int32)
            n = pos.shape[0]
        else:
            n = pos.shape[0]
        check(lib().gpe_pbf_set_state(self.h, _ptr(pos), _ptr(vel), _ptr(domain), n, _mem(pos, True), stream),
              "gpe_pbf_set_state")
        self._keep = (pos, vel, domain)

    @property
    def n(self) -> int:
        v = C.c_int64()
        check(lib().gpe_pbf_count(self.h, C.byref(v)), "gpe_pbf_count")
        return v.value

    @property
    def num_cells(self) -> int:
        v = C.c_int64()
        check(lib().gpe_pbf_num_cells(self.h, C.byref(v)), "gpe_pbf_num_cells")
        return v.value

    def get_state(self, pos=None, vel=None, stream=None):
        """Returns (pos, vel, scene id) in the current sorted order. With caller buffers (host arrays, CUDA
        tensors or device pointers) only pos/vel are written and the scene id is not read back; into
        page-locked CPU tensors the copy is asynchronous (synchronize the stream before reading them)."""
        n = self.n
        dom = None
        if pos is None:
            pos = np.empty((n, 2), np.float32)
            vel = np.empty((n, 2), np.float32)
            dom = np.empty(n, np.int32)
        check(lib().gpe_pbf_get_state(self.h, _ptr(pos), _ptr(vel), _ptr(dom), n, _mem(pos, True), stream),
              "gpe_pbf_get_state")
        return pos, vel, dom

    def step(self, n_steps: int = 1, stream=None) -> None:
        check(lib().gpe_pbf_step(self.h, int(n_steps), stream), "gpe_pbf_step")

    def stage(self, stage: int, stream=None) -> None:
        check(lib().gpe_pbf_stage(self.h, int(stage), stream), f"gpe_pbf_stage({stage})")

    def field(self, field: int, stream=None) -> np.ndarray:
        dt, w = _FIELD_DT[field]
        n = self.num_cells + 1 if field == PBF_FIELD_CELL_START else self.n
        out = np.empty((n, w) if w > 1 else (n,), dt)
        check(lib().gpe_pbf_get_field(self.h, field, out.ctypes.data, n, MEM_HOST, stream),
              f"gpe_pbf_get_field({field})")
        return out

    def set_field(self, field: int, values: np.ndarray, stream=None) -> None:
        dt, w = _FIELD_DT[field]
        v = np.ascontiguousarray(values, dtype=dt)
        n = v.shape[0]
        check(lib().gpe_pbf_set_field(self.h, field, v.ctypes.data, n, MEM_HOST, stream),
              f"gpe_pbf_set_field({field})")

    def density_error(self, stream=None) -> tuple[float, float]:
        mx, mn = C.c_float(), C.c_float()
        check(lib().gpe_pbf_density_error(self.h, C.byref(mx), C.byref(mn), stream), "gpe_pbf_density_error")
        return mx.value, mn.value

    def status(self, stream=None) -> int:
        v = C.c_uint32()
        check(lib().gpe_pbf_status(self.h, C.byref(v), stream), "gpe_pbf_status")
        return v.value

    def launches_per_step(self) -> int:
        v = C.c_int32()
        check(lib().gpe_pbf_launches_per_step(self.h, C.byref(v)), "gpe_pbf_launches_per_step")
        return v.value

    def emit(self, hose: Hose, seed: int = 0, stream=None) -> int:
        req = C.c_int32()
        check(lib().gpe_pbf_emit(self.h, C.byref(hose), int(seed), C.byref(req), stream), "gpe_pbf_emit")
        return req.value

    def publish(self, view: View, view_mem: int = MEM_HOST, stream=None) -> None:
        ptr = C.addressof(view) if view_mem == MEM_HOST else int(view)
        check(lib().gpe_pbf_publish(self.h, ptr, view_mem, stream), "gpe_pbf_publish")

    def enqueue(self, n_steps: int, stream=None) -> None:
        check(lib().gpe_pbf_enqueue(self.h, int(n_steps), stream), "gpe_pbf_enqueue")

    def tuning(self) -> Tuning:
        t = Tuning()
        check(lib().gpe_pbf_get_tuning(self.h, C.byref(t)), "gpe_pbf_get_tuning")
        return t

    def set_tuning(self, cell: float = 0.0, block: int = 256, persistent: int = 0, skin: float = 0.075) -> None:
        """persistent: 0 one launch per pass, 1 (or True) the passes in one cooperative launch, 2 the whole step
        (predict + sort included) in one cooperative launch."""
        t = Tuning(cell, block, int(persistent), skin)
        check(lib().gpe_pbf_set_tuning(self.h, C.byref(t)), "gpe_pbf_set_tuning")

    def autotune(self, trial_steps: int = 4, stream=None) -> tuple[Tuning, float]:
        t, ms = Tuning(), C.c_float()
        check(lib().gpe_pbf_autotune(self.h, int(trial_steps), C.byref(t), C.byref(ms), stream), "gpe_pbf_autotune")
        return t, ms.value

    def set_warm_start(self, mode: int, mlp: "Mlp | None" = None) -> None:
        check(lib().gpe_pbf_set_warm_start(self.h, int(mode), None if mlp is None else mlp.h),
              "gpe_pbf_set_warm_start")
        self._mlp = mlp  # keep the network alive while the engine uses it


def selftest_barrier_timeout() -> int:
    """Runs gpe_selftest_barrier_timeout and returns the device status word it recorded."""
    v = C.c_uint32()
    check(lib().gpe_selftest_barrier_timeout(C.byref(v)), "gpe_selftest_barrier_timeout")
    return int(v.value)


# ----- MPM ----------------------------------------------------------------------------------------------
class Mlp:
    """The warm-start network (gpe_mlp): parameters, training pairs, GPU training and inference."""

    def __init__(self, max_pairs: int = 0, seed: int = 0):
        h = C.c_void_p()
        check(lib().gpe_mlp_create(int(max_pairs), int(seed), C.byref(h)), "gpe_mlp_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gpe_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def blob(self) -> np.ndarray:
        b = np.empty(MLP_BLOB_FLOATS, np.float32)
        check(lib().gpe_mlp_get_blob(self.h, b.ctypes.data, b.size), "gpe_mlp_get_blob")
        return b

    def set_blob(self, blob) -> None:
        b = np.ascontiguousarray(blob, dtype=np.float32).reshape(-1)
        check(lib().gpe_mlp_set_blob(self.h, b.ctypes.data, b.size), "gpe_mlp_set_blob")

    def collect(self, pbf: Pbf, n_steps: int, stride: int = 1, seed: int = 0, stream=None) -> None:
        check(lib().gpe_mlp_collect(self.h, pbf.h, int(n_steps), int(stride), int(seed), stream), "gpe_mlp_collect")

    @property
    def num_pairs(self) -> int:
        v = C.c_int64()
        check(lib().gpe_mlp_num_pairs(self.h, C.byref(v)), "gpe_mlp_num_pairs")
        return v.value

    def pairs(self):
        n = self.num_pairs
        X = np.empty((n, MLP_FEATURES), np.float32)
        T = np.empty(n, np.float32)
        idx = np.empty(n, np.int32)
        check(lib().gpe_mlp_get_pairs(self.h, X.ctypes.data, T.ctypes.data, idx.ctypes.data, n, MEM_HOST, None),
              "gpe_mlp_get_pairs")
        return X, T, idx

    def set_pairs(self, X, T) -> None:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_FEATURES)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1)
        check(lib().gpe_mlp_set_pairs(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], MEM_HOST, None),
              "gpe_mlp_set_pairs")

    def train(self, params: TrainParams | None = None, stream=None) -> tuple[float, float]:
        params = params or make_train_params()
        tl, vl = C.c_float(), C.c_float()
        check(lib().gpe_mlp_train(self.h, C.byref(params), C.byref(tl), C.byref(vl), stream), "gpe_mlp_train")
        return tl.value, vl.value

    def infer(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_FEATURES)
        out = np.empty(X.shape[0], np.float32)
        check(lib().gpe_mlp_infer(self.h, X.ctypes.data, out.ctypes.data, X.shape[0], MEM_HOST, None),
              "gpe_mlp_infer")
        return out

    def gradient(self, X, T) -> tuple[np.ndarray, float]:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_FEATURES)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1)
        g = np.empty(MLP_NUM_WEIGHTS, np.float32)
        loss = C.c_float()
        check(lib().gpe_mlp_gradient(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], g.ctypes.data, C.byref(loss),
                                     MEM_HOST, None), "gpe_mlp_gradient")
        return g, loss.value


class Mpm:
    """One MLS-MPM engine handle (gpe_mpm)."""

    def __init__(self, params: MpmParams, capacity: int, scenes=None):
        """scenes: a list of MpmScene (gpe_mpm_create_scenes); None for one scene of params' grid."""
        self.params = params.copy()
        h = C.c_void_p()
        if scenes:
            arr = (MpmScene * len(scenes))(*scenes)
            check(lib().gpe_mpm_create_scenes(C.byref(self.params), arr, len(scenes), int(capacity), C.byref(h)),
                  "gpe_mpm_create_scenes")
            self.nodes = sum(s.nx * s.ny for s in scenes)
        else:
            check(lib().gpe_mpm_create(C.byref(self.params), int(capacity), C.byref(h)), "gpe_mpm_create")
            self.nodes = params.nx * params.ny
        self.h = h
        self.capacity = int(capacity)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gpe_mpm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: MpmParams) -> None:
        check(lib().gpe_mpm_set_params(self.h, C.byref(params)), "gpe_mpm_set_params")
        self.params = params.copy()

    def set_state(self, pos, vel=None, Cm=None, F=None, J=None, material=None, stream=None, scene_id=None) -> None:
        if isinstance(pos, np.ndarray):
            pos = _f32(pos, 2)
            vel = None if vel is None else _f32(vel, 2)
            Cm = None if Cm is None else _f32(Cm, 4)
            F = None if F is None else _f32(F, 4)
            J = None if J is None else np.ascontiguousarray(J, dtype=np.float32).reshape(-1)
            material = None if material is None else np.ascontiguousarray(material, dtype=np.int32)
        n = pos.shape[0]
        check(lib().gpe_mpm_set_state(self.h, _ptr(pos), _ptr(vel), _ptr(Cm), _ptr(F), _ptr(J), _ptr(material), n,
                                      _mem(pos), stream), "gpe_mpm_set_state")
        self._keep = (pos, vel, Cm, F, J, material)
        if scene_id is not None:
            self.set_scene_ids(scene_id, stream=stream)

    def set_scene_ids(self, scene_id, stream=None) -> None:
        if isinstance(scene_id, np.ndarray):
            scene_id = np.ascontiguousarray(scene_id, dtype=np.int32)
        check(lib().gpe_mpm_set_scene_ids(self.h, _ptr(scene_id), len(scene_id), _mem(scene_id), stream),
              "gpe_mpm_set_scene_ids")
        self._keep_sid = scene_id

    @property
    def n(self) -> int:
        v = C.c_int64()
        check(lib().gpe_mpm_count(self.h, C.byref(v)), "gpe_mpm_count")
        return v.value

    def get_state(self, stream=None):
        n = self.n
        pos = np.empty((n, 2), np.float32)
        vel = np.empty((n, 2), np.float32)
        Cm = np.empty((n, 4), np.float32)
        F = np.empty((n, 4), np.float32)
        J = np.empty(n, np.float32)
        check(lib().gpe_mpm_get_state(self.h, _ptr(pos), _ptr(vel), _ptr(Cm), _ptr(F), _ptr(J), n, MEM_HOST, stream),
              "gpe_mpm_get_state")
        return pos, vel, Cm, F, J

    def get_state_device(self, pos, vel=None, Cm=None, F=None, J=None, stream=None) -> None:
        check(lib().gpe_mpm_get_state(self.h, _ptr(pos), _ptr(vel), _ptr(Cm), _ptr(F), _ptr(J), self.n, _mem(pos),
                                      stream), "gpe_mpm_get_state")

    def step(self, n_steps: int = 1, stream=None) -> None:
        check(lib().gpe_mpm_step(self.h, int(n_steps), stream), "gpe_mpm_step")

    def stage(self, stage: int, stream=None) -> None:
        check(lib().gpe_mpm_stage(self.h, int(stage), stream), f"gpe_mpm_stage({stage})")

    def grid(self, stream=None) -> np.ndarray:
        nn = self.nodes
        out = np.empty((nn, 4), np.float32)
        check(lib().gpe_mpm_get_grid(self.h, out.ctypes.data, nn, MEM_HOST, stream), "gpe_mpm_get_grid")
        return out

    def status(self, stream=None) -> int:
        v = C.c_uint32()
        check(lib().gpe_mpm_status(self.h, C.byref(v), stream), "gpe_mpm_status")
        return v.value

    def p2g_wide_warps(self, stream=None) -> int:
        """Warps whose P2G needed the 5-round run reduction since the last call (read and cleared); a warp
        holds 64 particles, two per lane."""
        v = C.c_uint32()
        check(lib().gpe_mpm_p2g_wide_warps(self.h, C.byref(v), stream), "gpe_mpm_p2g_wide_warps")
        return v.value

    def emit(self, hose: Hose, seed: int = 0, stream=None) -> int:
        req = C.c_int32()
        check(lib().gpe_mpm_emit(self.h, C.byref(hose), int(seed), C.byref(req), stream), "gpe_mpm_emit")
        return req.value

    def publish(self, view: View, view_mem: int = MEM_HOST, stream=None) -> None:
        ptr = C.addressof(view) if view_mem == MEM_HOST else int(view)
        check(lib().gpe_mpm_publish(self.h, ptr, view_mem, stream), "gpe_mpm_publish")

    def enqueue(self, n_steps: int, stream=None) -> None:
        check(lib().gpe_mpm_enqueue(self.h, int(n_steps), stream), "gpe_mpm_enqueue")

    def launches_per_step(self) -> int:
        v = C.c_int32()
        check(lib().gpe_mpm_launches_per_step(self.h, C.byref(v)), "gpe_mpm_launches_per_step")
        return v.value

    def buffers(self) -> dict:
        ptrs = [C.c_void_p() for _ in range(6)]
        check(lib().gpe_mpm_buffers(self.h, *[C.byref(p) for p in ptrs]), "gpe_mpm_buffers")
        return dict(zip(["pos", "vel", "C", "F", "J", "count"], [p.value for p in ptrs]))
