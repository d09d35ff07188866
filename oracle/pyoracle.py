"""ctypes wrapper of the oracle (oracle.c). Test infrastructure: used by tests/, __graft_entry__.smoke() and
the CPU-baseline legs of bench.py, only as the checker / CPU baseline, never by the engine."""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent / "gpu-physics-engine_gb300"))

from gpe import Domain, MpmParams, PbfParams, make_domains  # noqa: E402  (struct layouts only)

from . import build as _build  # noqa: E402

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        pp, dp, mp = C.POINTER(PbfParams), C.POINTER(Domain), C.POINTER(MpmParams)
        L.orc_pbf_num_cells.restype = i64
        L.orc_pbf_num_cells.argtypes = [pp, dp, i32]
        L.orc_pbf_predict_sort.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_pbf_lambda.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp, vp]
        L.orc_pbf_delta_p.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp]
        L.orc_pbf_xsph.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp, vp]
        L.orc_pbf_vorticity.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp]
        L.orc_pbf_density.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp]
        L.orc_pbf_step.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, i32, vp, vp]
        L.orc_pbf_density_error.argtypes = [pp, dp, i32, i64, vp, vp, vp, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
        L.orc_pbf_features.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp, vp, vp]
        L.orc_mlp_forward.argtypes = [vp, i64, vp, vp, i32]
        L.orc_mlp_gradient.argtypes = [vp, i64, vp, vp, vp, vp, i32]
        L.orc_pbf_step_warm.argtypes = [pp, dp, i32, i64, vp, vp, vp, vp, vp, i32, vp, i32]
        L.orc_render_frame.argtypes = [i32, i32, C.c_float, C.c_float, i32, i32, vp, vp, vp]
        L.orc_mpm_p2g.argtypes = [mp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.orc_mpm_grid_update.argtypes = [mp, vp]
        L.orc_mpm_g2p.argtypes = [mp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.orc_mpm_step.argtypes = [mp, i64, vp, vp, vp, vp, vp, vp, i32]
        L.orc_num_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


class PbfOracle:
    def __init__(self, params: PbfParams, boxes):
        self.params = params.copy()
        self.boxes = [tuple(map(float, b)) for b in boxes]
        self.doms = make_domains(self.boxes)
        self.nd = len(self.boxes)

    @property
    def num_cells(self) -> int:
        return int(lib().orc_pbf_num_cells(C.byref(self.params), self.doms, self.nd))

    def predict_sort(self, x, v, dom=None):
        x = _c(x, np.float32).reshape(-1, 2)
        v = _c(v, np.float32).reshape(-1, 2)
        dom = _c(dom, np.int32)
        n = x.shape[0]
        key = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        cs = np.empty(self.num_cells + 1, np.uint32)
        xso = np.empty((n, 2), np.float32)
        xss = np.empty((n, 2), np.float32)
        ds = np.empty(n, np.int32)
        lib().orc_pbf_predict_sort(C.byref(self.params), self.doms, self.nd, n, _p(x), _p(v), _p(dom), _p(key),
                                   _p(perm), _p(cs), _p(xso), _p(xss), _p(ds))
        return dict(key=key, perm=perm, cell_start=cs, x=xso, xs=xss, dom=ds)

    def lambda_(self, xs, dom, cs, pair_id=None):
        xs = _c(xs, np.float32)
        n = xs.shape[0]
        lam = np.empty(n, np.float32)
        rho = np.empty(n, np.float32)
        lib().orc_pbf_lambda(C.byref(self.params), self.doms, self.nd, n, _p(xs), _p(_c(dom, np.int32)),
                             _p(_c(cs, np.uint32)), _p(_c(pair_id, np.uint32)), _p(lam), _p(rho))
        return lam, rho

    def delta_p(self, xs, dom, cs, lam):
        xs = _c(xs, np.float32)
        n = xs.shape[0]
        out = np.empty((n, 2), np.float32)
        lib().orc_pbf_delta_p(C.byref(self.params), self.doms, self.nd, n, _p(xs), _p(_c(dom, np.int32)),
                              _p(_c(cs, np.uint32)), _p(_c(lam, np.float32)), _p(out))
        return out

    def xsph(self, x, xs, dom, cs):
        x = _c(x, np.float32)
        xs = _c(xs, np.float32)
        n = xs.shape[0]
        v = np.empty((n, 2), np.float32)
        w = np.empty(n, np.float32)
        lib().orc_pbf_xsph(C.byref(self.params), self.doms, self.nd, n, _p(x), _p(xs), _p(_c(dom, np.int32)),
                           _p(_c(cs, np.uint32)), _p(v), _p(w))
        return v, w

    def vorticity(self, xs, dom, cs, omega, v):
        v = np.array(v, dtype=np.float32, copy=True)
        xs = _c(xs, np.float32)
        lib().orc_pbf_vorticity(C.byref(self.params), self.doms, self.nd, xs.shape[0], _p(xs),
                                _p(_c(dom, np.int32)), _p(_c(cs, np.uint32)), _p(_c(omega, np.float32)), _p(v))
        return v

    def density(self, xs, dom, cs):
        xs = _c(xs, np.float32)
        rho = np.empty(xs.shape[0], np.float32)
        lib().orc_pbf_density(C.byref(self.params), self.doms, self.nd, xs.shape[0], _p(xs),
                              _p(_c(dom, np.int32)), _p(_c(cs, np.uint32)), _p(rho))
        return rho

    def step(self, x, v, dom=None, n_steps=1, pair_id=None):
        x = np.array(x, dtype=np.float32, copy=True).reshape(-1, 2)
        v = np.array(v, dtype=np.float32, copy=True).reshape(-1, 2)
        dom = None if dom is None else np.array(dom, dtype=np.int32, copy=True)
        pid = None if pair_id is None else np.array(pair_id, dtype=np.uint32, copy=True)
        n = x.shape[0]
        lam = np.empty(n, np.float32)
        cs = np.empty(self.num_cells + 1, np.uint32)
        lib().orc_pbf_step(C.byref(self.params), self.doms, self.nd, n, _p(x), _p(v), _p(dom), _p(pid),
                           int(n_steps), _p(lam), _p(cs))
        return dict(x=x, v=v, dom=dom, lam=lam, cell_start=cs, pair_id=pid)

    def features(self, xs, x, prev, dom, cs, pair_id=None):
        xs = _c(xs, np.float32)
        n = xs.shape[0]
        f = np.empty((n, 12), np.float32)
        lib().orc_pbf_features(C.byref(self.params), self.doms, self.nd, n, _p(xs), _p(_c(x, np.float32)),
                               _p(_c(prev, np.float32)), _p(_c(dom, np.int32)), _p(_c(cs, np.uint32)),
                               _p(_c(pair_id, np.uint32)), _p(f))
        return f

    def step_warm(self, x, v, acc, mode, blob=None, dom=None, n_steps=1, pair_id=None):
        """Steps that keep the summed multipliers (mode 0 cold, 1 previous sum, 2 network blob)."""
        x = np.array(x, dtype=np.float32, copy=True).reshape(-1, 2)
        v = np.array(v, dtype=np.float32, copy=True).reshape(-1, 2)
        acc = np.array(acc, dtype=np.float32, copy=True).reshape(-1)
        dom = None if dom is None else np.array(dom, dtype=np.int32, copy=True)
        pid = None if pair_id is None else np.array(pair_id, dtype=np.uint32, copy=True)
        lib().orc_pbf_step_warm(C.byref(self.params), self.doms, self.nd, x.shape[0], _p(x), _p(v), _p(dom), _p(pid),
                                _p(acc), int(mode), _p(_c(blob, np.float32)), int(n_steps))
        return dict(x=x, v=v, acc=acc, dom=dom, pair_id=pid)

    def density_error(self, x, dom, cs):
        x = _c(x, np.float32)
        mx, mn = C.c_double(), C.c_double()
        lib().orc_pbf_density_error(C.byref(self.params), self.doms, self.nd, x.shape[0], _p(x),
                                    _p(_c(dom, np.int32)), _p(_c(cs, np.uint32)), C.byref(mx), C.byref(mn))
        return mx.value, mn.value


class MpmOracle:
    def __init__(self, params: MpmParams):
        self.params = params.copy()

    def p2g(self, x, v, Cm, F, J, mat=None):
        n = x.shape[0]
        g = np.empty((self.params.nx * self.params.ny, 3), np.float64)
        lib().orc_mpm_p2g(C.byref(self.params), n, _p(_c(x, np.float32)), _p(_c(v, np.float32)),
                          _p(_c(Cm, np.float32)), _p(_c(F, np.float32)), _p(_c(J, np.float32)),
                          _p(_c(mat, np.int32)), _p(g))
        return g

    def grid_update(self, grid):
        g = np.array(grid, dtype=np.float64, copy=True)
        lib().orc_mpm_grid_update(C.byref(self.params), _p(g))
        return g

    def g2p(self, grid, x, v, Cm, F, J, mat=None):
        x, v, Cm, F, J = (np.array(a, dtype=np.float32, copy=True) for a in (x, v, Cm, F, J))
        lib().orc_mpm_g2p(C.byref(self.params), x.shape[0], _p(np.ascontiguousarray(grid, np.float64)), _p(x),
                          _p(v), _p(Cm), _p(F), _p(J), _p(_c(mat, np.int32)))
        return x, v, Cm, F, J

    def step(self, x, v, Cm, F, J, mat=None, n_steps=1):
        x, v, Cm, F, J = (np.array(a, dtype=np.float32, copy=True) for a in (x, v, Cm, F, J))
        lib().orc_mpm_step(C.byref(self.params), x.shape[0], _p(x), _p(v), _p(Cm), _p(F), _p(J),
                           _p(_c(mat, np.int32)), int(n_steps))
        return x, v, Cm, F, J


def mlp_forward(blob, X, bf16=True):
    X = _c(X, np.float32).reshape(-1, 12)
    out = np.empty(X.shape[0], np.float32)
    lib().orc_mlp_forward(_p(_c(blob, np.float32)), X.shape[0], _p(X), _p(out), int(bool(bf16)))
    return out


def mlp_gradient(blob, X, T, bf16=True):
    X = _c(X, np.float32).reshape(-1, 12)
    T = _c(T, np.float32).reshape(-1)
    g = np.empty(5057, np.float64)
    loss = C.c_double()
    lib().orc_mlp_gradient(_p(_c(blob, np.float32)), X.shape[0], _p(X), _p(T), _p(g), C.byref(loss),
                           int(bool(bf16)))
    return g, loss.value


def render_frame(width, height, scale, chunk_dim, pos, counts):
    """pos: (chunks, capacity, 2) float32 chunk-major view arrays; counts: (chunks,) int32."""
    pos = np.ascontiguousarray(pos, np.float32)
    counts = np.ascontiguousarray(counts, np.int32)
    chunks, capacity = pos.shape[0], pos.shape[1]
    out = np.empty((height, width, 4), np.uint8)
    lib().orc_render_frame(int(width), int(height), float(scale), float(chunk_dim), chunks, capacity, _p(pos),
                           _p(counts), _p(out))
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())
