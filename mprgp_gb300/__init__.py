"""Python mirror of the GB300 MPRGP C ABI (include/mprgp_gpu.h).

The product is libmprgp_gb300.so (hand-written sm_103a CUDA behind a C ABI)
and the C++ façade in include/mprgp/.  This module binds the same C ABI with
ctypes so tests and bench.py can drive it; it holds no solver logic and no
fallback: if the shared library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# MPRGP_LIBRARY selects another build of the library, e.g. the bounds-checked
# debug build (buildlib.build(checks=True))
LIB_PATH = os.environ.get("MPRGP_LIBRARY") or os.path.join(HERE, "_build", "libmprgp_gb300.so")

OK, NOT_CONVERGED, BREAKDOWN, OOM, TIMEOUT, INVALID, CUDA_ERROR, NO_DEVICE, BUSY = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)
KIND_LOWER, KIND_BOX, KIND_DECOUPLED, KIND_PLANES = 0, 1, 2, 3
ALG_DEFAULT, ALG_MONOTONE, ALG_PLAIN = 0, 1, 2
PRECOND_DEFAULT, PRECOND_NONE, PRECOND_INFACE, PRECOND_DECOUPLE = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1


class Options(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_it", C.c_int), ("kind", C.c_int),
                ("algorithm", C.c_int), ("precond", C.c_int), ("precision", C.c_int),
                ("project_x0", C.c_int), ("use_ev", C.c_int), ("seed", C.c_uint64),
                ("wait_limit_s", C.c_double)]


class IcaStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("residual", C.c_double),
                ("pgs_sweeps", C.c_longlong), ("levels", C.c_int), ("device_ms", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("code", C.c_int), ("iterations", C.c_int), ("num_cg", C.c_int),
                ("num_exp", C.c_int), ("num_prop", C.c_int), ("power_iters", C.c_int),
                ("active", C.c_int), ("ev_updated", C.c_int), ("residual", C.c_double),
                ("alpha_bar", C.c_double), ("spec_rad", C.c_double),
                ("spmv_fp64", C.c_longlong), ("spmv_fp32", C.c_longlong),
                ("phases", C.c_longlong), ("device_ms", C.c_double),
                ("power_passes", C.c_longlong)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_slots", C.c_int), ("quantum_phases", C.c_int),
                ("power_launches", C.c_int), ("cluster_quantum", C.c_int), ("lanes", C.c_int),
                ("hbm_reserve", C.c_size_t)]


class BeamParams(C.Structure):
    _fields_ = [("a", C.c_int), ("b", C.c_int), ("c", C.c_int), ("edge", C.c_double),
                ("young", C.c_double), ("poisson", C.c_double), ("rho", C.c_double),
                ("dt", C.c_double), ("gravity", C.c_double), ("lift", C.c_double),
                ("v0_sigma", C.c_double), ("extra_planes_max", C.c_int),
                ("extra_planes_min", C.c_int), ("active_frac", C.c_double),
                ("seed", C.c_uint64), ("plane_band", C.c_double), ("max_tilt", C.c_double),
                ("plane_mode", C.c_int), ("facet_layers", C.c_int)]


_lib = None
_P = C.c_void_p
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
_UP = C.POINTER(C.c_ubyte)


def _sig(lib):
    def s(name, res, *args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = list(args)
    s("mprgp_version", C.c_int)
    s("mprgp_status_string", C.c_char_p, C.c_int)
    s("mprgp_last_error", C.c_char_p)
    s("mprgp_default_options", None, C.POINTER(Options))
    s("mprgp_device_count", C.c_int, _IP)
    s("mprgp_context_create", C.c_int, C.c_int, C.POINTER(_P))
    s("mprgp_context_destroy", C.c_int, _P)
    s("mprgp_context_stream", _P, _P)
    s("mprgp_context_sync", C.c_int, _P)
    s("mprgp_context_info", C.c_int, _P, _IP, _IP)
    s("mprgp_context_set_tuning", C.c_int, _P, C.c_int, C.c_int)
    s("mprgp_context_set_cluster", C.c_int, _P, C.c_int)
    s("mprgp_context_set_cluster_items", C.c_int, _P, C.c_int)
    s("mprgp_problem_create", C.c_int, _P, C.c_int, C.POINTER(_P))
    s("mprgp_problem_destroy", C.c_int, _P)
    s("mprgp_problem_set_matrix", C.c_int, _P, C.c_int, _P, _P, _P, C.c_int, C.c_int)
    s("mprgp_problem_set_rhs", C.c_int, _P, _P, C.c_int)
    s("mprgp_problem_set_planes", C.c_int, _P, _P, _P, C.c_int)
    s("mprgp_problem_set_bounds", C.c_int, _P, _P, _P)
    s("mprgp_problem_set_x", C.c_int, _P, _P, C.c_int)
    s("mprgp_problem_get_x", C.c_int, _P, _P, C.c_int)
    s("mprgp_problem_num_constraints", C.c_int, _P, _IP)
    s("mprgp_problem_get_face", C.c_int, _P, _P)
    s("mprgp_problem_set_ev", C.c_int, _P, _P)
    s("mprgp_problem_set_power_cache", C.c_int, _P, C.c_int)
    s("mprgp_problem_get_ev", C.c_int, _P, _P, _IP)
    s("mprgp_problem_solve", C.c_int, _P, C.POINTER(Options), C.POINTER(Stats))
    s("mprgp_problem_spmv", C.c_int, _P, _P, _P, C.c_int)
    s("mprgp_problem_set_trace", C.c_int, _P, C.c_int)
    s("mprgp_problem_get_trace", C.c_int, _P, _P, C.c_int, _IP)
    s("mprgp_problem_bytes", C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int)
    s("mprgp_solve_bsr", C.c_int, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P,
      C.POINTER(Options), _P, _P, _P, C.POINTER(Stats))
    s("mprgp_solve_batch", C.c_int, _P, C.c_int, C.POINTER(_P), C.POINTER(Options),
      C.POINTER(Stats))
    s("mprgp_solve_noalloc", C.c_int, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P,
      C.POINTER(Options), _P, _P, C.POINTER(Stats))
    s("mprgp_ica_solve", C.c_int, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, C.c_int,
      C.c_double, C.c_int, C.c_double, C.POINTER(IcaStats))
    s("mprgp_server_create", C.c_int, _P, C.POINTER(ServerConfig), C.POINTER(_P))
    s("mprgp_server_destroy", C.c_int, _P)
    s("mprgp_context_room", C.c_int, _P, C.POINTER(C.c_size_t))
    s("mprgp_server_submit", C.c_int, _P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P,
      C.c_int, C.c_int, C.POINTER(Options), C.POINTER(C.c_longlong))
    s("mprgp_server_step", C.c_int, _P, _IP, _IP, _IP)
    s("mprgp_server_poll", C.c_int, _P, C.POINTER(C.c_longlong), C.c_int, _IP)
    s("mprgp_context_counters", C.c_int, _P, C.POINTER(C.c_longlong), C.POINTER(C.c_double),
      C.POINTER(C.c_double))
    s("mprgp_server_result", C.c_int, _P, C.c_longlong, _P, _P, C.POINTER(Stats), _P, _IP)
    s("mprgp_server_info", C.c_int, _P, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), _IP)
    s("mprgp_beam_mesh", C.c_int, C.POINTER(BeamParams), _P, _P, _P, _P)
    s("mprgp_problem_num_vertices", C.c_int, _P, _IP)
    s("mprgp_problem_get_planes", C.c_int, _P, _P, _P)
    s("mprgp_planes_collide", C.c_int, _P, _P, _P, C.c_int, C.c_int, _P, C.c_double, C.c_int, _IP)
    s("mprgp_fem_create", C.c_int, _P, C.c_int, C.c_int, _P, _P, C.c_double, C.c_double,
      C.c_double, C.POINTER(_P))
    s("mprgp_fem_destroy", C.c_int, _P)
    s("mprgp_fem_sizes", C.c_int, _P, _IP, _IP)
    s("mprgp_fem_assemble", C.c_int, _P, C.c_double, _P, _P, _P, C.c_int, _P, C.c_int)
    s("mprgp_fem_rhs", C.c_int, _P, C.c_double, _P, _P, _P, C.c_int, _P)
    s("mprgp_fem_get", C.c_int, _P, _P, _P, _P, _P, _P)
    s("mprgp_beam_default", None, C.POINTER(BeamParams))
    s("mprgp_beam_sizes", C.c_int, C.POINTER(BeamParams), _IP, _IP, _IP)
    s("mprgp_beam_build", C.c_int, C.POINTER(BeamParams), _P, _P, _P, _P, _P, _P, _P)


def lib():
    """Loads libmprgp_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run mprgp_gb300.build() first")
        handle = C.CDLL(LIB_PATH)
        _sig(handle)
        _lib = handle
    return _lib


def build(**kw) -> str:
    from . import buildlib
    return buildlib.build(**kw)


class MPRGPError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        L = lib()
        msg = L.mprgp_status_string(code).decode()
        detail = L.mprgp_last_error().decode()
        super().__init__(f"{what}: {msg} ({code}) {detail}")
        self.code = code


def _check(code: int, what: str) -> int:
    if code < NOT_CONVERGED:
        raise MPRGPError(code, what)
    return code


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _set_fields(struct, kw):
    names = {f[0] for f in type(struct)._fields_}
    for k, v in kw.items():
        if k not in names:
            raise TypeError(f"{type(struct).__name__} has no field {k!r}")
        setattr(struct, k, v)
    return struct


def default_options(**kw) -> Options:
    o = Options()
    lib().mprgp_default_options(C.byref(o))
    return _set_fields(o, kw)


# ----------------------------------------------------------------- beams --
@dataclass
class BeamQP:
    nv: int
    row_ptr: np.ndarray
    cols: np.ndarray
    vals: np.ndarray      # (nnzb, 9) row-major 3x3 blocks
    b: np.ndarray
    x0: np.ndarray        # rest shape shifted to y = -lift (not projected)
    plane_ptr: np.ndarray
    planes: np.ndarray    # (m, 4): n, p with n.x + p >= 0
    params: dict

    @property
    def n(self) -> int:
        return 3 * self.nv

    @property
    def nnzb(self) -> int:
        return int(self.row_ptr[-1])


def beam(a: int, b: int, c: int, **kw) -> BeamQP:
    """Synthetic implicit-Euler FEM beam QP (mprgp_beam_build)."""
    L = lib()
    p = BeamParams()
    L.mprgp_beam_default(C.byref(p))
    p.a, p.b, p.c = a, b, c
    _set_fields(p, kw)
    nv, nnzb, npl = C.c_int(), C.c_int(), C.c_int()
    _check(L.mprgp_beam_sizes(C.byref(p), C.byref(nv), C.byref(nnzb), C.byref(npl)), "beam_sizes")
    nv, nnzb, npl = nv.value, nnzb.value, npl.value
    row_ptr = np.zeros(nv + 1, np.int32)
    cols = np.zeros(nnzb, np.int32)
    vals = np.zeros((nnzb, 9), np.float64)
    rhs = np.zeros(3 * nv, np.float64)
    x0 = np.zeros(3 * nv, np.float64)
    pptr = np.zeros(nv + 1, np.int32)
    planes = np.zeros((npl, 4), np.float64)
    _check(L.mprgp_beam_build(C.byref(p), _ptr(row_ptr), _ptr(cols), _ptr(vals), _ptr(rhs),
                              _ptr(x0), _ptr(pptr), _ptr(planes)), "beam_build")
    params = {k: getattr(p, k) for k, _ in BeamParams._fields_}
    return BeamQP(nv, row_ptr, cols, vals, rhs, x0, pptr, planes, params)


def beam_mesh(a: int, b: int, c: int, **kw):
    """The tetrahedral mesh behind beam(a, b, c, **kw): (tets (6abc, 4) int32,
    rest shape X, initial positions x0, initial velocities v0), each 3 nv."""
    L = lib()
    p = BeamParams()
    L.mprgp_beam_default(C.byref(p))
    p.a, p.b, p.c = a, b, c
    _set_fields(p, kw)
    nv = (a + 1) * (b + 1) * (c + 1)
    tets = np.zeros((6 * a * b * c, 4), np.int32)
    X, x0, v0 = np.zeros(3 * nv), np.zeros(3 * nv), np.zeros(3 * nv)
    _check(L.mprgp_beam_mesh(C.byref(p), _ptr(tets), _ptr(X), _ptr(x0), _ptr(v0)), "beam_mesh")
    return tets, X, x0, v0


class FemMesh:
    """GPU assembly of A = M + h^2 K and b for a tetrahedral mesh (mprgp_fem_*)."""

    def __init__(self, ctx, tets, X, young, poisson, rho):
        self.ctx = ctx
        tets = np.ascontiguousarray(tets, np.int32)
        X = np.ascontiguousarray(X, np.float64)
        self.nv = X.size // 3
        self.h = C.c_void_p()
        _check(lib().mprgp_fem_create(ctx.h, self.nv, tets.shape[0], _ptr(tets), _ptr(X), young,
                                      poisson, rho, C.byref(self.h)), "fem_create")
        n, nnzb = C.c_int(), C.c_int()
        _check(lib().mprgp_fem_sizes(self.h, C.byref(n), C.byref(nnzb)), "fem_sizes")
        self.nnzb = nnzb.value

    def close(self):
        if self.h:
            lib().mprgp_fem_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def assemble(self, h, gravity, x, v=None, prob=None, precisions=1):
        """A and b on the device; with `prob`, loaded into it."""
        g = np.ascontiguousarray(gravity, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        _check(lib().mprgp_fem_assemble(self.h, h, _ptr(g), _ptr(x), _ptr(v), 0,
                                        prob.h if prob is not None else None, precisions),
               "fem_assemble")

    def rhs(self, h, gravity, x, v=None, prob=None):
        """b only (A unchanged), for a later timestep."""
        g = np.ascontiguousarray(gravity, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        _check(lib().mprgp_fem_rhs(self.h, h, _ptr(g), _ptr(x), _ptr(v), 0,
                                   prob.h if prob is not None else None), "fem_rhs")

    def get_b(self):
        """The right-hand side of the last assembly or rhs call (host copy)."""
        b = np.zeros(3 * self.nv)
        _check(lib().mprgp_fem_get(self.h, None, None, None, _ptr(b), None), "fem_get")
        return b

    def get(self):
        """(row_ptr, cols, vals (nnzb, 9), b, mass) of the last assembly."""
        rp = np.zeros(self.nv + 1, np.int32)
        cols = np.zeros(self.nnzb, np.int32)
        vals = np.zeros((self.nnzb, 9))
        b = np.zeros(3 * self.nv)
        mass = np.zeros(self.nv)
        _check(lib().mprgp_fem_get(self.h, _ptr(rp), _ptr(cols), _ptr(vals), _ptr(b), _ptr(mass)),
               "fem_get")
        return rp, cols, vals, b, mass


# ------------------------------------------------------------- contexts --
class Context:
    def __init__(self, device: int = 0):
        self.h = C.c_void_p()
        _check(lib().mprgp_context_create(device, C.byref(self.h)), "context_create")

    @property
    def stream(self) -> int:
        return lib().mprgp_context_stream(self.h) or 0

    def info(self):
        nsm, bps = C.c_int(), C.c_int()
        _check(lib().mprgp_context_info(self.h, C.byref(nsm), C.byref(bps)), "context_info")
        return nsm.value, bps.value

    def sync(self):
        _check(lib().mprgp_context_sync(self.h), "sync")

    def counters(self):
        """(kernels launched, device ms of solver runs, device ms of the power
        loop) since creation."""
        n, ms, pms = C.c_longlong(), C.c_double(), C.c_double()
        _check(lib().mprgp_context_counters(self.h, C.byref(n), C.byref(ms), C.byref(pms)),
               "context_counters")
        return n.value, ms.value, pms.value

    def set_cluster(self, cluster: int = 8):
        """CTAs per cluster of the small-instance solver (0 = engine only)."""
        _check(lib().mprgp_context_set_cluster(self.h, cluster), "set_cluster")

    def set_cluster_items(self, items: int = 1):
        """Items per CTA allowed in the largest cluster (1..4)."""
        _check(lib().mprgp_context_set_cluster_items(self.h, items), "set_cluster_items")

    def room(self) -> int:
        """Device bytes new problems of this context can take now."""
        b = C.c_size_t()
        _check(lib().mprgp_context_room(self.h, C.byref(b)), "context_room")
        return b.value

    def set_tuning(self, stage: int = 0, ctas_per_sm: int = 0):
        _check(lib().mprgp_context_set_tuning(self.h, stage, ctas_per_sm), "set_tuning")

    def close(self):
        if self.h:
            lib().mprgp_context_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_bsr(self, qp: BeamQP, opt: Options, x: np.ndarray, L=None, U=None, ev=None,
                  want_face=True):
        """One-call solve with host buffers (mprgp_solve_bsr)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        st = Stats()
        m = len(qp.planes) if opt.kind >= KIND_DECOUPLED else 3 * qp.nv
        face = np.zeros(max(m, 1), np.uint8) if want_face else None
        rc = lib().mprgp_solve_bsr(
            self.h, qp.nv, qp.nnzb, _ptr(qp.row_ptr), _ptr(qp.cols), _ptr(qp.vals), _ptr(qp.b),
            _ptr(qp.plane_ptr), _ptr(qp.planes), _ptr(L), _ptr(U), C.byref(opt), _ptr(x),
            _ptr(face), _ptr(ev), C.byref(st))
        _check(rc, "solve_bsr")
        return x, (face[:m] if face is not None else None), st

    def ica_solve(self, qp: BeamQP, x0, r=None, max_it=1000, tol=1e-4, gs_max_it=20,
                  gs_tol=1e-3):
        """The ICA contact solver (mprgp_ica_solve, the reference's ICASolver)
        on a beam QP: A x = r + J^T lambda, 0 <= lambda _|_ J x - c >= 0 with
        r = b by default.  Returns (x, lambda, IcaStats); a run that did not
        reach tol returns normally with stats.converged == 0."""
        x = np.ascontiguousarray(x0, np.float64).copy()
        lam = np.zeros(max(len(qp.planes), 1))
        rhs = np.ascontiguousarray(qp.b if r is None else r, np.float64)
        st = IcaStats()
        _check(lib().mprgp_ica_solve(self.h, qp.nv, qp.nnzb, _ptr(qp.row_ptr), _ptr(qp.cols),
                                     _ptr(qp.vals), _ptr(rhs), _ptr(qp.plane_ptr), _ptr(qp.planes),
                                     _ptr(x), _ptr(lam), max_it, tol, gs_max_it, gs_tol,
                                     C.byref(st)), "ica_solve")
        return x, lam[:len(qp.planes)], st

    def solve_batch(self, probs, opts):
        n = len(probs)
        arr = (C.c_void_p * n)(*[p.h for p in probs])
        oarr = (Options * n)(*opts)
        sarr = (Stats * n)()
        _check(lib().mprgp_solve_batch(self.h, n, arr, oarr, sarr), "solve_batch")
        return [sarr[i] for i in range(n)]


class Problem:
    """One resident QP instance (mprgp_problem)."""

    def __init__(self, ctx: Context, nv: int):
        self.ctx = ctx
        self.nv = nv
        self.h = C.c_void_p()
        _check(lib().mprgp_problem_create(ctx.h, nv, C.byref(self.h)), "problem_create")

    def close(self):
        if self.h:
            lib().mprgp_problem_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_matrix(self, row_ptr, cols, vals, precisions=1):
        """Host BSR arrays; precisions bit 0 = FP64 copy, bit 1 = FP32 copy."""
        row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        _check(lib().mprgp_problem_set_matrix(self.h, int(row_ptr[-1]), _ptr(row_ptr), _ptr(cols),
                                              _ptr(vals), precisions, 0), "set_matrix")

    def set_matrix_device(self, nnzb, row_ptr_dev, cols_dev, vals_dev, precisions=1):
        """Device BSR arrays (raw device pointers)."""
        _check(lib().mprgp_problem_set_matrix(self.h, nnzb, C.c_void_p(row_ptr_dev),
                                              C.c_void_p(cols_dev), C.c_void_p(vals_dev),
                                              precisions, 1), "set_matrix_device")

    def set_rhs(self, b):
        _check(lib().mprgp_problem_set_rhs(self.h, _ptr(np.ascontiguousarray(b, np.float64)), 0),
               "set_rhs")

    def set_planes(self, plane_ptr, planes):
        _check(lib().mprgp_problem_set_planes(self.h, _ptr(plane_ptr), _ptr(planes), 0),
               "set_planes")

    def set_bounds(self, L, U=None):
        _check(lib().mprgp_problem_set_bounds(self.h, _ptr(L), _ptr(U)), "set_bounds")

    def set_x(self, x, on_device=False):
        if on_device:
            _check(lib().mprgp_problem_set_x(self.h, C.c_void_p(x), 1), "set_x")
        else:
            _check(lib().mprgp_problem_set_x(self.h, _ptr(np.ascontiguousarray(x, np.float64)), 0),
                   "set_x")

    def get_x(self) -> np.ndarray:
        x = np.zeros(3 * self.nv, np.float64)
        _check(lib().mprgp_problem_get_x(self.h, _ptr(x), 0), "get_x")
        return x

    def get_face(self) -> np.ndarray:
        m = C.c_int()
        _check(lib().mprgp_problem_num_constraints(self.h, C.byref(m)), "num_constraints")
        f = np.zeros(max(m.value, 1), np.uint8)
        _check(lib().mprgp_problem_get_face(self.h, _ptr(f)), "get_face")
        return f[:m.value]

    def get_planes(self):
        """(plane_ptr, planes (m, 4)) as set, in the (n, p) form."""
        m = C.c_int()
        _check(lib().mprgp_problem_num_constraints(self.h, C.byref(m)), "num_constraints")
        ptr = np.zeros(self.nv + 1, np.int32)
        planes = np.zeros((max(m.value, 1), 4))
        _check(lib().mprgp_problem_get_planes(self.h, _ptr(ptr), _ptr(planes)), "get_planes")
        return ptr, planes[:m.value]

    def collide_planes(self, planes, delta, decoupled=False, x=None) -> int:
        """Replaces the constraints by the planes (n, p) within `delta` of the
        vertices at x (default: the problem's current x); returns their count."""
        pl = np.ascontiguousarray(planes, np.float64).reshape(-1, 4)
        xx = None if x is None else np.ascontiguousarray(x, np.float64)
        m = C.c_int()
        _check(lib().mprgp_planes_collide(self.ctx.h, self.h, _ptr(xx), 0, pl.shape[0], _ptr(pl),
                                          delta, int(bool(decoupled)), C.byref(m)),
               "planes_collide")
        return m.value

    def set_power_cache(self, enable: bool):
        _check(lib().mprgp_problem_set_power_cache(self.h, int(bool(enable))), "set_power_cache")

    def set_ev(self, ev):
        _check(lib().mprgp_problem_set_ev(self.h, _ptr(ev)), "set_ev")

    def get_ev(self):
        ev = np.zeros(3 * self.nv, np.float64)
        valid = C.c_int()
        _check(lib().mprgp_problem_get_ev(self.h, _ptr(ev), C.byref(valid)), "get_ev")
        return ev if valid.value else None

    def set_trace(self, capacity: int):
        _check(lib().mprgp_problem_set_trace(self.h, capacity), "set_trace")

    def get_trace(self) -> np.ndarray:
        n = C.c_int()
        _check(lib().mprgp_problem_get_trace(self.h, None, 0, C.byref(n)), "get_trace")
        out = np.zeros((max(n.value, 1), 4))
        _check(lib().mprgp_problem_get_trace(self.h, _ptr(out), n.value, C.byref(n)), "get_trace")
        return out[:n.value]

    def solve(self, opt: Options) -> Stats:
        st = Stats()
        _check(lib().mprgp_problem_solve(self.h, C.byref(opt), C.byref(st)), "problem_solve")
        return st

    def spmv(self, x_dev: int, y_dev: int, precision=PREC_FP64):
        _check(lib().mprgp_problem_spmv(self.h, C.c_void_p(x_dev), C.c_void_p(y_dev), precision),
               "spmv")


def load_beam(ctx: Context, qp: BeamQP, precisions=1) -> Problem:
    pr = Problem(ctx, qp.nv)
    pr.set_planes(qp.plane_ptr, qp.planes)  # first: the matrix layout then builds once
    pr.set_matrix(qp.row_ptr, qp.cols, qp.vals, precisions)
    pr.set_rhs(qp.b)
    pr.set_x(qp.x0)
    return pr


class Server:
    """Continuous-batching QP server (mprgp_server_*)."""

    def __init__(self, ctx: Context, hbm_budget=0, max_slots=0, quantum_phases=0,
                 power_launches=256, cluster_quantum=0, lanes=0, hbm_reserve=0):
        self.ctx = ctx
        cfg = ServerConfig(hbm_budget, max_slots, quantum_phases, power_launches, cluster_quantum,
                           lanes, hbm_reserve)
        self.h = C.c_void_p()
        _check(lib().mprgp_server_create(ctx.h, C.byref(cfg), C.byref(self.h)), "server_create")
        self.nv = {}

    def close(self):
        if self.h:
            lib().mprgp_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scene: int, qp: BeamQP, opt: Options, b=None, followup=False) -> int:
        """Host-memory request: a new scene (qp) or, with followup=True, the
        next timestep of `scene` with right-hand side b."""
        t = C.c_longlong()
        rhs = np.ascontiguousarray(qp.b if b is None else b, np.float64)
        if followup:
            _check(lib().mprgp_server_submit(self.h, scene, qp.nv, 0, None, None, None, _ptr(rhs),
                                             None, None, None, -1, 0, C.byref(opt), C.byref(t)),
                   "server_submit")
        else:
            _check(lib().mprgp_server_submit(self.h, scene, qp.nv, qp.nnzb, _ptr(qp.row_ptr),
                                             _ptr(qp.cols), _ptr(qp.vals), _ptr(rhs),
                                             _ptr(qp.plane_ptr), _ptr(qp.planes), _ptr(qp.x0),
                                             len(qp.planes), 0, C.byref(opt), C.byref(t)),
                   "server_submit")
        self.nv[t.value] = (qp.nv, len(qp.planes))
        return t.value

    def submit_ref(self, scene: int, nv: int, nnzb: int, m: int, opt: Options, b: int,
                   row_ptr=0, cols=0, vals=0, plane_ptr=0, planes=0, x0=0,
                   on_device=True) -> int:
        """By-reference request from raw pointers (device memory, or host
        memory with on_device=False) that the caller keeps valid until the
        request completes; row_ptr == 0 makes it a follow-up of `scene`."""
        t = C.c_longlong()
        P = C.c_void_p
        mode = 1 if on_device else 2
        if not row_ptr:
            _check(lib().mprgp_server_submit(self.h, scene, nv, 0, None, None, None, P(b), None,
                                             None, None, m, mode, C.byref(opt), C.byref(t)),
                   "server_submit")
        else:
            _check(lib().mprgp_server_submit(self.h, scene, nv, nnzb, P(row_ptr), P(cols),
                                             P(vals), P(b), P(plane_ptr), P(planes), P(x0), m,
                                             mode, C.byref(opt), C.byref(t)), "server_submit")
        self.nv[t.value] = (nv, m)
        return t.value

    def poll(self, capacity=4096):
        """Tickets completed since the last poll."""
        arr = (C.c_longlong * capacity)()
        n = C.c_int()
        _check(lib().mprgp_server_poll(self.h, arr, capacity, C.byref(n)), "server_poll")
        return [arr[i] for i in range(n.value)]

    def step(self):
        r, q, c = C.c_int(), C.c_int(), C.c_int()
        _check(lib().mprgp_server_step(self.h, C.byref(r), C.byref(q), C.byref(c)), "server_step")
        return r.value, q.value, c.value

    def result(self, ticket: int):
        """(state, x, face, stats, times) -- x etc. are None until state == 2."""
        nv, m = self.nv[ticket]
        x = np.zeros(3 * nv)
        face = np.zeros(max(m, 1), np.uint8)
        st = Stats()
        times = np.zeros(3)
        state = C.c_int()
        rc = lib().mprgp_server_result(self.h, ticket, _ptr(x), _ptr(face), C.byref(st),
                                       _ptr(times), C.byref(state))
        if state.value != 2:
            return state.value, None, None, None, None
        _check(rc, "server_result")
        del self.nv[ticket]
        return 2, x, face[:m], st, times

    def info(self):
        b, u, n = C.c_size_t(), C.c_size_t(), C.c_int()
        _check(lib().mprgp_server_info(self.h, C.byref(b), C.byref(u), C.byref(n)), "server_info")
        return b.value, u.value, n.value


def solve_noalloc(stream: int, nv: int, nnzb: int, row_ptr: int, cols: int, vals: int, b: int,
                  plane_ptr: int, planes: int, opt: Options, x: int, face: int = 0):
    """mprgp_solve_noalloc with raw device pointers; returns (code, Stats)."""
    st = Stats()
    rc = lib().mprgp_solve_noalloc(C.c_void_p(stream), nv, nnzb, C.c_void_p(row_ptr),
                                   C.c_void_p(cols), C.c_void_p(vals), C.c_void_p(b),
                                   C.c_void_p(plane_ptr), C.c_void_p(planes), C.byref(opt),
                                   C.c_void_p(x), C.c_void_p(face or None), C.byref(st))
    return _check(rc, "solve_noalloc"), st


# ---------------------------------------------------------- conversions --
def bsr_to_csr(nv, row_ptr, cols, vals):
    """3x3-block CSR -> scalar CSR (rows 3v+i, columns sorted)."""
    nnzb = int(row_ptr[-1])
    blk_len = np.diff(row_ptr)
    vals = np.asarray(vals).reshape(nnzb, 3, 3)
    ptr = np.zeros(3 * nv + 1, np.int64)
    ptr[1:] = np.repeat(3 * blk_len, 3).cumsum()
    idx = np.empty(9 * nnzb, np.int32)
    val = np.empty(9 * nnzb, np.float64)
    brow = np.repeat(np.arange(nv), blk_len)
    # position of each block within its row
    pos = np.arange(nnzb) - row_ptr[brow]
    for i in range(3):
        base = ptr[3 * brow + i] + 3 * pos
        for j in range(3):
            idx[base + j] = 3 * cols + j
            val[base + j] = vals[:, i, j]
    return ptr.astype(np.int32), idx, val


def planes_to_J(nv, plane_ptr, planes):
    """Per-vertex planes (n, p) -> (J CSR, c) with J x >= c, c = -p (MPRGPUtility.h:120-154)."""
    m = len(planes)
    vert = np.repeat(np.arange(nv), np.diff(plane_ptr))
    jptr = (3 * np.arange(m + 1)).astype(np.int32)
    jidx = (3 * vert[:, None] + np.arange(3)[None, :]).reshape(-1).astype(np.int32)
    jval = np.asarray(planes)[:, :3].reshape(-1).astype(np.float64)
    c = -np.asarray(planes)[:, 3].astype(np.float64)
    return jptr, jidx, jval, c
