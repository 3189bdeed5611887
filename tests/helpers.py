"""Test-side bindings: the CPU oracle (oracle/), the QuadProg++ pin
(oracle/_ref/) and problem conversions.  Only tests, bench.py's CPU leg and
__graft_entry__.smoke() use these."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
QP_REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libquadprog_ref.so")

_orc = None
_qp = None
_P = C.c_void_p


def build_oracle() -> None:
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_oracle.sh")], check=True,
                   capture_output=True)


def oracle():
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_LIB) or _stale(ORACLE_LIB):
            build_oracle()
        L = C.CDLL(ORACLE_LIB)
        L.oracle_solve.restype = C.c_int
        L.oracle_solve.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int, _P, _P, _P,
                                   _P, _P, _P, C.c_double, C.c_int, C.c_uint64, _P, C.c_int,
                                   C.c_int, _P, _P, _P]
        L.oracle_projector_op.restype = C.c_int
        L.oracle_projector_op.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P,
                                          _P, _P, C.c_double, _P, _P]
        L.oracle_spmv.restype = None
        L.oracle_spmv.argtypes = [C.c_int, _P, _P, _P, _P, _P]
        L.oracle_spec_rad.restype = C.c_double
        L.oracle_spec_rad.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_uint64,
                                      C.POINTER(C.c_int)]
        L.oracle_set_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_seeded_uniform.restype = C.c_double
        L.oracle_seeded_uniform.argtypes = [C.c_uint64, C.c_uint64]
        L.oracle_ica_solve.restype = C.c_int
        L.oracle_ica_solve.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, C.c_int, C.c_double,
                                       C.c_int, C.c_double, _P]
        L.oracle_solve_warm.restype = C.c_int
        L.oracle_solve_warm.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, C.c_int, _P, _P, _P, _P,
                                        C.c_double, C.c_int, C.c_uint64, _P, _P, C.c_int, _P, _P,
                                        _P]
        L.oracle_set_scalar_test.restype = None
        L.oracle_set_scalar_test.argtypes = [C.c_int]
        L.oracle_beam_new.restype = C.c_void_p
        L.oracle_beam_new.argtypes = [_P, _P, C.c_uint64, _P, _P, _P]
        L.oracle_beam_take.restype = None
        L.oracle_beam_take.argtypes = [C.c_void_p, _P, _P, _P, _P, _P, _P, _P]
        _orc = L
    return _orc


def _stale(lib_path: str) -> bool:
    t = os.path.getmtime(lib_path)
    d = os.path.join(ROOT, "oracle")
    return any(os.path.getmtime(os.path.join(d, f)) > t for f in os.listdir(d)
               if f.endswith((".h", ".cpp")))


def quadprog_ref():
    """The reference's own QuadProg++ (built from its sources), or None."""
    global _qp
    if _qp is None:
        if not os.path.exists(QP_REF_LIB):
            # the recipe finds the reference tree (MPRGP_REFERENCE_ROOT) or skips
            subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True,
                           capture_output=True)
        if not os.path.exists(QP_REF_LIB):
            return None
        L = C.CDLL(QP_REF_LIB)
        L.ref_solve_qp.restype = C.c_double
        L.ref_solve_qp.argtypes = [C.c_int, _P, _P, C.c_int, _P, _P, _P]
        _qp = L
    return _qp


def ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def solve_qp_ref(A, b, J, c0):
    """min 0.5 x^T A x - b^T x  s.t.  J x >= c0 with the reference's QuadProg++."""
    L = quadprog_ref()
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    J = np.ascontiguousarray(J, np.float64).reshape(-1, len(b))
    c0 = np.ascontiguousarray(c0, np.float64)
    x = np.zeros(len(b))
    f = L.ref_solve_qp(len(b), ptr(A), ptr(b), J.shape[0], ptr(J), ptr(c0), ptr(x))
    return x, f


class Csr:
    def __init__(self, ptr_, idx, val, rows, cols):
        self.ptr = np.ascontiguousarray(ptr_, np.int32)
        self.idx = np.ascontiguousarray(idx, np.int32)
        self.val = np.ascontiguousarray(val, np.float64)
        self.rows, self.cols = rows, cols

    @staticmethod
    def from_dense(M):
        M = np.asarray(M, np.float64)
        rows, cols = M.shape
        ptr_, idx, val = [0], [], []
        for r in range(rows):
            nz = np.nonzero(M[r])[0]
            idx.extend(nz.tolist())
            val.extend(M[r, nz].tolist())
            ptr_.append(len(idx))
        return Csr(ptr_, idx, val, rows, cols)

    def dense(self):
        M = np.zeros((self.rows, self.cols))
        for r in range(self.rows):
            for k in range(self.ptr[r], self.ptr[r + 1]):
                M[r, self.idx[k]] += self.val[k]
        return M

    def matvec(self, x):
        y = np.zeros(self.rows)
        rows = np.repeat(np.arange(self.rows), np.diff(self.ptr))
        np.add.at(y, rows, self.val * x[self.idx])
        return y


STAT_KEYS = ["code", "iterations", "num_cg", "num_exp", "num_prop", "power_iters", "residual",
             "alpha_bar", "spec_rad", "spmv"]

KIND = {"lower": 0, "box": 1, "decoupled": 2, "general": 3,
        "plain_lower": 10, "plain_decoupled": 12, "plain_general": 13}


def oracle_solve(kind, A: Csr, b, x, J: Csr | None = None, c=None, L=None, U=None, tol=1e-3,
                 max_it=1000, seed=0x5EED, preconditioned=True, project_x0=True, ev=None):
    """Runs the restated reference solve; returns (x, face, stats dict, ev)."""
    O = oracle()
    n = A.rows
    x = np.ascontiguousarray(x, np.float64).copy()
    st = np.zeros(10)
    kind_i = KIND[kind] if isinstance(kind, str) else kind
    m = J.rows if J is not None else n
    face = np.zeros(max(m, 1), np.uint8)
    if J is None:
        J = Csr([0], [], [], 0, n)
        c = np.zeros(0)
    evbuf = None if ev is None else np.ascontiguousarray(ev, np.float64).copy()
    code = O.oracle_solve(kind_i, int(preconditioned), n, ptr(A.ptr), ptr(A.idx), ptr(A.val),
                          ptr(np.ascontiguousarray(b, np.float64)), J.rows, ptr(J.ptr),
                          ptr(J.idx), ptr(J.val), ptr(np.ascontiguousarray(c, np.float64)),
                          ptr(None if L is None else np.ascontiguousarray(L, np.float64)),
                          ptr(None if U is None else np.ascontiguousarray(U, np.float64)),
                          tol, max_it, seed, ptr(evbuf), 0 if evbuf is None else len(evbuf),
                          int(project_x0), ptr(x), ptr(face), ptr(st))
    stats = dict(zip(STAT_KEYS, st.tolist()))
    stats["code"] = code
    return x, face[:m], stats, evbuf


def oracle_solve_warm(kind, A: Csr, b, x, J: Csr, c, ev=None, tol=1e-3, max_it=1000,
                      seed=0x5EED, project_x0=True):
    """The restated solve with MprgpFemSolver's power-method warm start
    (MprgpFemSolver.cpp:533 passes &power_ev): `ev` is the stored vector or
    None.  Returns (x, face, stats dict, ev or None)."""
    O = oracle()
    n = A.rows
    x = np.ascontiguousarray(x, np.float64).copy()
    st = np.zeros(10)
    face = np.zeros(max(J.rows, 1), np.uint8)
    evbuf = np.zeros(n) if ev is None else np.ascontiguousarray(ev, np.float64).copy()
    valid = C.c_int(0 if ev is None else 1)
    code = O.oracle_solve_warm(KIND[kind] if isinstance(kind, str) else kind, n, ptr(A.ptr),
                               ptr(A.idx), ptr(A.val), ptr(np.ascontiguousarray(b, np.float64)),
                               J.rows, ptr(J.ptr), ptr(J.idx), ptr(J.val),
                               ptr(np.ascontiguousarray(c, np.float64)), tol, max_it, seed,
                               ptr(evbuf), C.byref(valid), int(project_x0), ptr(x), ptr(face),
                               ptr(st))
    stats = dict(zip(STAT_KEYS, st.tolist()))
    stats["code"] = code
    return x, face[:J.rows], stats, (evbuf if valid.value else None)


def oracle_scalar_test(on: bool):
    """Switches the oracle's monotone CG test to the scalar form the GPU
    evaluates (on) or back to the reference's comparison of f values."""
    oracle().oracle_set_scalar_test(int(on))


# Defaults of the synthetic beam (the library's mprgp_beam_default).
BEAM_DEFAULTS = dict(edge=0.05, young=1e5, poisson=0.45, rho=1000.0, dt=0.01, gravity=-9.8,
                     lift=0.01, v0_sigma=0.1, extra_planes_max=0, extra_planes_min=0,
                     active_frac=1.0, seed=1, plane_band=0.025, max_tilt=1.5707963267948966,
                     plane_mode=2, facet_layers=1)


def oracle_beam(a: int, b: int, c: int, **kw):
    """The synthetic beam QP built by the oracle's generator (beam_oracle.h),
    with the library's keyword names; returns a mprgp_gb300.BeamQP without
    loading the GPU library."""
    from mprgp_gb300 import BeamQP
    p = dict(BEAM_DEFAULTS)
    unknown = set(kw) - set(p)
    if unknown:
        raise TypeError(f"unknown beam parameters {sorted(unknown)}")
    p.update(kw)
    ip = np.array([a, b, c, p["extra_planes_max"], p["extra_planes_min"], p["plane_mode"],
                   p["facet_layers"]], np.int32)
    dp = np.array([p[k] for k in ("edge", "young", "poisson", "rho", "dt", "gravity", "lift",
                                  "v0_sigma", "active_frac", "plane_band", "max_tilt")], np.float64)
    O = oracle()
    nv, nnzb, npl = C.c_int(), C.c_int(), C.c_int()
    h = O.oracle_beam_new(ptr(ip), ptr(dp), int(p["seed"]), C.byref(nv), C.byref(nnzb),
                          C.byref(npl))
    if not h:
        raise ValueError(f"invalid beam parameters {a}x{b}x{c} {kw}")
    nv, nnzb, npl = nv.value, nnzb.value, npl.value
    row_ptr = np.zeros(nv + 1, np.int32)
    cols = np.zeros(nnzb, np.int32)
    vals = np.zeros((nnzb, 9))
    rhs, x0 = np.zeros(3 * nv), np.zeros(3 * nv)
    pptr = np.zeros(nv + 1, np.int32)
    planes = np.zeros((npl, 4))
    O.oracle_beam_take(h, ptr(row_ptr), ptr(cols), ptr(vals), ptr(rhs), ptr(x0), ptr(pptr),
                       ptr(planes))
    params = dict(p, a=a, b=b, c=c)
    return BeamQP(nv, row_ptr, cols, vals, rhs, x0, pptr, planes, params)


def qp_from_beam(qp):
    """(A CSR, b, J CSR, c) of a mprgp_gb300.BeamQP in the reference's (A, B, J, c) form."""
    import mprgp_gb300 as M
    aptr, aidx, aval = M.bsr_to_csr(qp.nv, qp.row_ptr, qp.cols, qp.vals)
    A = Csr(aptr, aidx, aval, qp.n, qp.n)
    jptr, jidx, jval, c = M.planes_to_J(qp.nv, qp.plane_ptr, qp.planes)
    J = Csr(jptr, jidx, jval, len(c), qp.n)
    return A, qp.b.copy(), J, c


def decide_face_planes(J: Csr, c, x, eps=1e-9):
    """DECIDE_FACE (MPRGPProjection.h:283-297) evaluated on the host."""
    return (np.abs(J.matvec(x) - c) < eps).astype(np.uint8)


def projected_gradient_norm(kind, A: Csr, b, x, J: Csr, c):
    """||phi + beta|| at x with a freshly decided face, via the oracle's projector."""
    O = oracle()
    g = A.matvec(x) - b
    n = A.rows
    phi = np.zeros(n)
    beta = np.zeros(n)
    kind_i = KIND[kind] % 10
    O.oracle_projector_op(kind_i, 2, n, J.rows, ptr(J.ptr), ptr(J.idx), ptr(J.val), ptr(c),
                          ptr(x), ptr(g), None, 0.0, ptr(phi), None)
    O.oracle_projector_op(kind_i, 3, n, J.rows, ptr(J.ptr), ptr(J.idx), ptr(J.val), ptr(c),
                          ptr(x), ptr(g), ptr(phi), 0.0, ptr(beta), None)
    return float(np.linalg.norm(phi + beta))


def oracle_trace(on: bool):
    O = oracle()
    O.oracle_set_trace.argtypes = [C.c_int]
    O.oracle_set_trace(int(on))


def oracle_get_trace() -> np.ndarray:
    O = oracle()
    O.oracle_get_trace.restype = C.c_int
    O.oracle_get_trace.argtypes = [_P, C.c_int]
    n = O.oracle_get_trace(None, 0)
    out = np.zeros((max(n, 1), 4))
    O.oracle_get_trace(ptr(out), n)
    return out[:n]


def collide_planes(x, planes, delta, decoupled=False):
    """CPU restatement of LinearConCollider::handle(body, plane, delta)
    (LinearConCollider.cpp:140-161) over a list of planes, with
    GeomConCache::addConPlane's 1e-4 duplicate test (:43-56) and the
    decoupled one-plane-per-vertex rule (:153-158).  Expressions are
    evaluated left to right in plain FP64.  Returns (plane_ptr, planes)."""
    import math
    nv = len(x) // 3
    ptr, out = [0], []
    for v in range(nv):
        xv = [float(x[3 * v]), float(x[3 * v + 1]), float(x[3 * v + 2])]
        mine = []
        for pl in planes:
            pl = [float(t) for t in pl]
            s = pl[0] * xv[0]
            s = s + pl[1] * xv[1]
            s = s + pl[2] * xv[2]
            s = s + pl[3]
            s = s - delta
            if not s <= 0.0:
                continue
            dup = False
            for q in mine:
                acc = 0.0
                for k in range(4):
                    d = q[k] - pl[k]
                    acc = acc + d * d
                dup = dup or math.sqrt(acc) <= 1e-4
            if dup:
                continue
            mine.append(pl)
            if decoupled:
                break
        out.extend(mine)
        ptr.append(len(out))
    return np.asarray(ptr, np.int32), np.asarray(out, np.float64).reshape(-1, 4)


def oracle_ica(qp, x0, r=None, max_it=1000, tol=1e-4, gs_max_it=20, gs_tol=1e-3):
    """The restated reference ICA solver (ICASolver.h:287-393) on a beam QP:
    A x = r + J^T lambda, 0 <= lambda _|_ J x - c >= 0.  Returns
    (x, lambda, stats dict)."""
    O = oracle()
    x = np.ascontiguousarray(x0, np.float64).copy()
    lam = np.zeros(max(len(qp.planes), 1))
    st = np.zeros(4)
    rhs = np.ascontiguousarray(qp.b if r is None else r, np.float64)
    code = O.oracle_ica_solve(qp.nv, ptr(qp.row_ptr), ptr(qp.cols), ptr(qp.vals), ptr(rhs),
                              ptr(qp.plane_ptr), ptr(qp.planes), ptr(x), ptr(lam), max_it, tol,
                              gs_max_it, gs_tol, ptr(st))
    return x, lam[:len(qp.planes)], {"code": code, "iterations": int(st[0]),
                                     "converged": int(st[1]), "residual": float(st[2]),
                                     "pgs_sweeps": int(st[3])}
