"""Regenerates the golden QP fixtures in this directory.

Each fixture is a small seeded beam QP (3x3-block A, b, x0, planes or
bounds) together with its exact solution from QuadProg++ -- the dense
active-set solver the reference vendors (src/MPRGPSolver/SimpleQP/) and uses
inside GeneralConProjector -- built from the reference's own sources into
oracle/_ref by oracle/build_ref.sh.  The fixtures let tests on machines
without the reference tree (the GPU host) check solutions against it.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import helpers as H  # noqa: E402
import mprgp_gb300 as M  # noqa: E402

CASES = {
    # name: beam kwargs (plane cases) or ("bounds", beam kwargs)
    "corner_2x2x4": dict(a=2, b=2, c=4, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=11),
    "floor_3x2x5": dict(a=3, b=2, c=5, seed=12),
    "tilted_2x2x5": dict(a=2, b=2, c=5, extra_planes_max=2, extra_planes_min=2, plane_mode=0,
                         seed=8),
    "bounds_2x3x4": ("bounds", dict(a=2, b=3, c=4, seed=13)),
}


def bounds_of(qp):
    n = qp.n
    L = np.full(n, -1e30)
    L[1::3] = 0.0
    U = np.full(n, 1e30)
    U[0::3] = qp.x0[0::3] + 0.0005
    return L, U


def main():
    if H.quadprog_ref() is None:
        sys.exit("oracle/_ref/libquadprog_ref.so missing: run oracle/build_oracle.sh with the "
                 "reference tree present")
    for name, spec in CASES.items():
        bounds = isinstance(spec, tuple)
        kw = dict(spec[1] if bounds else spec)
        a, b_, c_ = kw.pop("a"), kw.pop("b"), kw.pop("c")
        qp = M.beam(a, b_, c_, **kw)
        A, b, J, c = H.qp_from_beam(qp)
        Ad = A.dense()
        out = dict(nv=qp.nv, row_ptr=qp.row_ptr, cols=qp.cols, vals=qp.vals, b=qp.b, x0=qp.x0,
                   plane_ptr=qp.plane_ptr, planes=qp.planes)
        if bounds:
            L, U = bounds_of(qp)
            fin_l = L > -1e29
            fin_u = U < 1e29
            Jd = np.vstack([np.eye(qp.n)[fin_l], -np.eye(qp.n)[fin_u]])
            cd = np.concatenate([L[fin_l], -U[fin_u]])
            out.update(L=L, U=U)
        else:
            Jd = J.dense()
            cd = c
        x, f = H.solve_qp_ref(Ad, b, Jd, cd)
        assert np.isfinite(f), name
        out["x_qp"] = x
        out["f_qp"] = f
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "n", qp.n, "constraints", len(cd), "active",
              int((np.abs(Jd @ x - cd) < 1e-9).sum()), "f", f)


if __name__ == "__main__":
    main()
