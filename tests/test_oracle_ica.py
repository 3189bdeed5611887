"""CPU tests of the ICA restatement (oracle/ica_oracle.h, the reference's
ICASolver.h:287-463).  ICA solves the KKT system of the same QP as MPRGP
(A x = b + J^T lambda, 0 <= lambda _|_ J x - c >= 0), so its converged
solution is pinned by
  * the golden fixtures' QuadProg++ solutions (the reference's own dense QP
    solver, tests/golden/),
  * the MPRGP restatement's solution of the same QP,
  * the KKT conditions, and the properties the reference's comparison test
    logs (test_case/MPRGP_ICA_Compare.cpp:69-82: residual <= tol,
    lambda >= 0, complementarity lambda . (J x - p) ~ 0).
"""
import glob
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import helpers as H
import mprgp_gb300 as M

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if "L" not in np.load(p).files)  # plane fixtures (ICA takes planes)


def _mats(qp):
    A, b, J, c = H.qp_from_beam(qp)
    As = sp.csr_matrix((A.val, A.idx, A.ptr), shape=(A.rows, A.cols))
    Js = sp.csr_matrix((J.val, J.idx, J.ptr), shape=(J.rows, J.cols))
    return As, b, Js, c


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_ica_matches_golden_quadprog(path):
    d = np.load(path)
    qp = M.BeamQP(int(d["nv"]), d["row_ptr"], d["cols"], d["vals"], d["b"], d["x0"],
                  d["plane_ptr"], d["planes"], {})
    As, b, Js, c = _mats(qp)
    x0 = spl.spsolve(As.tocsc(), b)  # the reference's FEM loop starts ICA from the unconstrained solve
    x, lam, st = H.oracle_ica(qp, x0, max_it=100000, tol=1e-11 * np.linalg.norm(b),
                              gs_max_it=20, gs_tol=1e-14)
    assert st["converged"] == 1 and st["code"] == 0
    assert np.linalg.norm(x - d["x_qp"]) <= 1e-8 * np.linalg.norm(d["x_qp"])
    J, cc = H.qp_from_beam(qp)[2:]
    assert np.array_equal(H.decide_face_planes(J, cc, x), H.decide_face_planes(J, cc, d["x_qp"]))


@pytest.mark.parametrize("dims,extra,seed", [((3, 2, 5), 0, 4), ((3, 3, 4), 2, 7),
                                             ((2, 2, 6), 1, 11)])
def test_ica_kkt_and_mprgp_agree(dims, extra, seed):
    qp = M.beam(*dims, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2, seed=seed)
    As, b, Js, c = _mats(qp)
    nb = np.linalg.norm(b)
    x0 = spl.spsolve(As.tocsc(), b)
    x, lam, st = H.oracle_ica(qp, x0, max_it=100000, tol=1e-11 * nb, gs_max_it=20, gs_tol=1e-14)
    assert st["converged"] == 1
    # the loop's own residual, recomputed
    assert np.linalg.norm(As @ x - b - Js.T @ lam) == pytest.approx(st["residual"], rel=1e-6)
    assert lam.min() >= 0.0
    assert (Js @ x - c).min() >= -1e-9
    assert abs(lam @ (Js @ x - c)) <= 1e-10 * nb
    A, bb, J, cc = H.qp_from_beam(qp)
    xm, _, sm, _ = H.oracle_solve("general", A, bb, qp.x0, J, cc, tol=1e-11 * nb, max_it=20000)
    assert sm["code"] == 0
    assert np.linalg.norm(x - xm) <= 1e-8 * np.linalg.norm(xm)


def test_ica_reference_defaults_and_iteration_count():
    """ICASolver(max_it, tol) keeps gs_max_it = 20, gs_tol = 1e-3 (ICASolver.h:290);
    `iterations` is the index of the converging iteration (:361-393)."""
    qp = M.beam(3, 2, 5, extra_planes_max=1, extra_planes_min=1, plane_mode=2, seed=4)
    As, b, Js, c = _mats(qp)
    x0 = spl.spsolve(As.tocsc(), b)
    x, lam, st = H.oracle_ica(qp, x0, max_it=1000, tol=1e-4)
    assert st["converged"] == 1 and st["residual"] <= 1e-4
    k = st["iterations"]
    # one iteration fewer does not converge; stopping at k + 1 iterations
    # reproduces the same x (the loop ended at index k)
    _, _, st2 = H.oracle_ica(qp, x0, max_it=k, tol=1e-4)
    assert st2["converged"] == 0 and st2["iterations"] == k
    x3, lam3, st3 = H.oracle_ica(qp, x0, max_it=k + 1, tol=1e-4)
    assert st3["converged"] == 1 and np.array_equal(x3, x) and np.array_equal(lam3, lam)


def test_ica_zero_iterations_leaves_x():
    qp = M.beam(2, 2, 3, seed=2)
    x, lam, st = H.oracle_ica(qp, qp.x0, max_it=0, tol=1e-4)
    assert st["iterations"] == 0 and st["converged"] == 0
    assert np.array_equal(x, qp.x0) and not lam.any()
