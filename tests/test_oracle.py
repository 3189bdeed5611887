"""CPU tests of the oracle (tests/helpers + oracle/): the restatement of the
reference MPRGP is pinned against
  * the reference's own unit-test properties (test_case/MPRGPTest.cpp),
  * QuadProg++ built from the reference's sources (oracle/_ref; skipped
    where the reference tree is absent),
  * golden fixtures holding QuadProg++ solutions (tests/golden/),
  * the KKT conditions of the QP.
"""
import glob
import os

import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def need_qp():
    if H.quadprog_ref() is None:
        pytest.skip("reference QuadProg++ (oracle/_ref) not built here")


def proj_op(kind, op, J, c, x, g=None, phi=None, alpha=0.0):
    O = H.oracle()
    n = J.cols
    out = np.zeros(max(n, 1))
    face = np.zeros(max(J.rows, 1), np.uint8)
    O.oracle_projector_op(kind, op, n, J.rows, H.ptr(J.ptr), H.ptr(J.idx), H.ptr(J.val),
                          H.ptr(np.ascontiguousarray(c, np.float64)),
                          H.ptr(np.ascontiguousarray(x, np.float64)),
                          H.ptr(None if g is None else np.ascontiguousarray(g, np.float64)),
                          H.ptr(None if phi is None else np.ascontiguousarray(phi, np.float64)),
                          alpha, H.ptr(out), H.ptr(face))
    return out[:n], face[:J.rows]


@pytest.mark.parametrize("m", [0, 1])
def test_projector_decoupled_equals_general(m):
    """test_case/MPRGPTest.cpp:11-68: on J = Identity(m, n) the decoupled and
    general projectors agree on project, DECIDE_FACE, PHI and BETA."""
    rng = np.random.default_rng(m)
    n = 4
    J = H.Csr.from_dense(np.eye(m, n))
    c = rng.uniform(-1, 1, m)
    x = rng.uniform(-1, 1, n)
    g = rng.uniform(-1, 1, n)
    yd, _ = proj_op(2, 0, J, c, x)
    yg, _ = proj_op(3, 0, J, c, x)
    assert np.array_equal(yd, yg)
    _, fd = proj_op(2, 1, J, c, yd)
    _, fg = proj_op(3, 1, J, c, yg)
    assert np.array_equal(fd, fg)
    pd, _ = proj_op(2, 2, J, c, yd, g)
    pg, _ = proj_op(3, 2, J, c, yg, g)
    assert np.array_equal(pd, pg)
    phi = rng.uniform(-1, 1, n)
    bd, _ = proj_op(2, 3, J, c, yd, g, phi)
    bg, _ = proj_op(3, 3, J, c, yg, g, phi)
    assert np.array_equal(bd, bg)


def test_solver_small_dense():
    """test_case/MPRGPTest.cpp:70-98: a random SPD 5x5 with J = I converges
    (code 0) through both the general and the decoupled solve."""
    rng = np.random.default_rng(5)
    n = 5
    Mm = rng.uniform(-1, 1, (n, n)) + 3.0 * np.eye(n)
    A = H.Csr.from_dense(Mm.T @ Mm)
    J = H.Csr.from_dense(np.eye(n))
    B = rng.uniform(-1, 1, n)
    c = rng.uniform(-1, 1, n)
    x = rng.uniform(-1, 1, n)
    xg, _, sg, _ = H.oracle_solve("general", A, B, x, J, c)
    xd, _, sd, _ = H.oracle_solve("decoupled", A, B, x, J, c)
    assert sg["code"] == 0 and sd["code"] == 0
    assert (xg - c).min() >= -1e-9 and (xd - c).min() >= -1e-9


def test_solver_small_dense_matches_quadprog():
    need_qp()
    rng = np.random.default_rng(6)
    n = 5
    Mm = rng.uniform(-1, 1, (n, n)) + 3.0 * np.eye(n)
    Ad = Mm.T @ Mm
    B = rng.uniform(-1, 1, n)
    c = rng.uniform(-1, 1, n)
    x0 = rng.uniform(-1, 1, n)
    xr, _ = H.solve_qp_ref(Ad, B, np.eye(n), c)
    x, _, s, _ = H.oracle_solve("general", H.Csr.from_dense(Ad), B, x0, H.Csr.from_dense(np.eye(n)),
                                c, tol=1e-13)
    assert s["code"] == 0
    assert np.linalg.norm(x - xr) <= 1e-9 * max(1.0, np.linalg.norm(xr))


def test_general_projector_matches_quadprog():
    """project / PHI / BETA of the block-separable restatement against the
    reference's dense QuadProg++ solves (MPRGPProjection.h:412-467)."""
    need_qp()
    qp = M.beam(2, 2, 5, extra_planes_max=2, extra_planes_min=2, plane_mode=0, seed=8)
    _, _, J, c = H.qp_from_beam(qp)
    Jd = J.dense()
    rng = np.random.default_rng(1)
    for _ in range(3):
        x = qp.x0 + 0.02 * rng.standard_normal(qp.n)
        y, _ = proj_op(3, 0, J, c, x)
        lam, _ = H.solve_qp_ref(Jd @ Jd.T, c - Jd @ x, np.eye(J.rows), np.zeros(J.rows))
        yr = x + Jd.T @ lam
        assert np.abs(y - yr).max() <= 1e-13
        g = rng.standard_normal(qp.n)
        face = np.abs(Jd @ yr - c) < 1e-9
        Ja = Jd[face]
        phi, _ = proj_op(3, 2, J, c, yr, g)
        phir = g + Ja.T @ np.linalg.solve(Ja @ Ja.T, -Ja @ g) if len(Ja) else g
        assert np.abs(phi - phir).max() <= 1e-13
        beta, _ = proj_op(3, 3, J, c, yr, g, phi)
        gp = g - phi
        if len(Ja):
            lb, _ = H.solve_qp_ref(Ja @ Ja.T, Ja @ gp, np.eye(len(Ja)), np.zeros(len(Ja)))
            betar = gp - Ja.T @ lb
        else:
            betar = gp
        assert np.abs(beta - betar).max() <= 1e-13


def _golden(path):
    d = dict(np.load(path))
    nv = int(d["nv"])
    qp = M.BeamQP(nv, d["row_ptr"], d["cols"], d["vals"], d["b"], d["x0"], d["plane_ptr"],
                  d["planes"], {})
    return d, qp


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_golden(path):
    """The oracle's MPRGP solution equals the QuadProg++ solution stored in
    the fixture (same QP, solved by the reference's own dense solver)."""
    d, qp = _golden(path)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-10 * np.linalg.norm(b)
    if "L" in d:
        L, U = d["L"], d["U"]
        x, _, s, _ = H.oracle_solve("box", A, b, np.clip(qp.x0, L, U), L=L, U=U, tol=tol,
                                    max_it=20000)
        act = (np.abs(x - L) < 1e-9) | (np.abs(x - U) < 1e-9)
        act_r = (np.abs(d["x_qp"] - L) < 1e-9) | (np.abs(d["x_qp"] - U) < 1e-9)
    else:
        x, _, s, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=tol, max_it=20000)
        act = H.decide_face_planes(J, c, x)
        act_r = H.decide_face_planes(J, c, d["x_qp"])
    assert s["code"] == 0
    assert np.linalg.norm(x - d["x_qp"]) <= 1e-8 * np.linalg.norm(d["x_qp"])
    assert np.array_equal(act, act_r)


def test_kkt_of_oracle_solution():
    """A x - b = J^T lambda, lambda >= 0 on the active rows, J x >= c."""
    qp = M.beam(3, 2, 6, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=21)
    A, b, J, c = H.qp_from_beam(qp)
    x, _, s, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-11 * np.linalg.norm(b),
                                max_it=20000)
    assert s["code"] == 0
    r = J.matvec(x) - c
    assert r.min() >= -1e-12
    act = np.abs(r) < 1e-9
    Ja = J.dense()[act]
    g = A.matvec(x) - b
    lam, *_ = np.linalg.lstsq(Ja.T, g, rcond=None)
    assert np.linalg.norm(Ja.T @ lam - g) <= 1e-8 * np.linalg.norm(b)
    assert lam.min() >= -1e-8


def test_spectral_radius_power_method():
    """specRad (MPRGPSolver.h:42-79): the power method reaches the largest
    eigenvalue of A (here it converges before the 1001-iteration cap)."""
    qp = M.beam(2, 2, 3, seed=4)
    A, _, _, _ = H.qp_from_beam(qp)
    it = H.C.c_int()
    O = H.oracle()
    lam = O.oracle_spec_rad(A.rows, H.ptr(A.ptr), H.ptr(A.idx), H.ptr(A.val), 1e-14, 7,
                            H.C.byref(it))
    ev = np.linalg.eigvalsh(A.dense())
    assert it.value <= 1001
    assert abs(lam - ev[-1]) <= 1e-10 * ev[-1]


def test_seeded_start_vector_golden():
    """The seeded stand-in for setRandom() (splitmix64 -> [-1, 1)): fixed
    bit patterns, generated identically by the GPU power phase."""
    O = H.oracle()
    want = ["-0x1.cfabedff09d18p-1", "-0x1.b03ead40ea368p-3", "0x1.71ee9896c4dfcp-2",
            "-0x1.dd406d2224c8cp-1"]
    assert [O.oracle_seeded_uniform(0x5EED, i) for i in range(4)] == [float.fromhex(w) for w in want]


def test_reference_stall_is_reproduced():
    """On tilted planes near free vertices the reference's monotone loop keeps
    expanding (the non-proportional branch needs the previous trial point to
    be feasible, MPRGPSolver.h:431-439); the restatement reproduces that."""
    qp = M.beam(4, 4, 16, extra_planes_max=2, extra_planes_min=2, plane_mode=0, seed=2)
    A, b, J, c = H.qp_from_beam(qp)
    _, _, s, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-8 * np.linalg.norm(b),
                                max_it=300)
    assert s["code"] == -1 and s["num_exp"] > 250 and s["num_prop"] == 0


def test_power_method_keeps_ev_unless_it_converges():
    """specRad (MPRGPSolver.h:42-79) writes ev only when it stops early (the
    difference test or a vanishing norm).  A warm start that runs to the
    1001-iteration cap leaves ev as it was, so a second solve from the same ev
    runs the identical power method -- the property the GPU's exact reuse of
    warm-started power methods rests on."""
    qp = M.beam(6, 5, 12, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=13)
    A, b, J, c = H.qp_from_beam(qp)
    ev0 = np.random.default_rng(5).standard_normal(qp.n)
    ev0 /= np.linalg.norm(ev0)
    nb = float(np.linalg.norm(b))
    # a stopping test the power method does not meet in 1001 iterations from
    # this start: ev unchanged, results repeat
    x1, _, s1, ev1 = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-10 * nb,
                                    max_it=20000, ev=ev0)
    assert s1["power_iters"] == 1001 and np.array_equal(ev1, ev0)
    x2, _, s2, ev2 = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-10 * nb,
                                    max_it=20000, ev=ev1)
    assert np.array_equal(ev2, ev0) and np.array_equal(x2, x1)
    assert (s2["spec_rad"], s2["iterations"]) == (s1["spec_rad"], s1["iterations"])
    # a loose one: it stops early and stores a new ev
    _, _, s3, ev3 = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-2 * nb, max_it=20000,
                                   ev=ev0)
    assert s3["power_iters"] < 1001 and not np.array_equal(ev3, ev0)
