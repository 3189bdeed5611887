"""GPU parity: the CUDA solver through the C ABI against the CPU oracle (a
line-by-line restatement of the reference's MPRGP) on the same seeded inputs.

Tolerances (FP64):
  * x: ||x_gpu - x_oracle|| / ||x_oracle|| <= 1e-8 with both sides converged
    to 1e-10 * ||b||.  At the reference's own 1e-8 * ||b|| stopping test both
    iterates are only within ~kappa * tol of the solution, so there the test
    checks convergence, the projected gradient and the active set.
  * active set: DECIDE_FACE of the final x (|J x - c| < 1e-9,
    MPRGPProjection.h:283-297) identical.
  * spectral radius: 1e-10 relative (same seeded start vector, 1001 power
    iterations, FP64).
  * step trace: the same sequence of CG / expansion / proportioning steps with
    residuals equal to 1e-6 relative, up to the point where the oracle's
    f(P(y)) <= f(x) test compares values within rounding of each other.
"""
import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

SEED = 0x5EED
EV = {1: "cg", 2: "cgx", 3: "exp", 4: "prop", 5: "top"}


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def gpu_solve(ctx, qp, kind, tol, max_it=20000, precision=M.PREC_FP64, **kw):
    opt = M.default_options(tol=tol, max_it=max_it, kind=kind, project_x0=1, seed=SEED,
                            precision=precision, **kw)
    return ctx.solve_bsr(qp, opt, qp.x0)


def corner(a, b, c, seed=1):
    """Beam in a corner: floor + walls x, z (up to 3 planes per vertex)."""
    return M.beam(a, b, c, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=seed)


def test_spmv_matches_oracle(ctx):
    torch = pytest.importorskip("torch")
    qp = corner(5, 4, 9, seed=3)
    A, b, J, c = H.qp_from_beam(qp)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(qp.n)
    y_ref = A.matvec(x)
    pr = M.Problem(ctx, qp.nv)
    pr.set_matrix(qp.row_ptr, qp.cols, qp.vals, precisions=3)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(qp.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_FP64)
    ctx.sync()
    assert rel(yd.cpu().numpy(), y_ref) < 1e-14
    pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_MIXED)
    ctx.sync()
    assert rel(yd.cpu().numpy(), y_ref) < 1e-5  # FP32 values, FP32 accumulation
    pr.close()


@pytest.mark.parametrize("kind_name,kind", [("decoupled", M.KIND_DECOUPLED),
                                            ("general", M.KIND_PLANES)])
@pytest.mark.parametrize("extra", [0, 2])
def test_solve_parity(ctx, kind_name, kind, extra):
    qp = M.beam(4, 4, 16, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2, seed=1)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-10 * np.linalg.norm(b)
    xo, fo, so, _ = H.oracle_solve(kind_name, A, b, qp.x0, J, c, tol=tol, max_it=20000, seed=SEED)
    xg, fg, sg = gpu_solve(ctx, qp, kind, tol)
    assert so["code"] == 0 and sg.code == 0, (so, sg.as_dict())
    assert rel(xg, xo) <= 1e-8
    assert np.array_equal(H.decide_face_planes(J, c, xg), H.decide_face_planes(J, c, xo))
    assert sg.power_iters == so["power_iters"]
    assert abs(sg.spec_rad - so["spec_rad"]) <= 1e-10 * so["spec_rad"]
    assert (J.matvec(xg) - c).min() >= -1e-9
    # The reference's own stopping test, 1e-8 ||b||: both converge, the GPU's
    # projected gradient is below it, and the active sets agree.
    tol8 = 1e-8 * np.linalg.norm(b)
    xo8, _, so8, _ = H.oracle_solve(kind_name, A, b, qp.x0, J, c, tol=tol8, max_it=20000,
                                    seed=SEED)
    xg8, _, sg8 = gpu_solve(ctx, qp, kind, tol8)
    assert so8["code"] == 0 and sg8.code == 0 and sg8.residual <= tol8
    assert H.projected_gradient_norm(kind_name, A, b, xg8, J, c) <= 1.01 * tol8
    assert np.array_equal(H.decide_face_planes(J, c, xg8), H.decide_face_planes(J, c, xo8))
    assert rel(xg8, xo) <= 1e-6 and rel(xo8, xo) <= 1e-6


def _traces(ctx, qp, kind_name, kind, tol, max_it):
    A, b, J, c = H.qp_from_beam(qp)
    H.oracle_trace(True)
    xo, _, so, _ = H.oracle_solve(kind_name, A, b, qp.x0, J, c, tol=tol, max_it=max_it, seed=SEED)
    to = H.oracle_get_trace()
    H.oracle_trace(False)
    pr = M.load_beam(ctx, qp)
    pr.set_trace(200000)
    st = pr.solve(M.default_options(tol=tol, max_it=max_it, kind=kind, project_x0=1, seed=SEED))
    tg = pr.get_trace()
    xg = pr.get_x()
    pr.close()
    return xo, so, to, xg, st, tg


def test_trace_parity_converging(ctx):
    """Same steps as the reference until its f-comparison reaches rounding."""
    qp = corner(4, 4, 16, seed=2)
    tol = 1e-8 * np.linalg.norm(qp.b)
    xo, so, to, xg, sg, tg = _traces(ctx, qp, "general", M.KIND_PLANES, tol, 3000)
    n = 0
    for i in range(min(len(to), len(tg))):
        if to[i, 0] != tg[i, 0] or to[i, 1] != tg[i, 1]:
            break
        assert abs(to[i, 2] - tg[i, 2]) <= 1e-6 * abs(to[i, 2]), (i, to[i], tg[i])
        n += 1
    assert n >= 40, (n, to[n - 2:n + 2], tg[n - 2:n + 2])
    assert so["code"] == 0 and sg.code == 0


def test_stall_trace_parity(ctx):
    """Inputs on which the reference's monotone loop stalls (tilted planes
    near free vertices: the loop expands whenever the previous trial point is
    infeasible and never proportions): the GPU stalls in exactly the same way."""
    qp = M.beam(4, 4, 16, extra_planes_max=2, extra_planes_min=2, plane_mode=0, seed=2)
    tol = 1e-8 * np.linalg.norm(qp.b)
    xo, so, to, xg, sg, tg = _traces(ctx, qp, "general", M.KIND_PLANES, tol, 300)
    assert so["code"] == -1 and sg.code == -1
    assert sg.num_exp == so["num_exp"] and sg.num_cg == so["num_cg"]
    assert len(to) == len(tg)
    assert np.array_equal(to[:, :2], tg[:, :2])
    assert np.allclose(to[:, 2], tg[:, 2], rtol=1e-6)
    assert rel(xg, xo) <= 1e-8


@pytest.mark.parametrize("extra,seed", [(1, 6), (2, 8)])
def test_tilted_planes_parity(ctx, extra, seed):
    """Tilted global planes (up to 3 non-orthogonal planes per vertex) on
    inputs where the reference converges."""
    qp = M.beam(4, 4, 16, extra_planes_max=extra, extra_planes_min=extra, plane_mode=0, seed=seed)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-10 * np.linalg.norm(b)
    xo, _, so, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=tol, max_it=20000, seed=SEED)
    xg, _, sg = gpu_solve(ctx, qp, M.KIND_PLANES, tol)
    assert so["code"] == 0 and sg.code == 0
    assert rel(xg, xo) <= 1e-8
    assert np.array_equal(H.decide_face_planes(J, c, xg), H.decide_face_planes(J, c, xo))


def test_mixed_precision(ctx):
    qp = corner(4, 4, 16, seed=2)
    A, b, J, c = H.qp_from_beam(qp)
    xo, _, so, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=1e-10 * np.linalg.norm(b),
                                  max_it=20000, seed=SEED)
    tol8 = 1e-8 * np.linalg.norm(b)
    xm, _, sm = gpu_solve(ctx, qp, M.KIND_PLANES, tol8, precision=M.PREC_MIXED)
    assert sm.code == 0
    assert sm.spmv_fp32 > 0
    # the FP64 residual replacement certifies the true projected gradient
    assert H.projected_gradient_norm("general", A, b, xm, J, c) <= 1.01 * tol8
    assert rel(xm, xo) <= 1e-6
    assert np.array_equal(H.decide_face_planes(J, c, xm), H.decide_face_planes(J, c, xo))


def _bounds_problem(seed=4):
    qp = M.beam(3, 3, 8, seed=seed)
    n = qp.n
    L = np.full(n, -1e30)
    L[1::3] = 0.0            # y >= 0 as a lower bound
    U = np.full(n, 1e30)
    U[0::3] = qp.x0[0::3] + 0.0005  # x may not move right by more than 0.5 mm
    return qp, L, U


@pytest.mark.parametrize("kind_name,kind", [("lower", M.KIND_LOWER), ("box", M.KIND_BOX)])
def test_bounds_parity(ctx, kind_name, kind):
    qp, L, U = _bounds_problem()
    A, b, _, _ = H.qp_from_beam(qp)
    x0 = np.clip(qp.x0, L, U)
    tol = 1e-10 * np.linalg.norm(b)
    Uo = U if kind_name == "box" else None
    xo, fo, so, _ = H.oracle_solve(kind_name, A, b, x0, L=L, U=Uo, tol=tol, max_it=20000,
                                   seed=SEED)
    opt = M.default_options(tol=tol, max_it=20000, kind=kind, seed=SEED)
    xg, fg, sg = ctx.solve_bsr(qp, opt, x0, L=L, U=Uo)
    assert so["code"] == 0 and sg.code == 0, (so, sg.as_dict())
    assert rel(xg, xo) <= 1e-8
    assert np.array_equal(fg, fo)


def test_batch_equals_single(ctx):
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(4, 4, 6, 0, 5), (3, 5, 7, 2, 6), (6, 4, 9, 1, 7)]]
    probs, opts, singles = [], [], []
    for qp in qps:
        tol = 1e-10 * np.linalg.norm(qp.b)
        kind = M.KIND_PLANES if qp.params["extra_planes_max"] else M.KIND_DECOUPLED
        opt = M.default_options(tol=tol, max_it=20000, kind=kind, project_x0=1, seed=SEED)
        xs, _, ss = ctx.solve_bsr(qp, opt, qp.x0)
        singles.append((xs, ss))
        pr = M.load_beam(ctx, qp)
        probs.append(pr)
        opts.append(opt)
    stats = ctx.solve_batch(probs, opts)
    for pr, st, (xs, ss) in zip(probs, stats, singles):
        assert st.code == 0
        xb = pr.get_x()
        assert np.array_equal(xb, xs)          # deterministic reductions
        assert st.iterations == ss.iterations
        pr.close()


def _solve_all(c, qps, precision):
    out = []
    for qp in qps:
        tol = 1e-10 * np.linalg.norm(qp.b)
        opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                precision=precision)
        out.append(c.solve_bsr(qp, opt, qp.x0))
    return out


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_cluster_solver_equals_engine(precision):
    """Small instances run on the thread-block-cluster solver; its results are
    bitwise those of the persistent engine (the per-item and per-instance
    reductions run in the same order), for every cluster size (instances of
    1, 2, 3, 7 and 10 items of 256 vertices, the last item partial) and with
    the largest cluster size capped so some of them go to the engine."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(2, 2, 3, 1, 3), (5, 5, 10, 2, 4), (6, 6, 14, 0, 7),
                                   (8, 8, 20, 1, 11), (9, 9, 24, 1, 5)]]
    c = M.Context(0)
    try:
        c.set_cluster(0)
        ref = _solve_all(c, qps, precision)
        tried = 0
        for cluster in (2, 4, 8, 16):
            try:
                c.set_cluster(cluster)
            except M.MPRGPError:
                continue  # cluster size not available on this device
            tried += 1
            got = _solve_all(c, qps, precision)
            for (xe, fe, se), (xc, fc, sc) in zip(ref, got):
                assert se.code == 0 and sc.code == 0
                assert np.array_equal(xe, xc)
                assert np.array_equal(fe, fc)
                assert (se.iterations, se.phases, se.power_iters) == (sc.iterations, sc.phases,
                                                                     sc.power_iters)
                assert se.spec_rad == sc.spec_rad and se.residual == sc.residual
        assert tried >= 2
    finally:
        c.close()


def test_batch_mixes_cluster_and_engine(ctx):
    """One batch with instances on both paths equals the single solves."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(4, 4, 6, 1, 8), (16, 16, 40, 2, 9), (9, 9, 24, 0, 10)]]
    singles = _solve_all(ctx, qps, M.PREC_MIXED)
    probs, opts = [], []
    for qp in qps:
        probs.append(M.load_beam(ctx, qp, precisions=3))
        opts.append(M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000,
                                      kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                      precision=M.PREC_MIXED))
    stats = ctx.solve_batch(probs, opts)
    for pr, st, (xs, fs, ss) in zip(probs, stats, singles):
        assert st.code == 0
        assert np.array_equal(pr.get_x(), xs)
        assert st.iterations == ss.iterations
        pr.close()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_power_cache_is_exact(ctx, precision):
    """A re-solve of a resident problem with the same A, seed and form reuses
    the power method's result: the solution and every reported quantity are
    bitwise those of a solve that runs the power method again."""
    qp = M.beam(6, 5, 12, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=12)
    opt = M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                            project_x0=1, seed=SEED, precision=precision)
    pr = M.load_beam(ctx, qp, precisions=3)
    runs = []
    for cache in (True, True, False):
        pr.set_power_cache(cache)
        pr.set_x(qp.x0)
        st = pr.solve(opt)
        assert st.code == 0
        runs.append((pr.get_x(), pr.get_face(), st))
    (x0, f0, s0), (x1, f1, s1), (x2, f2, s2) = runs
    for x, f, st in ((x1, f1, s1), (x2, f2, s2)):
        assert np.array_equal(x, x0) and np.array_equal(f, f0)
        assert (st.iterations, st.power_iters, st.spec_rad, st.alpha_bar, st.residual) == \
            (s0.iterations, s0.power_iters, s0.spec_rad, s0.alpha_bar, s0.residual)
    # the cached run skipped the power method's matrix passes, the uncached did not
    assert s1.spmv_fp64 + s1.spmv_fp32 < s0.spmv_fp64 + s0.spmv_fp32
    assert s2.spmv_fp64 + s2.spmv_fp32 == s0.spmv_fp64 + s0.spmv_fp32
    # a new A invalidates it
    pr.set_power_cache(True)
    pr.set_matrix(qp.row_ptr, qp.cols, qp.vals, 3)
    pr.set_x(qp.x0)
    s3 = pr.solve(opt)
    assert s3.spmv_fp64 + s3.spmv_fp32 == s0.spmv_fp64 + s0.spmv_fp32
    assert np.array_equal(pr.get_x(), x0)
    pr.close()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_warm_start_power_cache_is_exact(ctx, precision):
    """A solve whose power method starts from the stored vector ev and runs to
    its iteration limit leaves ev unchanged; the next solve of the same
    problem from the same ev reuses its result and is bitwise the solve that
    runs it again.  A new ev or a new A invalidates the reuse."""
    qp = M.beam(6, 5, 12, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=13)
    # a tol the power method does not reach in 1001 iterations from a fixed,
    # non-eigen start vector: it stores no new ev
    opt = M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                            project_x0=1, seed=SEED, precision=precision, use_ev=1)
    ev = np.random.default_rng(5).standard_normal(qp.n)
    ev /= np.linalg.norm(ev)
    pr = M.load_beam(ctx, qp, precisions=3)
    pr.set_ev(ev)
    runs = []
    for cache in (True, True, False):
        pr.set_power_cache(cache)
        pr.set_x(qp.x0)
        st = pr.solve(opt)
        runs.append((pr.get_x(), pr.get_face(), st))
    (x0, f0, s0), (x1, f1, s1), (x2, f2, s2) = runs
    assert s0.power_iters == 1001  # ran to the limit: ev kept
    for x, f, st in ((x1, f1, s1), (x2, f2, s2)):
        assert np.array_equal(x, x0) and np.array_equal(f, f0)
        assert (st.code, st.iterations, st.power_iters, st.spec_rad, st.alpha_bar, st.residual) == \
            (s0.code, s0.iterations, s0.power_iters, s0.spec_rad, s0.alpha_bar, s0.residual)
    assert s1.spmv_fp64 + s1.spmv_fp32 < s0.spmv_fp64 + s0.spmv_fp32  # reused
    assert s2.spmv_fp64 + s2.spmv_fp32 == s0.spmv_fp64 + s0.spmv_fp32  # cache off: recomputed
    # with the cache off a solve still records its result: back on, the next
    # solve reuses it
    pr.set_power_cache(True)
    pr.set_x(qp.x0)
    sb = pr.solve(opt)
    assert sb.spmv_fp64 + sb.spmv_fp32 < s0.spmv_fp64 + s0.spmv_fp32
    assert np.array_equal(pr.get_x(), x0) and sb.spec_rad == s0.spec_rad
    # a new ev (here the same values, uploaded again) and a new A invalidate it
    pr.set_ev(ev)
    pr.set_x(qp.x0)
    s3 = pr.solve(opt)
    assert s3.spmv_fp64 + s3.spmv_fp32 == s0.spmv_fp64 + s0.spmv_fp32
    pr.set_matrix(qp.row_ptr, qp.cols, qp.vals, 3)
    pr.set_x(qp.x0)
    s4 = pr.solve(opt)
    assert s4.spmv_fp64 + s4.spmv_fp32 == s0.spmv_fp64 + s0.spmv_fp32
    assert np.array_equal(pr.get_x(), x0)
    pr.close()


GOLDEN = sorted(__import__("glob").glob(__import__("os").path.join(
    __import__("os").path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[p.rsplit("/", 1)[-1][:-4] for p in GOLDEN])
def test_gpu_matches_golden(ctx, path):
    """GPU solutions against the QuadProg++ solutions stored in the fixtures
    (the reference's own dense QP solver, run where the reference is present)."""
    d = dict(np.load(path))
    qp = M.BeamQP(int(d["nv"]), d["row_ptr"], d["cols"], d["vals"], d["b"], d["x0"],
                  d["plane_ptr"], d["planes"], {})
    tol = 1e-10 * np.linalg.norm(qp.b)
    xr = d["x_qp"]
    if "L" in d:
        L, U = d["L"], d["U"]
        opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_BOX, seed=SEED)
        x, face, st = ctx.solve_bsr(qp, opt, np.clip(qp.x0, L, U), L=L, U=U)
        act = (np.abs(x - L) < 1e-9) | (np.abs(x - U) < 1e-9)
        act_r = (np.abs(xr - L) < 1e-9) | (np.abs(xr - U) < 1e-9)
    else:
        A, b, J, c = H.qp_from_beam(qp)
        x, face, st = gpu_solve(ctx, qp, M.KIND_PLANES, tol)
        act = H.decide_face_planes(J, c, x)
        act_r = H.decide_face_planes(J, c, xr)
    assert st.code == 0
    assert rel(x, xr) <= 1e-8
    assert np.array_equal(act, act_r)


def test_autotune_pick_is_result_invariant(tmp_path, monkeypatch):
    """The autotuner's launch shapes never change a solution: it verifies its
    pick against the default bitwise, and the pick round-trips its cache."""
    from mprgp_gb300 import autotune
    monkeypatch.setenv("MPRGP_TUNING_CACHE", str(tmp_path / "tuning.json"))
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(4, 4, 6, 1, 21), (9, 9, 24, 2, 22), (16, 16, 40, 1, 23)]]
    c = M.Context(0)
    try:
        r = autotune.tune(c, qps, precision=M.PREC_MIXED, reps=1)
        assert not r["cached"] and r["ms"] <= r["default_ms"] * 1.0001
        assert set(r["config"]) == set(autotune.DEFAULT)
        r2 = autotune.tune(c, qps, precision=M.PREC_MIXED, reps=1)
        assert r2["cached"] and r2["config"] == r["config"]
    finally:
        c.close()


def test_relayout_when_planes_change(ctx):
    """The SELL row order groups vertices with several planes; changing the
    planes after the matrix rebuilds it, and the solve equals that of a
    problem loaded with the final planes from the start."""
    corner = M.beam(7, 6, 12, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=31)
    floor = M.beam(7, 6, 12, extra_planes_max=0, extra_planes_min=0, plane_mode=2, seed=31)
    assert np.array_equal(corner.vals, floor.vals)
    opt = M.default_options(tol=1e-10 * np.linalg.norm(corner.b), max_it=20000,
                            kind=M.KIND_PLANES, project_x0=1, seed=SEED, precision=M.PREC_MIXED)
    pr = M.load_beam(ctx, floor, precisions=3)        # identity layout (one plane each)
    pr.set_planes(corner.plane_ptr, corner.planes)    # walls: multi-plane rows regrouped
    pr.set_rhs(corner.b)
    pr.set_x(corner.x0)
    st = pr.solve(opt)
    x_re = pr.get_x()
    pr.close()
    fresh = M.load_beam(ctx, corner, precisions=3)
    st2 = fresh.solve(opt)
    assert st.code == 0 and st2.code == 0
    assert np.array_equal(x_re, fresh.get_x())
    # and the standalone product follows the layout
    import torch
    xd = torch.from_numpy(np.random.default_rng(5).standard_normal(corner.n)).cuda()
    yd = torch.zeros(corner.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    fresh.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_FP64)
    ctx.sync()
    A, _, _, _ = H.qp_from_beam(corner)
    assert rel(yd.cpu().numpy(), A.matvec(xd.cpu().numpy())) < 1e-14
    fresh.close()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_multi_item_clusters_equal_engine(precision):
    """With several items per CTA, instances beyond the largest cluster also
    run on the cluster solver (a 47-item and a 34-item beam on 16 CTAs), and
    still give bitwise the engine's results."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(16, 16, 40, 2, 61), (20, 12, 30, 1, 62), (8, 8, 20, 1, 63)]]
    c = M.Context(0)
    try:
        c.set_cluster(0)
        ref = _solve_all(c, qps, precision)
        c.set_cluster(16)
        for items in (2, 4):
            c.set_cluster_items(items)
            got = _solve_all(c, qps, precision)
            for (xe, fe, se), (xc, fc, sc) in zip(ref, got):
                assert se.code == 0 and sc.code == 0
                assert np.array_equal(xe, xc) and np.array_equal(fe, fc)
                assert (se.iterations, se.phases) == (sc.iterations, sc.phases)
    finally:
        c.close()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_engine_graph_loop_equals_persistent_engine(precision):
    """The large instances' phases as a CUDA-graph loop of one launch per
    phase give bitwise the persistent engine's results (one instance alone
    and two in one batch)."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(16, 16, 40, 2, 71), (24, 20, 30, 1, 72)]]
    c = M.Context(0)
    try:
        res = {}
        for bits in (0, 16):
            c.set_tuning(bits, 0)
            single = _solve_all(c, qps, precision)
            probs, opts = [], []
            for qp in qps:
                probs.append(M.load_beam(c, qp, precisions=3))
                opts.append(M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000,
                                              kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                              precision=precision))
            stats = c.solve_batch(probs, opts)
            batch = [(pr.get_x(), st) for pr, st in zip(probs, stats)]
            for pr in probs:
                pr.close()
            res[bits] = (single, batch)
        for (xa, fa, sa), (xb, fb, sb) in zip(res[0][0], res[16][0]):
            assert sa.code == 0 and sb.code == 0
            assert np.array_equal(xa, xb) and np.array_equal(fa, fb)
            assert (sa.iterations, sa.phases) == (sb.iterations, sb.phases)
        for (xa, sa), (xb, sb) in zip(res[0][1], res[16][1]):
            assert sa.code == 0 and sb.code == 0 and np.array_equal(xa, xb)
    finally:
        c.close()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_persistent_power_loop_equals_launch_loop(precision):
    """The power method as one persistent cooperative launch (grid barrier per
    phase, every CTA advancing its own copy of the state) gives bitwise the
    launch loop's results: one instance alone, and a batch whose items exceed
    one per CTA (several items a CTA)."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(16, 16, 40, 2, 81), (24, 20, 30, 1, 82), (20, 12, 60, 2, 83)]]
    c = M.Context(0)
    try:
        c.set_cluster(0)  # every instance on the engine path, so the batch has many items
        res = {}
        for bits in (0, 32):
            c.set_tuning(bits, 0)
            single = _solve_all(c, qps[:1], precision)
            probs, opts = [], []
            for qp in qps * 6:  # 18 instances, about 1,900 items
                probs.append(M.load_beam(c, qp, precisions=3))
                probs[-1].set_power_cache(False)
                opts.append(M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000,
                                              kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                              precision=precision))
            stats = c.solve_batch(probs, opts)
            batch = [(pr.get_x(), st) for pr, st in zip(probs, stats)]
            for pr in probs:
                pr.close()
            res[bits] = (single, batch)
        for (xa, fa, sa), (xb, fb, sb) in zip(res[0][0], res[32][0]):
            assert sa.code == 0 and sb.code == 0
            assert np.array_equal(xa, xb) and np.array_equal(fa, fb)
            assert (sa.iterations, sa.phases, sa.power_iters) == (sb.iterations, sb.phases,
                                                                   sb.power_iters)
            assert sa.spec_rad == sb.spec_rad
        for (xa, sa), (xb, sb) in zip(res[0][1], res[32][1]):
            assert sa.code == 0 and sb.code == 0 and np.array_equal(xa, xb)
            assert sa.spec_rad == sb.spec_rad and sa.power_iters == sb.power_iters
    finally:
        c.close()


@pytest.mark.parametrize("precision", [M.PREC_MIXED, M.PREC_FP64])
def test_power_step_loop_equals_launch_loop(precision):
    """The power-step loop (each launch advances the states the previous one
    left, the reduction warp overlapping the rows' products; a settle kernel
    per body) gives bitwise the launch loop's results, as a graph loop and as
    stream launches: one instance alone and a batch with several items per
    CTA."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(16, 16, 40, 2, 91), (24, 20, 30, 1, 92), (20, 12, 60, 2, 93)]]
    c = M.Context(0)
    try:
        c.set_cluster(0)  # every instance on the engine path
        res = {}
        for bits in (64, 0, 4):  # launch loop (the reference), power-step graph and stream
            c.set_tuning(bits, 0)
            single = _solve_all(c, qps[:1], precision)
            probs, opts = [], []
            for qp in qps * 6:  # 18 instances, about 1,900 items
                probs.append(M.load_beam(c, qp, precisions=3))
                probs[-1].set_power_cache(False)
                opts.append(M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000,
                                              kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                              precision=precision))
            stats = c.solve_batch(probs, opts)
            batch = [(pr.get_x(), st) for pr, st in zip(probs, stats)]
            for pr in probs:
                pr.close()
            res[bits] = (single, batch)
        for other in (0, 4):
            for (xa, fa, sa), (xb, fb, sb) in zip(res[64][0], res[other][0]):
                assert sa.code == 0 and sb.code == 0
                assert np.array_equal(xa, xb) and np.array_equal(fa, fb)
                assert (sa.iterations, sa.phases, sa.power_iters) == (sb.iterations, sb.phases,
                                                                       sb.power_iters)
                assert sa.spec_rad == sb.spec_rad
            for (xa, sa), (xb, sb) in zip(res[64][1], res[other][1]):
                assert sa.code == 0 and sb.code == 0 and np.array_equal(xa, xb)
                assert sa.spec_rad == sb.spec_rad and sa.power_iters == sb.power_iters
                assert sa.phases == sb.phases
    finally:
        c.close()


@pytest.mark.parametrize("precision", [M.PREC_MIXED, M.PREC_FP64])
def test_power_step_loop_mixed_starts(precision):
    """A batch whose instances start in different places -- half of them with
    the power method cached (they skip it), half running it -- gives in the
    power-step loop what each instance gives alone in the launch loop: the
    step kernels carry the states of instances outside the power method
    through unchanged."""
    qps = [M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=s)
           for (a, b, c, e, s) in [(16, 16, 40, 2, 71), (24, 20, 30, 1, 72), (20, 12, 60, 2, 73),
                                   (18, 14, 36, 1, 74)]]
    c = M.Context(0)
    try:
        c.set_cluster(0)
        c.set_tuning(64, 0)  # the launch loop, one instance at a time
        ref = _solve_all(c, qps, precision)
        c.set_tuning(0, 0)   # the power-step loop
        probs, opts = [], []
        for i, qp in enumerate(qps):
            pr = M.load_beam(c, qp, precisions=3)
            opt = M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000,
                                    kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                                    precision=precision)
            if i % 2 == 0:  # a first solve stores the power method's result
                pr.set_x(qp.x0)
                assert pr.solve(opt).code == 0
            pr.set_x(qp.x0)
            probs.append(pr)
            opts.append(opt)
        stats = c.solve_batch(probs, opts)
        for i, (pr, st, (xr, fr, sr)) in enumerate(zip(probs, stats, ref)):
            assert st.code == 0 and sr.code == 0
            assert np.array_equal(pr.get_x(), xr) and np.array_equal(pr.get_face(), fr)
            assert (st.iterations, st.power_iters, st.spec_rad) == \
                (sr.iterations, sr.power_iters, sr.spec_rad)
            assert (st.power_passes == 0) == (i % 2 == 0)  # cached ones skipped it
        for pr in probs:
            pr.close()
    finally:
        c.close()


def test_invalid_column_reports_invalid(ctx):
    """A block column outside 0..nv-1 is caught on the device as A is
    converted (the conversion keeps every index in range): the solve and the
    standalone SpMV return MPRGP_INVALID, and a valid matrix loaded next into
    the same context solves normally."""
    torch = pytest.importorskip("torch")
    qp = corner(4, 4, 8, seed=5)
    cols = qp.cols.copy()
    cols[len(cols) // 2] = qp.nv + 7
    bad = M.BeamQP(qp.nv, qp.row_ptr, cols, qp.vals, qp.b, qp.x0, qp.plane_ptr, qp.planes, {})
    opt = M.default_options(tol=1e-8 * np.linalg.norm(qp.b), max_it=200, kind=M.KIND_PLANES,
                            project_x0=1, seed=SEED)
    with pytest.raises(M.MPRGPError) as e:
        ctx.solve_bsr(bad, opt, qp.x0)
    assert e.value.code == M.INVALID
    pr = M.Problem(ctx, qp.nv)
    pr.set_matrix(bad.row_ptr, bad.cols, bad.vals, precisions=1)
    xd = torch.zeros(qp.n, dtype=torch.float64, device="cuda")
    yd = torch.zeros(qp.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(M.MPRGPError) as e:
        pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_FP64)
    assert e.value.code == M.INVALID
    pr.set_matrix(qp.row_ptr, qp.cols, qp.vals, precisions=1)  # a valid A clears it
    pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_FP64)
    pr.close()
    x, face, st = ctx.solve_bsr(qp, opt, qp.x0)
    assert st.code == 0


@pytest.mark.parametrize("far", [False, True])
def test_spmv_column_forms(ctx, far):
    """The matrix passes read 16-bit column offsets from the row's vertex
    when every offset fits, else the 32-bit columns.  A block-tridiagonal
    matrix of 40,000 vertices has offsets of at most 1; a symmetric pair of
    blocks coupling the first and the last vertex (offset 39,999) sends every
    pass to the 32-bit columns.  Both products match numpy's."""
    torch = pytest.importorskip("torch")
    nv = 40000
    rng = np.random.default_rng(7)
    rows, cols = [], []
    for v in range(nv):
        for u in (v - 1, v, v + 1):
            if 0 <= u < nv:
                rows.append(v)
                cols.append(u)
    if far:
        rows += [0, nv - 1]
        cols += [nv - 1, 0]
    order = np.lexsort((np.array(cols), np.array(rows)))
    rows = np.array(rows)[order]
    cols = np.array(cols, dtype=np.int32)[order]
    nnzb = len(rows)
    row_ptr = np.zeros(nv + 1, dtype=np.int32)
    np.add.at(row_ptr, rows + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    vals = rng.standard_normal((nnzb, 3, 3))
    vals[rows == cols] += 8.0 * np.eye(3)  # a dominant diagonal block
    x = rng.standard_normal(3 * nv)
    y_ref = np.zeros((nv, 3))  # y = A x block by block
    np.add.at(y_ref, rows, np.einsum("kij,kj->ki", vals, x.reshape(nv, 3)[cols]))
    y_ref = y_ref.reshape(-1)
    pr = M.Problem(ctx, nv)
    pr.set_matrix(row_ptr, cols, np.ascontiguousarray(vals.reshape(-1)), precisions=3)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(3 * nv, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_FP64)
    ctx.sync()
    assert rel(yd.cpu().numpy(), y_ref) < 1e-14
    pr.spmv(xd.data_ptr(), yd.data_ptr(), M.PREC_MIXED)
    ctx.sync()
    assert rel(yd.cpu().numpy(), y_ref) < 1e-5
    pr.close()
