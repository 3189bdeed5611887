"""GPU parity at the measured sizes, and the step sequence explained.

1. The GPU solver evaluates CGMonotonicStep's test f(P(y)) <= f(x)
   (MPRGPSolver.h:289, 305-309) from scalars; the reference compares two
   separately rounded function values, which near convergence differ by less
   than their rounding, so its comparison flips and it expands instead of
   continuing CG.  With the oracle switched to the scalar form the GPU takes
   exactly the oracle's steps: the whole trace (every CG step, expansion and
   proportioning, in order) and the step counts are equal.  That one line is
   the whole difference between the GPU's and the reference's iteration
   counts.
2. The 32x32x128 corner beam (421,443 DOF, floor + walls x, z, up to 3 planes
   per vertex) in plain FP64 against the oracle (reference form, all host
   cores): the same DECIDE_FACE active set at the reference's stopping test
   1e-8 ||b|| and at 1e-10 ||b||, and ||x - x_ref|| / ||x_ref|| <= 1e-8 at
   1e-10 ||b|| (at 1e-8 ||b|| both iterates are only within ~kappa * tol of
   the solution).  The mixed form on the same QP: the same active set at both
   tolerances and within 1e-8 of the oracle at 1e-10 ||b||.
"""
import os

import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_traced(kind_name, A, b, x0, J, c, tol, max_it, scalar):
    H.oracle_scalar_test(scalar)
    H.oracle_trace(True)
    try:
        x, face, st, _ = H.oracle_solve(kind_name, A, b, x0, J, c, tol=tol, max_it=max_it,
                                        seed=SEED)
        tr = H.oracle_get_trace()
    finally:
        H.oracle_trace(False)
        H.oracle_scalar_test(False)
    return x, face, st, tr


def gpu_traced(ctx, qp, kind, tol, max_it):
    pr = M.load_beam(ctx, qp)
    pr.set_trace(200000)
    st = pr.solve(M.default_options(tol=tol, max_it=max_it, kind=kind, project_x0=1, seed=SEED))
    tr = pr.get_trace()
    x = pr.get_x()
    pr.close()
    return x, st, tr


CASES = {
    # name: (beam kwargs, oracle kind, GPU kind)
    "floor-decoupled": (dict(a=4, b=4, c=16, seed=1), "decoupled", M.KIND_DECOUPLED),
    "corner-general": (dict(a=4, b=4, c=16, extra_planes_max=2, extra_planes_min=2,
                            plane_mode=2, seed=2), "general", M.KIND_PLANES),
    "corner-8x8x32": (dict(a=8, b=8, c=32, extra_planes_max=2, extra_planes_min=2,
                           plane_mode=2, v0_sigma=0.2, seed=3), "general", M.KIND_PLANES),
}


@pytest.mark.parametrize("rel_tol", [1e-8, 1e-10])
@pytest.mark.parametrize("case", sorted(CASES))
def test_steps_equal_scalar_test_oracle(ctx, case, rel_tol):
    kw, kind_name, kind = CASES[case]
    kw = dict(kw)
    qp = M.beam(kw.pop("a"), kw.pop("b"), kw.pop("c"), **kw)
    A, b, J, c = H.qp_from_beam(qp)
    tol = rel_tol * np.linalg.norm(b)
    xs, fs, ss, ts = oracle_traced(kind_name, A, b, qp.x0, J, c, tol, 20000, scalar=True)
    xr, fr, sr, tr = oracle_traced(kind_name, A, b, qp.x0, J, c, tol, 20000, scalar=False)
    xg, sg, tg = gpu_traced(ctx, qp, kind, tol, 20000)
    print(f"{case} tol {rel_tol:g}||b||: GPU {sg.iterations} iterations "
          f"(cg {sg.num_cg}, exp {sg.num_exp}, prop {sg.num_prop}); oracle, scalar test "
          f"{int(ss['iterations'])} ({int(ss['num_cg'])}/{int(ss['num_exp'])}/"
          f"{int(ss['num_prop'])}); oracle, reference test {int(sr['iterations'])} "
          f"({int(sr['num_cg'])}/{int(sr['num_exp'])}/{int(sr['num_prop'])})")
    assert sg.code == 0 and ss["code"] == 0 and sr["code"] == 0
    # The oracle records the CG loop's exit (event 2) also when the loop ends
    # because the residual met the tolerance; the GPU goes straight to the
    # final projection there.  That last entry is the only difference allowed.
    if len(ts) == len(tg) + 1:
        assert ts[-1, 0] == 2 and ts[-1, 2] <= tol and tg[-1, 0] == 1, (ts[-3:], tg[-3:])
        ts = ts[:-1]
    # the whole step sequence: event kind and iteration number of every entry
    assert len(tg) == len(ts), (len(tg), len(ts))
    assert np.array_equal(tg[:, :2], ts[:, :2])
    # residuals agree to rounding (different summation orders) while they are
    # large; CG amplifies the rounding differences as it converges, so below
    # 1e-5 of the first residual they agree to 25 %
    big = ts[:, 2] > 1e-5 * ts[0, 2]
    assert np.allclose(tg[big, 2], ts[big, 2], rtol=1e-6, atol=0.0)
    assert np.allclose(tg[~big, 2], ts[~big, 2], rtol=0.25, atol=0.0)
    assert (sg.iterations, sg.num_cg, sg.num_exp, sg.num_prop) == (
        int(ss["iterations"]), int(ss["num_cg"]), int(ss["num_exp"]), int(ss["num_prop"]))
    # and all three land on the same active set
    face = H.decide_face_planes(J, c, xg)
    assert np.array_equal(face, H.decide_face_planes(J, c, xs))
    assert np.array_equal(face, H.decide_face_planes(J, c, xr))
    if rel_tol <= 1e-10:
        assert rel(xg, xr) <= 1e-8 and rel(xg, xs) <= 1e-8


@pytest.fixture(scope="module")
def c1_qp():
    return M.beam(32, 32, 128, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=1)


def test_c1_fp64_matches_oracle(ctx, c1_qp):
    qp = c1_qp
    A, b, J, c = H.qp_from_beam(qp)
    O = H.oracle()
    O.oracle_set_threads(os.cpu_count() or 1)
    try:
        out = {}
        for rel_tol in (1e-8, 1e-10):
            tol = rel_tol * np.linalg.norm(b)
            xr, _, sr, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=tol, max_it=20000,
                                          seed=SEED)
            H.oracle_scalar_test(True)
            try:
                xs, _, ss, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=tol,
                                              max_it=20000, seed=SEED)
            finally:
                H.oracle_scalar_test(False)
            opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=1,
                                    seed=SEED, precision=M.PREC_FP64)
            xg, fg, sg = ctx.solve_bsr(qp, opt, qp.x0)
            out[rel_tol] = (xr, sr, xs, ss, xg, sg)
            face_g = H.decide_face_planes(J, c, xg)
            face_r = H.decide_face_planes(J, c, xr)
            print(f"c1 tol {rel_tol:g}||b||: GPU {sg.iterations} iterations, oracle (reference "
                  f"test) {int(sr['iterations'])}, oracle (scalar test) {int(ss['iterations'])}; "
                  f"power iterations {sg.power_iters} / {int(sr['power_iters'])}; "
                  f"rel x err vs oracle {rel(xg, xr):.3e}; active rows {int(face_g.sum())} of "
                  f"{len(c)}, differing {int((face_g != face_r).sum())}")
            assert sg.code == 0 and sr["code"] == 0 and ss["code"] == 0
            assert np.array_equal(face_g, face_r)
            assert np.array_equal(face_g, H.decide_face_planes(J, c, xs))
            assert (J.matvec(xg) - c).min() >= -1e-9
            assert sg.power_iters == int(sr["power_iters"])
            assert abs(sg.spec_rad - sr["spec_rad"]) <= 1e-10 * sr["spec_rad"]
            assert (sg.iterations, sg.num_cg, sg.num_exp, sg.num_prop) == (
                int(ss["iterations"]), int(ss["num_cg"]), int(ss["num_exp"]),
                int(ss["num_prop"]))
            # the mixed form (FP32 A, FP64 steps and projection) on the same QP:
            # the oracle's active set, feasible, and at the tight tolerance
            # within 1e-8 of the oracle's solution
            optm = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=1,
                                     seed=SEED, precision=M.PREC_MIXED)
            xm, _, sm = ctx.solve_bsr(qp, optm, qp.x0)
            print(f"c1 mixed tol {rel_tol:g}||b||: {sm.iterations} iterations, rel x err vs "
                  f"oracle {rel(xm, xr):.3e}")
            assert sm.code == 0
            assert np.array_equal(H.decide_face_planes(J, c, xm), face_r)
            assert (J.matvec(xm) - c).min() >= -1e-9
            if rel_tol <= 1e-10:
                assert rel(xm, xr) <= 1e-8
        xr, _, xs, _, xg, _ = out[1e-10]
        assert rel(xg, xr) <= 1e-8
        assert rel(xg, xs) <= 1e-8
    finally:
        O.oracle_set_threads(1)
