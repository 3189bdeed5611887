"""CPU tests of the oracle's additions for the measured runs:
  * its beam generator (oracle/beam_oracle.h) builds the library's beam QPs
    bit for bit, so the CPU side of the measurements needs no GPU library;
  * the scalar form of CGMonotonicStep's decrease test converges to the
    reference form's solution and active set, and only removes the
    expansions that the reference's rounding-level comparisons cause;
  * the power-method warm start across timesteps behaves as the reference's
    specRad (ev stored only when the method stops early).
"""
import ctypes as C

import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

BEAMS = [
    (4, 4, 16, {}),
    (3, 2, 5, dict(extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=11)),
    (5, 3, 7, dict(extra_planes_max=2, extra_planes_min=0, plane_mode=0, seed=8,
                   active_frac=0.6)),
    (6, 4, 5, dict(extra_planes_max=2, extra_planes_min=1, plane_mode=1, seed=5,
                   active_frac=0.4, facet_layers=2, max_tilt=0.7)),
    (9, 5, 13, dict(extra_planes_max=1, extra_planes_min=1, plane_mode=2, v0_sigma=0.2,
                    young=1e6, poisson=0.49, seed=123456789)),
]


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.dtype == np.float64 else a


@pytest.mark.parametrize("a,b,c,kw", BEAMS)
def test_oracle_beam_equals_library_beam_bitwise(lib_built, a, b, c, kw):
    p = M.beam(a, b, c, **kw)
    q = H.oracle_beam(a, b, c, **kw)
    for k in ("row_ptr", "cols", "vals", "b", "x0", "plane_ptr", "planes"):
        assert np.array_equal(bits(getattr(p, k)), bits(getattr(q, k))), k
    assert p.params == q.params


def test_oracle_beam_defaults_are_the_library_defaults(lib_built):
    P = M.BeamParams()
    M.lib().mprgp_beam_default(C.byref(P))
    lib_defaults = {k: getattr(P, k) for k, _ in M.BeamParams._fields_ if k not in "abc"}
    assert lib_defaults == H.BEAM_DEFAULTS


def test_serving_window_with_oracle_builder_is_the_same_window(lib_built):
    from mprgp_gb300 import workloads as W
    w1 = W.serving_window(24, 3, hi=(8, 8, 16))
    w2 = W.serving_window(24, 3, hi=(8, 8, 16), builder=H.oracle_beam)
    assert np.array_equal(w1.t_unit, w2.t_unit)
    for r1, r2 in zip(w1.reqs, w2.reqs):
        assert (r1.scene, r1.followup) == (r2.scene, r2.followup)
        if not r1.followup:
            assert np.array_equal(bits(r1.qp.vals), bits(r2.qp.vals))
            assert np.array_equal(bits(r1.qp.planes), bits(r2.qp.planes))


@pytest.mark.parametrize("kind,kw", [
    ("decoupled", dict(seed=1)),
    ("general", dict(extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=2)),
    ("general", dict(extra_planes_max=2, extra_planes_min=2, plane_mode=2, v0_sigma=0.2,
                     seed=3)),
])
def test_scalar_decrease_test_same_solution(kind, kw):
    qp = H.oracle_beam(6, 5, 18, **kw)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-10 * np.linalg.norm(b)
    xr, fr, sr, _ = H.oracle_solve(kind, A, b, qp.x0, J, c, tol=tol, max_it=20000)
    H.oracle_scalar_test(True)
    try:
        xs, fs, ss, _ = H.oracle_solve(kind, A, b, qp.x0, J, c, tol=tol, max_it=20000)
    finally:
        H.oracle_scalar_test(False)
    assert sr["code"] == 0 and ss["code"] == 0
    assert np.array_equal(H.decide_face_planes(J, c, xr), H.decide_face_planes(J, c, xs))
    assert np.linalg.norm(xs - xr) <= 1e-8 * np.linalg.norm(xr)
    # the same power method; the scalar test never expands more often
    assert ss["power_iters"] == sr["power_iters"] and ss["spec_rad"] == sr["spec_rad"]
    assert ss["num_exp"] <= sr["num_exp"]
    # the switch is off again: the reference form reproduces its own run
    xr2, _, sr2, _ = H.oracle_solve(kind, A, b, qp.x0, J, c, tol=tol, max_it=20000)
    assert np.array_equal(bits(xr2), bits(xr)) and sr2 == sr


def test_scalar_decrease_matches_function_values_away_from_rounding():
    """Where f(P(y)) - f(x) is well above rounding, both forms decide alike:
    on a loose tolerance the scalar form takes exactly the reference steps."""
    qp = H.oracle_beam(4, 4, 16, seed=1)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-4 * np.linalg.norm(b)
    runs = []
    for scalar in (False, True):
        H.oracle_scalar_test(scalar)
        H.oracle_trace(True)
        try:
            _, _, st, _ = H.oracle_solve("decoupled", A, b, qp.x0, J, c, tol=tol, max_it=20000)
            tr = H.oracle_get_trace()
        finally:
            H.oracle_trace(False)
            H.oracle_scalar_test(False)
        runs.append((st, tr))
    (sr, tr), (ss, ts) = runs
    assert np.array_equal(tr[:, :2], ts[:, :2])
    committed = tr[:, 0] == 1
    # recorded decreases f(P(y)) - f(x) agree where they are well above rounding
    big = committed & (np.abs(tr[:, 3]) > 1e-6 * np.abs(tr[:, 3]).max())
    assert big.sum() > 5
    assert np.allclose(tr[big, 3], ts[big, 3], rtol=1e-5)


def test_power_warm_start_across_timesteps():
    """MprgpFemSolver passes &power_ev (MprgpFemSolver.cpp:533): specRad starts
    from it when it holds a vector and stores its iterate only when it stops
    early (MPRGPSolver.h:62-74)."""
    qp = H.oracle_beam(4, 4, 12, extra_planes_max=1, extra_planes_min=1, seed=4)
    A, b, J, c = H.qp_from_beam(qp)
    tol = 1e-8 * np.linalg.norm(b)
    # loose enough that the power method stops early and stores ev
    x1, _, s1, ev1 = H.oracle_solve_warm("general", A, b, qp.x0, J, c, ev=None, tol=1e-3)
    assert s1["power_iters"] < 1001 and ev1 is not None
    x2, _, s2, ev2 = H.oracle_solve_warm("general", A, b, x1, J, c, ev=ev1, tol=1e-3,
                                         project_x0=False)
    assert s2["power_iters"] <= s1["power_iters"] and ev2 is not None
    # tight: the method runs to its cap and keeps the given ev unchanged
    _, _, s3, ev3 = H.oracle_solve_warm("general", A, b, x2, J, c, ev=ev2, tol=tol,
                                        project_x0=False)
    assert s3["power_iters"] == 1001 and np.array_equal(ev3, ev2)
    # from no ev and a tight tolerance nothing is stored
    _, _, s4, ev4 = H.oracle_solve_warm("general", A, b, qp.x0, J, c, ev=None, tol=tol)
    assert s4["power_iters"] == 1001 and ev4 is None and s4["code"] == 0
