"""GPU plane-constraint generation (mprgp_planes_collide) against the CPU
restatement of LinearConCollider::handle(plane) in tests/helpers.py: the same
plane lists, bitwise, for the general and the decoupled rule, and a solve
with the generated constraints."""
import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

pytestmark = pytest.mark.gpu


def _planes():
    t = np.array([0.1, -1.0, 0.05])
    t /= np.linalg.norm(t)
    return np.array([
        [0.0, 1.0, 0.0, 0.0],          # floor
        [1.0, 0.0, 0.0, 0.0],          # wall x = 0
        [0.0, 1.0, 0.0, 3e-5],         # near-duplicate of the floor (within 1e-4)
        [0.0, 0.0, 1.0, 0.0],          # wall z = 0
        [t[0], t[1], t[2], 0.185],     # tilted ceiling over the top layer
        [0.0, 1.0, 0.0, 0.0],          # exact duplicate of the floor
    ])


@pytest.mark.parametrize("decoupled", [False, True])
def test_collide_matches_restatement(ctx, decoupled):
    qp = M.beam(5, 4, 9, seed=51)
    pr = M.load_beam(ctx, qp, precisions=3)
    planes, delta = _planes(), 0.005
    m = pr.collide_planes(planes, delta, decoupled)          # the problem's current x (= x0)
    ptr, got = pr.get_planes()
    ref_ptr, ref = H.collide_planes(qp.x0, planes, delta, decoupled)
    assert m == len(ref)
    assert np.array_equal(ptr, ref_ptr)
    assert np.array_equal(got, ref)
    assert np.diff(ptr).max() <= (1 if decoupled else 3)
    # host positions give the same result
    x = qp.x0 + 0.004
    m2 = pr.collide_planes(planes, delta, decoupled, x=x)
    ptr2, got2 = pr.get_planes()
    ref_ptr2, ref2 = H.collide_planes(x, planes, delta, decoupled)
    assert m2 == len(ref2) and np.array_equal(ptr2, ref_ptr2) and np.array_equal(got2, ref2)
    pr.close()


def test_solve_with_generated_constraints(ctx):
    """Axis-aligned planes (floor, walls, a level ceiling): the monotone MPRGP
    of the reference stalls on tilted planes near free vertices, which the
    parity tests cover separately."""
    qp = M.beam(5, 4, 9, seed=52)
    pr = M.load_beam(ctx, qp, precisions=3)
    planes = np.array([[0.0, 1.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0],
                       [0.0, -1.0, 0.0, 0.185]])
    pr.collide_planes(planes, 0.005)
    ptr, pl = pr.get_planes()
    opt = M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                            project_x0=1, seed=0x5EED)
    st = pr.solve(opt)
    assert st.code == 0
    x = pr.get_x()
    # every generated constraint holds: n . x_v + p >= -1e-9
    v = np.repeat(np.arange(qp.nv), np.diff(ptr))
    gap = np.einsum("ij,ij->i", pl[:, :3], x.reshape(-1, 3)[v]) + pl[:, 3]
    assert gap.min() >= -1e-9
    # the same QP through the one-call entry gives the same solution
    q2 = M.BeamQP(qp.nv, qp.row_ptr, qp.cols, qp.vals, qp.b, qp.x0, ptr, pl, qp.params)
    x2, _, s2 = ctx.solve_bsr(q2, opt, qp.x0)
    assert s2.code == 0
    assert np.linalg.norm(x - x2) <= 1e-10 * np.linalg.norm(x2)
    pr.close()


def test_more_than_three_planes_is_an_error(ctx):
    """The solver holds at most 3 planes per vertex: a corner vertex within
    delta of four planes is rejected, not silently truncated."""
    qp = M.beam(3, 3, 3, seed=53)
    pr = M.load_beam(ctx, qp, precisions=1)
    four = np.array([[0.0, 1.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0],
                     [np.sqrt(0.5), 0.0, np.sqrt(0.5), 0.0]])
    with pytest.raises(M.MPRGPError):
        pr.collide_planes(four, 0.005)
    pr.close()
