"""GPU ICA solver (mprgp_ica_solve, the reference's ICASolver.h:287-463)
against its CPU restatement (oracle/ica_oracle.h).

Both perform the same operations in the same order without fused
multiply-adds, so x, lambda, the iteration count and the number of projected
Gauss-Seidel sweeps are compared bitwise; the residual, a reduction whose
summation order differs between the two, to 1e-12 relative.  Sizes cover one
CTA, several CTAs and a grid of every SM (dependency-level sweep across CTAs).
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import helpers as H
import mprgp_gb300 as M

pytestmark = pytest.mark.gpu


def _start(qp):
    A, b, J, c = H.qp_from_beam(qp)
    As = sp.csr_matrix((A.val, A.idx, A.ptr), shape=(A.rows, A.cols))
    return spl.spsolve(As.tocsc(), b)  # the reference's FEM loop starts from the unconstrained solve


@pytest.mark.parametrize("dims,extra,seed,max_it,tol", [
    ((4, 4, 16), 0, 1, 1000, 1e-4),      # c0-shaped, one plane a vertex, 2 CTAs
    ((3, 3, 4), 2, 7, 1000, 1e-6),       # 3 planes a vertex
    ((12, 6, 20), 1, 5, 300, 1e-5),      # several CTAs
    ((24, 16, 96), 2, 9, 12, 1e-12),     # > 152 x 256 vertices: every SM, fixed 12 iterations
])
def test_ica_bitwise_equals_oracle(ctx, dims, extra, seed, max_it, tol):
    qp = M.beam(*dims, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2, seed=seed)
    x0 = _start(qp) if qp.nv < 5000 else qp.x0
    xo, lo, so = H.oracle_ica(qp, x0, max_it=max_it, tol=tol)
    xg, lg, sg = ctx.ica_solve(qp, x0, max_it=max_it, tol=tol)
    assert sg.iterations == so["iterations"]
    assert sg.converged == so["converged"]
    assert sg.pgs_sweeps == so["pgs_sweeps"]
    assert np.array_equal(xg, xo)
    assert np.array_equal(lg, lo)
    assert sg.residual == pytest.approx(so["residual"], rel=1e-12)
    assert sg.levels >= 1 and sg.device_ms > 0


def test_ica_solution_matches_mprgp(ctx):
    """Converged tightly, ICA and the GPU MPRGP solve the same QP."""
    qp = M.beam(6, 4, 10, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=3)
    nb = float(np.linalg.norm(qp.b))
    xg, lg, sg = ctx.ica_solve(qp, _start(qp), max_it=100000, tol=1e-11 * nb, gs_tol=1e-14)
    assert sg.converged == 1
    opt = M.default_options(tol=1e-11 * nb, max_it=20000, kind=M.KIND_PLANES, project_x0=1,
                            seed=0x5EED, precision=M.PREC_FP64)
    xm, face, st = ctx.solve_bsr(qp, opt, qp.x0)
    assert st.code == 0
    assert np.linalg.norm(xg - xm) <= 1e-8 * np.linalg.norm(xm)
    A, b, J, c = H.qp_from_beam(qp)
    assert np.array_equal(H.decide_face_planes(J, c, xg), H.decide_face_planes(J, c, xm))
    assert lg.min() >= 0.0


def test_ica_rejects_bad_input(ctx):
    qp = M.beam(2, 2, 3, seed=2)
    # a row without its diagonal block
    cols = qp.cols.copy()
    k = int(np.nonzero(cols[qp.row_ptr[0]:qp.row_ptr[1]] == 0)[0][0])
    cols[qp.row_ptr[0] + k] = 1 if qp.cols[qp.row_ptr[0] + k + 1] != 1 else 2
    bad = M.BeamQP(qp.nv, qp.row_ptr, cols, qp.vals, qp.b, qp.x0, qp.plane_ptr, qp.planes, {})
    with pytest.raises(M.MPRGPError) as e:
        ctx.ica_solve(bad, qp.x0)
    assert e.value.code == M.INVALID
    # four planes on one vertex
    pp = qp.plane_ptr.copy()
    pl = np.vstack([qp.planes[:1]] * 3 + [qp.planes])
    pp[1:] += 3
    bad = M.BeamQP(qp.nv, qp.row_ptr, qp.cols, qp.vals, qp.b, qp.x0, pp, pl, {})
    with pytest.raises(M.MPRGPError) as e:
        ctx.ica_solve(bad, qp.x0)
    assert e.value.code == M.INVALID
