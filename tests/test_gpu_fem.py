"""GPU FEM assembly (mprgp_fem_*): A = M + h^2 K and b = M(x + h v) + h^2 M g
+ h^2 K X of a tetrahedral mesh, against the host assembly of the same beam
(mprgp_beam_build), and solves from the GPU-assembled system."""
import numpy as np
import pytest

import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

KW = dict(extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=41)


def _sorted_rows(row_ptr, cols, vals):
    """Per row, blocks sorted by column (the host generator's order may differ)."""
    out_c, out_v = [], []
    for r in range(len(row_ptr) - 1):
        s, e = row_ptr[r], row_ptr[r + 1]
        o = np.argsort(cols[s:e], kind="stable")
        out_c.append(cols[s:e][o])
        out_v.append(vals[s:e][o])
    return np.concatenate(out_c), np.concatenate(out_v)


@pytest.mark.parametrize("dims", [(3, 2, 5), (6, 5, 12)])
def test_gpu_assembly_matches_host(ctx, dims):
    qp = M.beam(*dims, **KW)
    p = qp.params
    tets, X, x0, v0 = M.beam_mesh(*dims, **KW)
    assert np.array_equal(x0, qp.x0)
    fem = M.FemMesh(ctx, tets, X, p["young"], p["poisson"], p["rho"])
    fem.assemble(p["dt"], (0.0, p["gravity"], 0.0), x0, v0)
    rp, cols, vals, b, mass = fem.get()
    fem.close()
    assert np.array_equal(rp, qp.row_ptr)
    hc, hv = _sorted_rows(qp.row_ptr, np.asarray(qp.cols), np.asarray(qp.vals).reshape(-1, 9))
    assert np.array_equal(cols, hc)
    assert np.abs(vals - hv).max() <= 1e-13 * np.abs(hv).max()
    assert np.linalg.norm(b - qp.b) <= 1e-13 * np.linalg.norm(qp.b)
    assert np.all(mass > 0)


def test_solve_from_gpu_assembly(ctx):
    dims = (6, 5, 12)
    qp = M.beam(*dims, **KW)
    p = qp.params
    grav = (0.0, p["gravity"], 0.0)
    tets, X, x0, v0 = M.beam_mesh(*dims, **KW)
    fem = M.FemMesh(ctx, tets, X, p["young"], p["poisson"], p["rho"])
    pr = M.Problem(ctx, qp.nv)
    fem.assemble(p["dt"], grav, x0, v0, prob=pr, precisions=3)
    pr.set_planes(qp.plane_ptr, qp.planes)
    pr.set_x(x0)
    opt = M.default_options(tol=1e-10 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                            project_x0=1, seed=0x5EED)
    st = pr.solve(opt)
    xg = pr.get_x()
    xh, _, sh = ctx.solve_bsr(qp, opt, qp.x0)
    assert st.code == 0 and sh.code == 0
    assert np.linalg.norm(xg - xh) <= 1e-8 * np.linalg.norm(xh)
    # the next timestep: only b is recomputed on the device
    v1 = (xg - x0) / p["dt"]
    fem.rhs(p["dt"], grav, xg, v1, prob=pr)
    _, _, _, b1, mass = fem.get()
    m3 = np.repeat(mass, 3)
    g3 = np.tile(grav, qp.nv)
    kx = (qp.b - m3 * (x0 + p["dt"] * v0) - p["dt"] ** 2 * m3 * g3) / p["dt"] ** 2
    b1_ref = m3 * (xg + p["dt"] * v1) + p["dt"] ** 2 * m3 * g3 + p["dt"] ** 2 * kx
    assert np.linalg.norm(b1 - b1_ref) <= 1e-10 * np.linalg.norm(b1_ref)
    opt.project_x0 = 0
    st2 = pr.solve(opt)
    assert st2.code == 0
    fem.close()
    pr.close()
