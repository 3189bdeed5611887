"""mprgp_solve_noalloc: the solve for callers that cannot allocate device
memory (graph-replayed simulation steps, real-time loops, fixed GPU memory
budgets).  It must give the same answer as the allocating entry point
mprgp_solve_bsr, call after call, although every call reuses the same
file-scope scratch array.  Collected last on purpose (test_zz_*).
"""
import numpy as np
import pytest

import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype, copy=False)).cuda()


def _solve_noalloc(torch, qp, opt):
    rp = _dev(torch, qp.row_ptr, np.int32)
    cols = _dev(torch, qp.cols, np.int32)
    vals = _dev(torch, qp.vals.reshape(-1), np.float64)
    b = _dev(torch, qp.b, np.float64)
    pp = _dev(torch, qp.plane_ptr, np.int32)
    pl = _dev(torch, qp.planes.reshape(-1), np.float64)
    x = _dev(torch, qp.x0, np.float64)
    face = torch.zeros(len(qp.planes), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    code, st = M.solve_noalloc(stream.cuda_stream, qp.nv, qp.nnzb, rp.data_ptr(),
                               cols.data_ptr(), vals.data_ptr(), b.data_ptr(), pp.data_ptr(),
                               pl.data_ptr(), opt, x.data_ptr(), face.data_ptr())
    torch.cuda.synchronize()
    return code, st, x.cpu().numpy(), face.cpu().numpy()


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_noalloc_matches_allocating_entry(ctx, precision):
    torch = pytest.importorskip("torch")
    # Two calls in a row on different problems: the second sees the first's
    # leftovers in the shared scratch array.
    for dims, extra, seed in [((4, 4, 16), 2, 1), ((5, 4, 9), 2, 3)]:
        qp = M.beam(*dims, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2,
                    seed=seed)
        tol = 1e-10 * np.linalg.norm(qp.b)
        opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=1,
                                seed=SEED, precision=precision)
        x_ref, face_ref, st_ref = ctx.solve_bsr(qp, opt, qp.x0)
        code, st, x, face = _solve_noalloc(torch, qp, opt)
        assert code == 0 and st.code == 0 and st_ref.code == 0
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
        assert np.array_equal(face, face_ref)
        assert st.iterations == st_ref.iterations


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    qp = M.beam(32, 32, 64, extra_planes_max=2, extra_planes_min=2, plane_mode=2)
    opt = M.default_options(tol=1e-8 * np.linalg.norm(qp.b), kind=M.KIND_PLANES, project_x0=1)
    with pytest.raises(M.MPRGPError) as ei:
        _solve_noalloc(torch, qp, opt)
    assert ei.value.code == M.INVALID
    assert "64 MiB" in str(ei.value)
