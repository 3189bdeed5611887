"""mprgp_solve_noalloc: the solve for callers that cannot allocate device
memory while they solve (real-time loops kept off the allocator, plug-ins
inside a program that owns all device memory, hosts under a fixed GPU memory
quota).  It must give the same answer as the allocating entry point
mprgp_solve_bsr, call after call, although every call reuses the same
file-scope scratch array, and a call must not change the device's free
memory.  Collected last on purpose (test_zz_*).
"""
import numpy as np
import pytest

import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype, copy=False)).cuda()


def _stage(torch, qp):
    return dict(rp=_dev(torch, qp.row_ptr, np.int32), cols=_dev(torch, qp.cols, np.int32),
                vals=_dev(torch, qp.vals.reshape(-1), np.float64),
                b=_dev(torch, qp.b, np.float64), pp=_dev(torch, qp.plane_ptr, np.int32),
                pl=_dev(torch, qp.planes.reshape(-1), np.float64),
                x=_dev(torch, qp.x0, np.float64),
                face=torch.zeros(len(qp.planes), dtype=torch.uint8, device="cuda"))


def _call(torch, qp, d, opt):
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    code, st = M.solve_noalloc(stream.cuda_stream, qp.nv, qp.nnzb, d["rp"].data_ptr(),
                               d["cols"].data_ptr(), d["vals"].data_ptr(), d["b"].data_ptr(),
                               d["pp"].data_ptr(), d["pl"].data_ptr(), opt, d["x"].data_ptr(),
                               d["face"].data_ptr())
    torch.cuda.synchronize()
    return code, st


def _solve_noalloc(torch, qp, opt):
    d = _stage(torch, qp)
    code, st = _call(torch, qp, d, opt)
    return code, st, d["x"].cpu().numpy(), d["face"].cpu().numpy()


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
        assert st.power_passes == st_ref.power_passes > 0


def test_noalloc_allocates_nothing(ctx):
    """After a first call (the one-time set-up), a call leaves the device's
    free memory exactly as it found it."""
    torch = pytest.importorskip("torch")
    qp = M.beam(5, 4, 9, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=3)
    opt = M.default_options(tol=1e-8 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                            project_x0=1, seed=SEED)
    first = _stage(torch, qp)
    assert _call(torch, qp, first, opt)[0] == 0
    again = _stage(torch, qp)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    code, st = _call(torch, qp, again, opt)
    free1, _ = torch.cuda.mem_get_info()
    assert code == 0 and st.code == 0
    assert free1 == free0
    assert torch.equal(again["x"], first["x"])


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    qp = M.beam(32, 32, 64, extra_planes_max=2, extra_planes_min=2, plane_mode=2)
    opt = M.default_options(tol=1e-8 * np.linalg.norm(qp.b), kind=M.KIND_PLANES, project_x0=1)
    with pytest.raises(M.MPRGPError) as ei:
        _solve_noalloc(torch, qp, opt)
    assert ei.value.code == M.INVALID
    assert "64 MiB" in str(ei.value)
