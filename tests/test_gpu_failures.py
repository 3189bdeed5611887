"""Failure paths of the C ABI, produced from the host side (no GPU fault):

  * a bounded device wait that runs out returns MPRGP_TIMEOUT: the
    persistent engine's grid barrier is given a wait limit far shorter than
    any phase, so the first CTA to reach it gives up, sets the error flag and
    every CTA returns; the context stays usable;
  * a NaN in b returns MPRGP_BREAKDOWN at the first loop top (the residual is
    NaN, so no step could meet the stopping test; the reference would iterate
    to max_it and return -1), x is left as passed, and the context stays
    usable;
  * admission of the serving form re-reads the device's free memory: a new
    scene that would leave less than the server's reserve free waits for room
    (idle scenes are evicted), and one that cannot fit while nothing else is
    in flight completes with MPRGP_OOM.
"""
import numpy as np
import pytest

import mprgp_gb300 as M

pytestmark = pytest.mark.gpu

SEED = 0x5EED


def corner(a, b, c, seed=1):
    return M.beam(a, b, c, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=seed)


def opts(qp, **kw):
    base = dict(tol=1e-8 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES, project_x0=1,
                seed=SEED)
    base.update(kw)
    return M.default_options(**base)


@pytest.fixture()
def fresh_ctx(lib_built):
    c = M.Context(0)
    yield c
    c.close()


def test_wait_limit_timeout_then_normal_solve(fresh_ctx):
    ctx = fresh_ctx
    qp = corner(12, 12, 30)  # 5,239 vertices: 21 items, the persistent engine
    assert qp.nv > 16 * 256
    with pytest.raises(M.MPRGPError) as ei:
        ctx.solve_bsr(qp, opts(qp, wait_limit_s=1e-9), qp.x0)
    assert ei.value.code == M.TIMEOUT
    x, face, st = ctx.solve_bsr(qp, opts(qp), qp.x0)
    assert st.code == 0 and st.residual <= 1e-8 * np.linalg.norm(qp.b)


@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
@pytest.mark.parametrize("dims", [(4, 4, 16), (12, 12, 30)])  # cluster solver, engine
def test_nan_in_b_is_a_breakdown(fresh_ctx, dims, precision):
    ctx = fresh_ctx
    qp = corner(*dims)
    bad = M.BeamQP(qp.nv, qp.row_ptr, qp.cols, qp.vals, qp.b.copy(), qp.x0, qp.plane_ptr,
                   qp.planes, qp.params)
    bad.b[7] = np.nan
    x_in = qp.x0.copy()
    o = opts(qp, precision=precision)
    xs = x_in.copy()
    st = M.Stats()
    rc = M.lib().mprgp_solve_bsr(ctx.h, bad.nv, bad.nnzb, M._ptr(bad.row_ptr), M._ptr(bad.cols),
                                 M._ptr(bad.vals), M._ptr(bad.b), M._ptr(bad.plane_ptr),
                                 M._ptr(bad.planes), None, None, M.C.byref(o), M._ptr(xs), None,
                                 None, M.C.byref(st))
    assert rc == M.BREAKDOWN and st.code == M.BREAKDOWN
    assert st.iterations == 0
    assert np.array_equal(xs, x_in)  # x left as passed
    x, face, st2 = ctx.solve_bsr(qp, o, qp.x0)
    assert st2.code == 0


def test_nan_in_b_plain_algorithm(fresh_ctx):
    """The box-bound kind runs the plain MPRGP::solve (MPRGPSolver.h:356-396)."""
    ctx = fresh_ctx
    qp = corner(4, 4, 16)
    L = np.full(qp.n, -1e30)
    L[1::3] = 0.0
    U = np.full(qp.n, 1e30)
    b = qp.b.copy()
    b[4] = np.nan
    bad = M.BeamQP(qp.nv, qp.row_ptr, qp.cols, qp.vals, b, qp.x0, qp.plane_ptr, qp.planes,
                   qp.params)
    o = opts(qp, kind=M.KIND_BOX)
    with pytest.raises(M.MPRGPError) as ei:
        ctx.solve_bsr(bad, o, qp.x0, L=L, U=U)
    assert ei.value.code == M.BREAKDOWN
    x, face, st = ctx.solve_bsr(qp, o, qp.x0, L=L, U=U)
    assert st.code == 0


def _serve(srv, qps, opt_of, cap=200000):
    tickets = {srv.submit(i, q, opt_of(q)): i for i, q in enumerate(qps)}
    codes, max_scenes = {}, 0
    for _ in range(cap):
        srv.step()
        max_scenes = max(max_scenes, srv.info()[2])
        for t in list(tickets):
            try:
                state, x, face, st, _ = srv.result(t)
            except M.MPRGPError as e:  # completed with an error status
                codes[tickets.pop(t)] = e.code
                continue
            if state == 2:
                codes[tickets.pop(t)] = st.code
        if not tickets:
            break
    return codes, max_scenes


@pytest.mark.parametrize("lanes", [0, 3])
def test_admission_waits_for_device_room(fresh_ctx, lanes):
    """Room for one scene only: the second new scene waits until the first is
    idle and evicted, then both are solved."""
    ctx = fresh_ctx
    qps = [corner(24, 24, 48, seed=s) for s in (1, 2)]
    mixed = lambda q: opts(q, precision=M.PREC_MIXED)  # noqa: E731
    # warm the context (its run buffers come from the same pool) and measure
    # what one resident scene takes
    warm = M.Server(ctx, quantum_phases=-1, power_launches=1003, lanes=lanes)
    assert _serve(warm, qps[:1], mixed)[0] == {0: 0}
    warm.close()
    srv = M.Server(ctx, quantum_phases=-1, power_launches=1003, lanes=lanes)
    before = ctx.room()
    assert _serve(srv, qps[:1], mixed)[0] == {0: 0}
    one = before - ctx.room()
    srv.close()
    assert one > 0
    # admission asks for the footprint estimate `need`; after the first scene
    # the room is `one` smaller, so the reserve lets exactly one scene in
    need = M.lib().mprgp_problem_bytes(qps[0].nv, qps[0].nnzb, len(qps[0].planes), 3)
    srv = M.Server(ctx, quantum_phases=-1, power_launches=1003, lanes=lanes,
                   hbm_reserve=ctx.room() - need - one // 2)
    codes, max_scenes = _serve(srv, qps, mixed)
    srv.close()
    assert codes == {0: 0, 1: 0}
    assert max_scenes == 1


def test_admission_without_room_is_oom(fresh_ctx):
    ctx = fresh_ctx
    qp = corner(6, 6, 12)
    srv = M.Server(ctx, quantum_phases=-1, power_launches=1003,
                   hbm_reserve=ctx.room() + (1 << 40))
    codes, _ = _serve(srv, [qp], lambda q: opts(q))
    srv.close()
    assert codes == {0: M.OOM}
    # the context still serves with room
    srv = M.Server(ctx, quantum_phases=-1, power_launches=1003)
    codes, _ = _serve(srv, [qp], lambda q: opts(q))
    srv.close()
    assert codes == {0: 0}
