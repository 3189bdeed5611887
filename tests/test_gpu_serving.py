"""Serving form: continuous batching (mprgp_server_*).

* every request's result is the same alone (mprgp_solve_bsr) and in the
  served mix, where requests arrive while others are on the GPU;
* follow-up timesteps warm-start from the resident scene and converge to the
  same solution as a cold solve of the same QP;
* admission respects the HBM budget (scenes are evicted, never overcommitted);
* all of the above hold for every server form: one synchronous run per step,
  two asynchronous lanes (small and large requests on separate streams), and
  three or more (power-method lanes sharing one queue).
Tolerance: the stopping test 1e-8 ||b||; x compared to 1e-12 relative
(in practice bitwise: each instance reduces in a fixed order).
"""
import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M
from mprgp_gb300 import workloads as W

pytestmark = pytest.mark.gpu
SEED = 0x5EED


def opts_for(qp, precision=M.PREC_MIXED, project=1):
    return M.default_options(tol=1e-8 * np.linalg.norm(qp.b), max_it=20000,
                             kind=M.KIND_PLANES, project_x0=project, seed=SEED,
                             precision=precision)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("lanes", [0, 2, 3, 5])
@pytest.mark.parametrize("precision", [M.PREC_FP64, M.PREC_MIXED])
def test_same_alone_and_in_the_mix(ctx, precision, lanes):
    # sizes on both sides of the cluster solver's limit (16 items of 256
    # vertices): the last two run on the engine
    dims = [(4, 4, 6), (9, 5, 12), (3, 3, 4), (6, 8, 10), (5, 5, 5), (12, 6, 9), (14, 8, 30),
            (16, 8, 32)]
    qps = [M.beam(*d, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=10 + i)
           for i, (d, e) in enumerate(zip(dims, [0, 2, 1, 2, 0, 1, 2, 1]))]
    assert qps[-1].nv > 16 * 256 and qps[-2].nv > 16 * 256
    alone = [ctx.solve_bsr(q, opts_for(q, precision), q.x0) for q in qps]
    srv = M.Server(ctx, quantum_phases=64, power_launches=128, max_slots=4, lanes=lanes)
    tickets, done = {}, {}
    # staggered arrivals: two at a time while earlier ones are in flight
    pending = list(range(len(qps)))
    steps = 0
    while len(done) < len(qps):
        for _ in range(2):
            if pending:
                i = pending.pop(0)
                tickets[srv.submit(i, qps[i], opts_for(qps[i], precision))] = i
        srv.step()
        steps += 1
        for t, i in list(tickets.items()):
            state, x, face, st, times = srv.result(t)
            if state == 2:
                assert st.code == 0
                done[i] = (x, face, st)
                del tickets[t]
        assert steps < 200000
    for i, (xa, fa, sa) in enumerate(alone):
        xs, fs, ss = done[i]
        assert rel(xs, xa) <= 1e-12, i
        assert np.array_equal(fs, fa)
        assert ss.iterations == sa.iterations
    srv.close()


@pytest.mark.parametrize("lanes", [0, 3])
def test_power_step_loop_served(ctx, lanes):
    """Served with the power-step loop (the default) and power runs cut into
    short pieces (20 launches a step: the loop stops at a body boundary and
    the next run resumes from the settled state), every result equals the
    launch loop's result for the request solved alone."""
    dims = [(14, 8, 30), (16, 8, 32), (12, 10, 24), (5, 5, 5)]
    qps = [M.beam(*d, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=40 + i)
           for i, (d, e) in enumerate(zip(dims, [2, 1, 2, 0]))]
    precision = M.PREC_MIXED
    ctx.set_tuning(64, 0)  # the launch loop for the requests alone
    try:
        alone = [ctx.solve_bsr(q, opts_for(q, precision), q.x0) for q in qps]
    finally:
        ctx.set_tuning(0, 0)
    try:
        srv = M.Server(ctx, quantum_phases=64, power_launches=20, max_slots=4, lanes=lanes)
        tickets, done = {}, {}
        for i, q in enumerate(qps):
            tickets[srv.submit(i, q, opts_for(q, precision))] = i
        steps = 0
        while len(done) < len(qps):
            srv.step()
            steps += 1
            for t, i in list(tickets.items()):
                state, x, face, st, times = srv.result(t)
                if state == 2:
                    assert st.code == 0
                    done[i] = (x, face, st)
                    del tickets[t]
            assert steps < 200000
        srv.close()
    finally:
        ctx.set_tuning(0, 0)
    for i, (xa, fa, sa) in enumerate(alone):
        xs, fs, ss = done[i]
        assert np.array_equal(xs, xa), i
        assert np.array_equal(fs, fa)
        assert (ss.iterations, ss.power_iters) == (sa.iterations, sa.power_iters)
        assert ss.spec_rad == sa.spec_rad


@pytest.mark.parametrize("lanes", [0, 2, 3])
def test_followup_warm_start(ctx, lanes):
    qp = M.beam(6, 5, 10, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=3)
    srv = M.Server(ctx, quantum_phases=128, power_launches=256, lanes=lanes)
    t = srv.submit(0, qp, opts_for(qp))
    while True:
        srv.step()
        state, x1, face1, st1, _ = srv.result(t)
        if state == 2:
            break
    assert st1.code == 0
    # next timestep: a new right-hand side, x warm-starts from x1 on the device
    m = np.repeat(W.lumped_mass(qp), 3)
    b2 = qp.b + m * (x1 - qp.x0)
    t2 = srv.submit(0, qp, opts_for(qp, project=0), b=b2, followup=True)
    while True:
        srv.step()
        state, x2, face2, st2, _ = srv.result(t2)
        if state == 2:
            break
    assert st2.code == 0
    # cold solve of the same next-step QP from the same start point
    qp2 = M.BeamQP(qp.nv, qp.row_ptr, qp.cols, qp.vals, b2, x1, qp.plane_ptr, qp.planes,
                   qp.params)
    xc, fc, sc = ctx.solve_bsr(qp2, opts_for(qp2, project=0), x1)
    assert sc.code == 0
    A, b, J, c = H.qp_from_beam(qp2)
    # the follow-up reuses the scene's power method (same A and seed): bitwise
    assert np.array_equal(x2, xc)
    assert st2.iterations == sc.iterations and st2.spec_rad == sc.spec_rad
    assert np.array_equal(H.decide_face_planes(J, c, x2), H.decide_face_planes(J, c, xc))
    srv.close()


@pytest.mark.parametrize("lanes", [0, 2, 3])
def test_admission_by_hbm_budget(ctx, lanes):
    qps = [M.beam(8, 8, 16, extra_planes_max=2, extra_planes_min=2, plane_mode=2, seed=s)
           for s in range(4)]
    one = M.lib().mprgp_problem_bytes(qps[0].nv, qps[0].nnzb, len(qps[0].planes), 3)
    srv = M.Server(ctx, hbm_budget=int(2.5 * one), quantum_phases=64, power_launches=64,
                   lanes=lanes)
    tickets = [srv.submit(i, q, opts_for(q)) for i, q in enumerate(qps)]
    max_running, finished = 0, 0
    for _ in range(100000):
        running, queued, completed = srv.step()
        budget, used, scenes = srv.info()
        assert used <= budget and scenes <= 2
        max_running = max(max_running, running)
        for t in list(tickets):
            state, x, face, st, _ = srv.result(t)
            if state == 2:
                assert st.code == 0
                tickets.remove(t)
                finished += 1
        if finished == len(qps):
            break
    assert finished == len(qps) and max_running <= 2
    srv.close()


@pytest.mark.parametrize("lanes", [0, 3])
def test_invalid_request_fails_alone(ctx, lanes):
    """A request whose matrix has a column outside 0..nv-1 completes with
    MPRGP_INVALID; the requests beside it are served normally."""
    qps = [M.beam(5, 4, 6, extra_planes_max=1, extra_planes_min=1, plane_mode=2, seed=40 + i)
           for i in range(3)]
    cols = qps[1].cols.copy()
    cols[3] = -2
    q = qps[1]
    qps[1] = M.BeamQP(q.nv, q.row_ptr, cols, q.vals, q.b, q.x0, q.plane_ptr, q.planes, {})
    srv = M.Server(ctx, quantum_phases=128, power_launches=256, lanes=lanes)
    tickets = [srv.submit(i, qp, opts_for(qp)) for i, qp in enumerate(qps)]
    codes = {}
    for _ in range(200000):
        srv.step()
        for i, t in enumerate(tickets):
            if i in codes:
                continue
            try:
                state, x, face, st, _ = srv.result(t)
                if state == 2:
                    codes[i] = st.code
            except M.MPRGPError as e:  # a done ticket with an error code raises
                codes[i] = e.code
        if len(codes) == 3:
            break
    assert codes == {0: 0, 1: M.INVALID, 2: 0}
    srv.close()
