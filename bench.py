#!/usr/bin/env python3
"""MPRGP QP solves/s on GB300 (one JSON line on rank 0).

Default workload (--config c4): the serving stream.  A window of 512 seeded
requests with Poisson arrivals at 5000 req/s: beams of 4x4x4..32x32x64
Kuhn-tet cubes (E=1e5, nu=0.45, rho=1000, h=0.01) in contact with the floor
and 0-2 walls (1-3 planes per vertex), 30 % of them follow-up timesteps of a
live scene; every request solved to ||g_P|| <= 1e-8 ||b||.  A step is one
window served by the continuous-batching server (mixed form):
  value  solves/s with every request's arrays staged in device memory
         before the timed region (the server copies them at admission);
  e2e    the same stream submitted by reference to pinned host buffers,
         copied host->device at admission, x and face read back;
beside it the plain FP64 GPU solve of the same stream one request at a time,
the error of every served result against it, an arrival-rate sweep, the
roofline of the solver kernels and the CPU restatement (oracle/) on a
bounded sample.

Other workloads: c1 (one 32x32x128 beam, 421,443 DOF; --form plain|mixed),
c0 (4x4x16, floor), c2 (256 uneven beams in one batched run), c3 (48x48x144,
E=1e6, nu=0.49, 20 warm-started timesteps, mixed vs FP64 per step).
--impl reference times the CPU restatement of the reference MPRGP (oracle/)
on the host cores instead.  --spmv times the standalone y = A x
(mprgp_problem_spmv) on the c0/c1/c3 matrix, FP64 and FP32, with its HBM
and FP64-unit roofline fractions.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (a, b, c, extra planes, plane mode, young, poisson, v0 sigma)
    "c1": (32, 32, 128, 2, 2, 1e5, 0.45, 0.1),
    # c2 (batch of 256 uneven beams) is generated by mprgp_gb300.workloads.batch
    "c0": (4, 4, 16, 0, 2, 1e5, 0.45, 0.1),
    "c3": (48, 48, 144, 2, 2, 1e6, 0.49, 0.1),
}
REL_TOL = 1e-8
SEED = 0x5EED
FLUSH_BYTES = 256 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c4", choices=sorted(WORKLOADS) + ["c2", "c4"])
    ap.add_argument("--form", default=None, choices=["plain", "mixed"],
                    help="plain FP64 or mixed precision (default: mixed for c2/c4, plain else)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="c4: skip the arrival-rate sweep")
    ap.add_argument("--no-plain", action="store_true",
                    help="c4: skip the plain FP64 one-at-a-time play (profiling runs)")
    ap.add_argument("--no-ica", action="store_true",
                    help="c0/c1: skip the ICA comparison solve beside the line")
    ap.add_argument("--lanes", type=int, default=SERVE_LANES, choices=[0, 2, 3, 4, 5, 6],
                    help="c4: server form (0 one synchronous run per step, 2 asynchronous "
                         "small/large lanes, 3 plus a lane for the large ones' power method)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the launch-shape autotuner (mprgp_gb300.autotune) before warm-up")
    ap.add_argument("--ctas-per-sm", type=int, default=0,
                    help="with --tuning: cap on the persistent grid's CTAs per SM (0 = all resident)")
    ap.add_argument("--single", action="store_true",
                    help="c3: one solve of the timestep beam's first QP (the c0/c1 line) instead "
                         "of the 20-timestep loop")
    ap.add_argument("--spmv", action="store_true",
                    help="time the standalone y = A x (mprgp_problem_spmv) on the config's "
                         "matrix instead of the solver, FP64 and FP32 values")
    ap.add_argument("--tuning", type=int, default=None,
                    help="launch-form bits for mprgp_context_set_tuning (bit 6: phase-kernel power "
                         "loop instead of the power-step loop; bit 2: power loop from "
                         "host-stream launches instead of the CUDA-graph WHILE loop)")
    return ap.parse_args()


def workload_qp(name, builder=None):
    """The config's beam QP, from the library's generator or `builder` (the
    oracle's, bitwise the same, for the CPU arm)."""
    if builder is None:
        import mprgp_gb300 as M
        builder = M.beam
    a, b, c, extra, mode, E, nu, sig = WORKLOADS[name]
    return builder(a, b, c, extra_planes_max=extra, extra_planes_min=extra, plane_mode=mode,
                   young=E, poisson=nu, v0_sigma=sig, seed=1)


def workload_desc(name, qp):
    a, b, c, extra, mode, E, nu, sig = WORKLOADS[name]
    return {"workload": f"beam {a}x{b}x{c} cubes, 6 Kuhn tets each: {qp.nv} vertices, "
                        f"{qp.n} DOF, {qp.nnzb} 3x3 blocks; floor + walls x,z "
                        f"({len(qp.planes)} plane rows); E={E:g} nu={nu} rho=1000 h=0.01; "
                        f"tol 1e-8*||b||",
            "config": name}


def spmv_bytes(qp, s_a):
    """Algorithmic bytes of one y = A x at matrix precision s_a (8 or 4 bytes):
    A (values + block column), row pointers, x and y at the same precision.
    The block column counts 2 bytes: the matrix passes read 16-bit offsets
    from the row's vertex, which every beam's offsets fit."""
    return qp.nnzb * (9 * s_a + 2) + (qp.nv + 1) * 4 + 2 * qp.n * s_a


# n-vector traffic of the solver phases beyond the matrix pass, in FP64
# vectors of n = 3 nv unknowns (8n bytes each; an FP32 shadow counts half),
# counted from the row functions of mprgp_gb300/csrc/engine.cu.  The matrix
# pass's own x gather and y store are in spmv_bytes.
#   power pass   FP32 form: t_k read, t_{k-1} read, t_k store (3 x 4n)   1.5
#                FP64 form: the same in FP64                              3
#   CG step      PH_CG_SPMV: g, z, p read; p', Ap stored (mixed: p' FP32
#                shadow, second FP32 source)                              5 (+1)
#                PH_CG_YF: x, p, Ap, g read; y, g_y, delta, z, beta
#                stored (mixed: z FP32 shadow)                            9 (+0.5)
#   expansion    PH_EXP_A 2, PH_EXP_B 4, PH_EXP_C 6 (mixed +1)           12 (+1)
#   proportioning PH_PROP_A 4, PH_PROP_B 9 (mixed +1)                    13 (+1)
#   any other phase (init, CG entry, residual replacement, projections)   6
# and each phase that reads the constraints reads 49 B per plane row
# (n, c, 1/|n|^2, 1/(n.D^-1 n), face).
VEC_K = {"pow32": 1.5, "pow64": 3.0, "cg": 14.0, "cg_mixed": 15.5, "exp": 12.0, "exp_mixed": 13.0,
         "prop": 13.0, "prop_mixed": 14.0, "other": 6.0}
PLANE_ROW_BYTES = 49


def vector_bytes(st, qp, mixed, include_power=True):
    """Estimated n-vector and constraint bytes of a solve beyond its matrix
    passes, from its step counts (VEC_K); include_power=False leaves out the
    power method's."""
    n8 = 8 * qp.n
    m = len(qp.planes)
    pw = int(st.power_passes)
    cg, ex, pr = int(st.num_cg), int(st.num_exp), int(st.num_prop)
    other = max(0, int(st.phases) - pw - 2 * cg - 3 * ex - 2 * pr)
    k = (VEC_K["pow32" if mixed else "pow64"] * pw * include_power
         + VEC_K["cg_mixed" if mixed else "cg"] * cg
         + VEC_K["exp_mixed" if mixed else "exp"] * ex
         + VEC_K["prop_mixed" if mixed else "prop"] * pr + VEC_K["other"] * other)
    return int(k * n8 + PLANE_ROW_BYTES * m * (cg + 2 * ex + pr + other))


def read_stream_peak():
    """Read-only HBM throughput measured here and now: torch's sum over a
    1 GiB FP32 buffer, L2 flushed before each of 6 timed runs, best run.  A
    matrix pass reads far more than it writes, so its fraction of this figure
    says how close it is to the stream it is bound by (the copy peak counts
    read and write bytes alike)."""
    import torch
    x = torch.ones(256 << 20, dtype=torch.float32, device="cuda")
    fl = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for r in range(7):
        fl.fill_(r)
        e0.record()
        x.sum()
        e1.record()
        e1.synchronize()
        if r:
            best = min(best, e0.elapsed_time(e1))
    del x, fl
    return round(4.0 * (256 << 20) / best / 1e6, 1)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(name, form, kernel="engine_kernel"):
    """Per-launch DRAM bytes (read + write) of a kernel from the committed ncu
    summary profiles/traffic.json, keyed "<config>:<form>:<kernel>"."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return d.get(f"{name}:{form}:{kernel}")


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        # the timed region as an NVTX range ("timed"), so that a profiler can
        # capture exactly it (ncu --nvtx --nvtx-include "timed/")
        self.nvtx = False
        try:
            import torch
            torch.cuda.nvtx.range_push("timed")
            self.nvtx = True
        except Exception:
            pass
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvtx:
            import torch
            torch.cuda.nvtx.range_pop()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [t.strip() for t in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax = float(p[2])
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def autotune_ctx(args, ctx, sample, precision, power_cache=False, fixed=None):
    """Untimed: pick launch shapes for this workload on a sample of it (an
    explicit --tuning wins).  power_cache: tune the solves that reuse a first
    solve's power method (timestep loops)."""
    if args.tuning is not None:
        ctx.set_tuning(args.tuning, args.ctas_per_sm)
        return {"explicit_tuning_bits": args.tuning}
    if args.no_autotune:
        return None
    from mprgp_gb300 import autotune
    r = autotune.tune(ctx, sample, precision=precision, reps=1, use_cache=False,
                      power_cache=power_cache, fixed=fixed)
    return {"config": r["config"], "sample_ms": round(r["ms"], 3),
            "default_ms": round(r["default_ms"], 3), "candidates": len(r["tried"]),
            "seconds": round(r["seconds"], 2), "sample_size": len(sample)}


def power_form(tuning):
    """The power-method loop a tuning selects (autotuner config or explicit
    mprgp_context_set_tuning bits)."""
    if not tuning:
        return "step"
    if "config" in tuning:
        f = tuning["config"].get("power", "step")
        return {"step-stream": "step", "stream": "graph"}.get(f, f)
    bits = tuning.get("explicit_tuning_bits", 0)
    if bits & 2:
        return "engine"
    if bits & 32:
        return "persistent"
    return "graph" if bits & 64 else "step"


def cpu_baseline(qp, threads=1):
    """One full solve of the same QP by the CPU restatement of the reference."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers as H
    A, b, J, c = H.qp_from_beam(qp)
    H.oracle().oracle_set_threads(threads)
    tol = REL_TOL * float(np.linalg.norm(b))
    t = time.perf_counter()
    x, face, st, _ = H.oracle_solve("general", A, b, qp.x0, J, c, tol=tol, max_it=20000,
                                    seed=SEED)
    dt = time.perf_counter() - t
    return dt, st


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_gb300(args):
    import torch
    import mprgp_gb300 as M
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    M.build()
    qp = workload_qp(args.config)
    tol = REL_TOL * float(np.linalg.norm(qp.b))
    ctx = M.Context(local)
    mixed = args.form == "mixed"
    prec = M.PREC_MIXED if mixed else M.PREC_FP64
    tuning = autotune_ctx(args, ctx, [qp], prec)
    opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=1, seed=SEED,
                            precision=prec)
    prob = M.load_beam(ctx, qp, precisions=3 if mixed else 1)
    prob.set_power_cache(False)  # every timed solve runs its power method
    x0_dev = torch.from_numpy(qp.x0).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def one_step():
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        prob.set_x(x0_dev.data_ptr(), on_device=True)
        st = prob.solve(opt)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), st

    for _ in range(args.warmup):
        one_step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    times, stats = [], []
    launches0, solver0, power0 = ctx.counters()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ms, st = one_step()
            times.append(ms)
            stats.append(st)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches1, solver1, power1 = ctx.counters()
    launches = launches1 - launches0
    if world > 1:
        torch.distributed.barrier()
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    st = stats[-1]
    for s in stats:
        if s.code != 0:
            raise RuntimeError(f"solve did not converge: {s.as_dict()}")
    value = world * args.steps / (total_ms / 1e3)
    # Roofline.  The dominant kernel of a solve is the power kernel (1001 of
    # its ~1150 matrix passes, one pass per launch of the graph loop): bytes
    # of one matrix pass / the loop's device time per working launch.  The
    # engine (the MPRGP phases) is reported beside it.
    s_pow = 4 if mixed else 8
    pass_bytes = spmv_bytes(qp, s_pow)
    passes = sum(s.power_passes for s in stats)
    power_ms = power1 - power0
    peak, peak_kind = measured_peaks()
    read_peak = read_stream_peak()
    all_bytes = sum(s.spmv_fp64 * spmv_bytes(qp, 8) + s.spmv_fp32 * spmv_bytes(qp, 4)
                    for s in stats)
    eng_bytes = all_bytes - passes * pass_bytes
    eng_vec = sum(vector_bytes(s, qp, mixed, include_power=False) for s in stats)
    if power_ms > 0:  # the power loop ran as its own kernel
        pow_launch_ms = power_ms / max(1, passes)
        achieved = pass_bytes / (pow_launch_ms / 1e3) / 1e9
        form = power_form(tuning)
        kname = {"step": "power_step_kernel", "persistent": "power_persistent_kernel"}.get(
            form, "power_kernel")
        traffic = committed_traffic(args.config, args.form, kname)
        dominant = {"step": "mprgp::power_step_kernel (power-step loop, CUDA graph)",
                    "persistent": "mprgp::power_persistent_kernel (one cooperative launch)"}.get(
            form, "mprgp::phase_kernel (power phases, CUDA-graph loop)")
        eng_ms = (solver1 - solver0) - power_ms
    else:  # the tuning put the power phases into the persistent engine
        pow_launch_ms = (solver1 - solver0) / max(1, len(stats))
        achieved = (all_bytes / max(1, len(stats))) / (pow_launch_ms / 1e3) / 1e9
        pass_bytes = all_bytes / max(1, len(stats))
        passes = len(stats)
        traffic = None
        dominant = "mprgp::engine_kernel (power and MPRGP phases, one launch per solve)"
        eng_bytes, eng_ms = all_bytes, solver1 - solver0
    eng_achieved = (eng_bytes + eng_vec) / (eng_ms / 1e3) / 1e9 if eng_ms > 0 else None
    line = {
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(value, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if not mixed else "f32 A (f32 accumulate) + f64 steps/projection/residual",
        "data": "synthetic (seeded beam QP, no dataset)",
        "config": dict(workload_desc(args.config, qp), form=args.form + "-" + ("mixed" if mixed else "fp64"),
                       l2="flushed between solves (256 MB device write)",
                       parallelism="replicas" if world > 1 else "single GPU", autotune=tuning),
        "latency_ms": {"p50": round(float(np.percentile(times, 50)), 4),
                       "p99": round(float(np.percentile(times, 99)), 4)},
        "solve": {"iterations": st.iterations, "cg": st.num_cg, "exp": st.num_exp,
                  "prop": st.num_prop, "power_iters": st.power_iters, "active": st.active,
                  "residual": st.residual, "tol": tol, "spmv_fp64": st.spmv_fp64,
                  "spmv_fp32": st.spmv_fp32, "phases": st.phases},
        "roofline": {"bound": "hbm", "kernel": dominant,
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "read_peak": read_peak, "frac_of_read_peak": round(achieved / read_peak, 4),
                     "traffic": traffic, "bytes_per_launch": int(pass_bytes),
                     "launch_ms": round(pow_launch_ms, 5), "launches": int(passes),
                     "share_of_solve": round(power_ms / max(1e-9, solver1 - solver0), 3)
                     if power_ms > 0 else 1.0,
                     "bytes_rule": "per matrix pass: nnzb*(9*s+2) + (nv+1)*4 + 2*n*s, s = 8 (FP64) or 4 (FP32)"},
        "roofline_engine": {"kernel": "mprgp::engine_kernel (MPRGP phases)",
                            "achieved": None if eng_achieved is None else round(eng_achieved, 2),
                            "frac": None if eng_achieved is None else round(eng_achieved / peak, 4),
                            "bytes": int(eng_bytes + eng_vec), "bytes_matrix": int(eng_bytes),
                            "bytes_vectors": int(eng_vec), "ms": round(eng_ms, 3),
                            "traffic": committed_traffic(args.config, args.form, "engine_kernel"),
                            "note": "matrix passes plus the estimated vector traffic (VEC_K); "
                                    "the MPRGP phases are FP64-issue bound (ncu)"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "wall_s_timed": round(wall, 3),
    }
    if not args.no_e2e:
        line["e2e"] = run_e2e(ctx, qp, opt, args, world, mixed)
    if not args.no_ica and args.config in ("c0", "c1"):
        line["ica_comparison"] = run_ica(ctx, qp, tol, prob)
    if not args.no_e2e and rank == 0 and args.form == "plain":
        line["e2e_facade"] = run_facade_newton(qp)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, cst = cpu_baseline(qp, 1)
        line["cpu_baseline"] = {
            "value": round(1.0 / dt, 5), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"one full solve of the same QP by the CPU restatement (oracle/), "
                      f"serial like the reference; {dt:.2f} s, {int(cst['iterations'])} "
                      f"iterations, code {int(cst['code'])}"}
    prob.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def run_ica(ctx, qp, tol, prob):
    """The reference's comparison (test_case/MPRGP_ICA_Compare.cpp,
    script/data/ica_mprgp.txt): its ICA contact solver on the same QP and
    stopping scale, on the GPU (mprgp_ica_solve), from the same start x0,
    with the reference's projected Gauss-Seidel defaults (20 sweeps,
    1e-3).  Reported beside the MPRGP solve: device time, iterations and the
    distance between the two solutions."""
    x_m = prob.get_x()
    ms = []
    for _ in range(2):
        x, lam, st = ctx.ica_solve(qp, qp.x0, max_it=100000, tol=tol)
        ms.append(st.device_ms)
    return {"solver": "ICA (ICASolver.h:287-463) on the GPU, exact level-scheduled "
                      "block Gauss-Seidel + per-vertex projected Gauss-Seidel",
            "converged": bool(st.converged), "iterations": st.iterations,
            "pgs_sweeps": int(st.pgs_sweeps), "levels": st.levels,
            "device_ms": round(min(ms), 3), "residual": st.residual, "tol": tol,
            "rel_diff_to_mprgp_x": float(np.linalg.norm(x - x_m) / np.linalg.norm(x_m))}


def write_qp_file(qp, path):
    """The QP as the reference's binary (A, B, J, c, x0) file
    (MPRGPUtility.h:407-443): triplets in column-major order."""
    import mprgp_gb300 as M
    ptr, idx, val = M.bsr_to_csr(qp.nv, qp.row_ptr, qp.cols, qp.vals)
    rows = np.repeat(np.arange(qp.n, dtype=np.int32), np.diff(ptr))
    jptr, jidx, jval, c = M.planes_to_J(qp.nv, qp.plane_ptr, qp.planes)
    jrows = np.repeat(np.arange(len(c), dtype=np.int32), np.diff(jptr))
    rec = np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")])

    def sparse(f, nr, nc, r, cc, v):
        order = np.lexsort((r, cc))
        np.array([nr, nc, len(v)], "<u8").tofile(f)
        t = np.empty(len(v), rec)
        t["r"], t["c"], t["v"] = r[order], np.asarray(cc)[order], np.asarray(v)[order]
        t.tofile(f)

    with open(path, "wb") as f:
        sparse(f, qp.n, qp.n, rows, idx, val)
        np.asarray(qp.b, "<f8").tofile(f)
        sparse(f, len(c), qp.n, jrows, jidx, jval)
        np.asarray(c, "<f8").tofile(f)
        np.asarray(qp.x0, "<f8").tofile(f)


def run_facade_newton(qp, steps=4):
    """The C++ façade as the reference's FEM driver calls it: the same QP
    (from a reference-layout file) solved `steps` times through
    MPRGPGeneralCon<double>::solve with the same sparsity and new values each
    time (tests/cpp/facade_newton.cpp).  Wall time per call, host conversion
    and copies included: the first call builds the 3x3-block pattern, the
    later ones refill its values."""
    import subprocess
    import tempfile
    import mprgp_gb300 as M
    libdir = os.path.dirname(M.build())
    with tempfile.TemporaryDirectory() as tmp:
        exe, qpf = os.path.join(tmp, "facade_newton"), os.path.join(tmp, "qp.b")
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "facade_newton.cpp"), "-L", libdir,
                        "-lmprgp_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
        write_qp_file(qp, qpf)
        res = subprocess.run([exe, qpf, str(steps), str(REL_TOL)], capture_output=True,
                             text=True, timeout=600)
    kv = dict(t.split("=") for t in res.stdout.split())
    if res.returncode != 0:
        return {"error": res.stdout.strip() + res.stderr.strip()[-300:]}
    later = float(kv["later_ms"])
    return {"value": round(1e3 / later, 4), "unit": "solves/s",
            "first_call_ms": float(kv["first_ms"]), "later_call_ms": later,
            "calls": int(kv["solves"]), "pattern_builds": int(kv["pattern_builds"]),
            "pattern_refills": int(kv["pattern_refills"]),
            "path": "C++ façade MPRGPGeneralCon<double>::solve (include/mprgp/MPRGPSolver.h) "
                    "from host Eigen-like CSR: a Newton loop's re-solves with the same "
                    "sparsity (new values each call; the block pattern is kept, values "
                    "refilled), wall time per call with conversion and copies"}


def run_e2e(ctx, qp, opt, args, world, mixed):
    """Solves through mprgp_solve_bsr from pinned host memory, copies inside the timing."""
    import torch
    import mprgp_gb300 as M

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t, t.numpy()

    keep = []
    arrs = {}
    for k in ("row_ptr", "cols", "vals", "b", "x0", "plane_ptr", "planes"):
        t, a = pinned(getattr(qp, k))
        keep.append(t)
        arrs[k] = a
    hq = M.BeamQP(qp.nv, arrs["row_ptr"], arrs["cols"], arrs["vals"], arrs["b"], arrs["x0"],
                  arrs["plane_ptr"], arrs["planes"], qp.params)
    xout_t, _ = pinned(np.zeros(qp.n))
    h2d = sum(a.nbytes for a in arrs.values())
    d2h = qp.n * 8 + len(qp.planes)
    times = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        x, face, st = ctx.solve_bsr(hq, opt, hq.x0)
        dt = time.perf_counter() - t
        if st.code != 0:
            raise RuntimeError(f"e2e solve did not converge: {st.as_dict()}")
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    return {"value": round(world * args.steps / total, 4), "unit": "solves/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": round(1e3 * total / args.steps, 3),
            "path": "mprgp_solve_bsr (C ABI) from pinned host buffers",
            "gpu_launches_per_step": 3}


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    qp = workload_qp(args.config, builder=oracle_helpers().oracle_beam)
    for _ in range(args.warmup):
        cpu_baseline(qp, threads)
    times, st = [], None
    for _ in range(args.steps):
        dt, st = cpu_baseline(qp, threads)
        times.append(dt)
    total = sum(times)
    v = args.steps / total
    line = {
        "impl": "reference",
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(v, 5), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded beam QP, no dataset)",
        "config": workload_desc(args.config, qp),
        "latency_ms": {"p50": round(1e3 * float(np.percentile(times, 50)), 2),
                       "p99": round(1e3 * float(np.percentile(times, 99)), 2)},
        "cpu_baseline": {"value": round(v, 5), "unit": "solves/s", "cores": threads,
                         "kind": "port",
                         "sample": "full solves of the workload QP by the CPU restatement of "
                                   "the reference MPRGP (oracle/), OpenMP SpMV/dots on all "
                                   f"host threads; last solve {int(st['iterations'])} iterations"},
        "e2e": {"value": round(v, 5), "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_batch(args):
    """configs c2: 256 uneven beams solved in one persistent launch (mixed
    form), against the plain FP64 GPU solve of the same instances one at a time."""
    import torch
    import mprgp_gb300 as M
    from mprgp_gb300 import workloads as W
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    M.build()
    qps = W.batch()
    ctx = M.Context(local)
    tuning = autotune_ctx(args, ctx, qps[:48], M.PREC_MIXED if args.form != "plain" else M.PREC_FP64)
    probs, opts64, optsmx, x0s = [], [], [], []
    for qp in qps:
        pr = M.load_beam(ctx, qp, precisions=3)
        pr.set_power_cache(False)  # every timed solve runs its power method
        probs.append(pr)
        tol = REL_TOL * float(np.linalg.norm(qp.b))
        kind = M.KIND_PLANES
        opts64.append(M.default_options(tol=tol, max_it=20000, kind=kind, project_x0=1, seed=SEED))
        optsmx.append(M.default_options(tol=tol, max_it=20000, kind=kind, project_x0=1, seed=SEED,
                                        precision=M.PREC_MIXED if args.form != "plain" else M.PREC_FP64))
        x0s.append(torch.from_numpy(qp.x0).cuda())
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def reset():
        for pr, x0 in zip(probs, x0s):
            pr.set_x(x0.data_ptr(), on_device=True)

    def batched_step():
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        reset()
        st = ctx.solve_batch(probs, optsmx)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), st

    for _ in range(args.warmup):
        batched_step()
    times, stats = [], None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ms, stats = batched_step()
            times.append(ms)
    bad = [s.as_dict() for s in stats if s.code != 0]
    if bad:
        raise RuntimeError(f"{len(bad)} batched solves did not converge: {bad[:2]}")
    total_ms = sum(times)
    value = len(qps) * args.steps / (total_ms / 1e3)
    # plain FP64, one instance at a time, same stream of instances
    t_plain = 0.0
    plain_ms = []
    for pr, x0, o in zip(probs, x0s, opts64):
        pr.set_x(x0.data_ptr(), on_device=True)
        st = pr.solve(o)
        if st.code != 0:
            raise RuntimeError(f"plain solve did not converge: {st.as_dict()}")
        plain_ms.append(st.device_ms)
    t_plain = sum(plain_ms) / 1e3
    alg = sum(s.spmv_fp64 * spmv_bytes(q, 8) + s.spmv_fp32 * spmv_bytes(q, 4)
              for s, q in zip(stats, qps))
    dev_ms = statistics.mean(s.device_ms for s in stats)
    peak, peak_kind = measured_peaks()
    achieved = alg / (dev_ms / 1e3) / 1e9
    nvs = [q.nv for q in qps]
    line = {
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 A (f32 accumulate) + f64 steps/projection/residual" if args.form != "plain" else "f64",
        "data": "synthetic (seeded beam QPs, no dataset)",
        "config": {"workload": f"batch of {len(qps)} beams, cube counts log-uniform 4..24 x 4..24 x 4..48 "
                               f"({min(nvs)}..{max(nvs)} vertices, {3 * sum(nvs)} DOF total), floor + 0-2 walls, "
                               f"v0 ~ N(0, 0.2^2), tol 1e-8||b|| each", "config": "c2",
                   "form": "batched-" + ("mixed" if args.form != "plain" else "fp64"),
                   "l2": "flushed between batched solves (256 MB device write)",
                   "autotune": tuning},
        "plain_fp64_one_at_a_time": {"value": round(len(qps) / t_plain, 3), "unit": "solves/s",
                                     "speedup_of_value": round(value / (len(qps) / t_plain), 2)},
        "solve": {"iterations_max": max(s.iterations for s in stats),
                  "iterations_mean": round(statistics.mean(s.iterations for s in stats), 1),
                  "phases": max(s.phases for s in stats)},
        "roofline": {"bound": "hbm", "kernel": "mprgp::engine_kernel", "achieved": round(achieved, 2),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": None, "bytes_per_launch": alg,
                     "launch_ms": round(dev_ms, 3)},
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
    }
    for pr in probs:
        pr.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line))


C3_PLANES = np.array([[0.0, 1.0, 0.0, 0.0],    # floor y >= 0
                      [1.0, 0.0, 0.0, 0.0],    # wall x >= 0
                      [0.0, 0.0, 1.0, 0.0]])   # wall z >= 0
C3_DELTA = 0.025                               # contact distance of the plane query


def run_timesteps(args):
    """configs c3: one 48x48x144 stiff beam (E=1e6, nu=0.49) advanced W + K
    implicit-Euler timesteps with every part of the step on the GPU: A = M +
    h^2 K assembled once from the tetrahedra (mprgp_fem), then per step b
    from the current x and v (mprgp_fem_rhs), the contact planes (floor and
    two walls, up to 3 per vertex) regenerated from the previous solution by
    the proximity query (mprgp_planes_collide), and the QP solve warm-started
    from the previous x.  A step is one timestep in the chosen form; every
    timestep's solution is compared with the plain FP64 solve of the same QP
    from the same start."""
    import torch
    import mprgp_gb300 as M
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    M.build()
    a_, b_, c_, extra, mode, E, nu, sig = WORKLOADS["c3"]
    tets, X, x0, v0 = M.beam_mesh(a_, b_, c_, young=E, poisson=nu, v0_sigma=sig, seed=1)
    qp = workload_qp("c3")  # same mesh and material; its planes serve the launch-shape tuning
    params = qp.params
    h, grav = params["dt"], (0.0, params["gravity"], 0.0)
    ctx = M.Context(local)
    mixed = args.form != "plain"
    prec = M.PREC_MIXED if mixed else M.PREC_FP64
    # every timestep after the first reuses the power method (A is fixed)
    tuning = autotune_ctx(args, ctx, [qp], prec, power_cache=True)
    fem = M.FemMesh(ctx, tets, X, params["young"], params["poisson"], params["rho"])
    prob, ref = M.Problem(ctx, qp.nv), M.Problem(ctx, qp.nv)
    torch.cuda.synchronize()
    t_asm = time.perf_counter()
    fem.assemble(h, grav, x0, v0, prob=prob, precisions=3)
    assemble_ms = 1e3 * (time.perf_counter() - t_asm)
    fem.assemble(h, grav, x0, v0, prob=ref, precisions=1)
    prob.set_x(x0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush_buf = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    x_cur, v_cur = x0.copy(), v0.copy()
    records, times, stats = [], [], []
    n0 = None
    total = args.warmup + args.steps
    clk = ClockSampler(local)

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        return e

    for k in range(total):
        if k == args.warmup:
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            n0 = ctx.counters()
            clk.__enter__()
        flush_buf.fill_(1.0)
        torch.cuda.synchronize()
        proj = 1 if k == 0 else 0
        e0 = ev()
        if k > 0:
            fem.rhs(h, grav, x_cur, v_cur, prob=prob)
        e1 = ev()
        m = prob.collide_planes(C3_PLANES, C3_DELTA)  # from the problem's current x
        e2 = ev()
        b = fem.get_b()
        tol = REL_TOL * float(np.linalg.norm(b))
        opt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=proj,
                                seed=SEED, precision=prec, use_ev=1)
        e2b = ev()
        st = prob.solve(opt)
        e3 = ev()
        e3.synchronize()
        if st.code != 0:
            raise RuntimeError(f"timestep {k} did not converge: {st.as_dict()}")
        x = prob.get_x()
        face = prob.get_face()
        # the same QP (A, b, planes, start) in plain FP64
        ref.set_rhs(b)
        ptr, pl = prob.get_planes()
        ref.set_planes(ptr, pl)
        ref.set_x(x_cur)
        ropt = M.default_options(tol=tol, max_it=20000, kind=M.KIND_PLANES, project_x0=proj,
                                 seed=SEED, precision=M.PREC_FP64, use_ev=1)
        rst = ref.solve(ropt)
        xr, fr = ref.get_x(), ref.get_face()
        step_ms = e0.elapsed_time(e3)
        records.append({"step": k, "constraints": int(m), "iterations": st.iterations,
                        "fp64_iterations": rst.iterations, "fp64_code": rst.code,
                        "rel_err_x": float(np.linalg.norm(x - xr) / np.linalg.norm(xr)),
                        "active": int(st.active), "active_fp64": int(rst.active),
                        "face_mismatch": int(np.count_nonzero(face != fr)),
                        "rhs_ms": round(e0.elapsed_time(e1), 3),
                        "collide_ms": round(e1.elapsed_time(e2), 3),
                        "solve_ms": round(e2b.elapsed_time(e3), 3), "ms": round(step_ms, 3)})
        if k >= args.warmup:
            times.append(step_ms)
            stats.append(st)
        v_cur = (x - x_cur) / h
        x_cur = x
    clk.__exit__(None, None, None)
    launches = ctx.counters()[0] - n0[0]
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms / 1e3)
    alg = sum(s.spmv_fp64 * spmv_bytes(qp, 8) + s.spmv_fp32 * spmv_bytes(qp, 4) for s in stats)
    dev_ms = sum(s.device_ms for s in stats)
    peak, peak_kind = measured_peaks()
    achieved = alg / (dev_ms / 1e3) / 1e9
    desc = (f"beam {a_}x{b_}x{c_} cubes, 6 Kuhn tets each: {qp.nv} vertices, {qp.n} DOF, "
            f"{len(tets)} tets, {qp.nnzb} 3x3 blocks; E={E:g} nu={nu} rho=1000 h={h}; "
            f"{total} implicit-Euler timesteps on the GPU: A = M + h^2 K assembled once from the "
            f"tets, per step b from x and v, contact planes (floor, walls x and z, delta "
            f"{C3_DELTA}) regenerated from the previous solution, QP solve warm-started; "
            f"tol 1e-8*||b|| per step")
    line = {
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(value, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 A (f32 accumulate) + f64 steps/projection/residual" if mixed else "f64",
        "data": "synthetic (seeded beam mesh, no dataset)",
        "config": {"workload": desc, "config": "c3",
                   "form": "timesteps-" + ("mixed" if mixed else "fp64"),
                   "step": "b assembly + plane generation + solve, all timed",
                   "assemble_ms_once": round(assemble_ms, 2),
                   "power_method": "reused across timesteps while A and the seed are unchanged "
                                   "(bitwise the same alpha_bar)",
                   "l2": "flushed before every timestep (256 MB device write)",
                   "autotune": tuning},
        "latency_ms": {"p50": round(float(np.percentile(times, 50)), 3),
                       "p99": round(float(np.percentile(times, 99)), 3)},
        "per_timestep": records,
        "roofline": {"bound": "hbm",
                     "kernel": "solver kernels of the timestep (engine_kernel; the power loop "
                               "on the first step)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": None,
                     "bytes_per_launch": int(alg / max(1, launches)),
                     "launch_ms": round(dev_ms / max(1, launches), 5),
                     "bytes_rule": "per matrix pass: nnzb*(9*s+2) + (nv+1)*4 + 2*n*s, s = 8 (FP64) or 4 (FP32)"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": None,
        "cpu_baseline_note": "not run for this workload: one solve of the CPU restatement on "
                             "1.04M DOF exceeds the bounded sample (use c1 or c4)",
    }
    fem.close()
    prob.close()
    ref.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


SERVE_COUNT = 512          # requests per window (one step)
SERVE_SEED = 7
SERVE_RATE = 5000.0        # headline arrival rate, req/s (saturates the server)
SERVE_SWEEP = (100.0, 1000.0, 5000.0)
SERVE_CPU_SAMPLE = 32      # new-scene requests per reference-arm step
SERVE_LANES = 3            # server form: 0 synchronous steps, 2 or 3 asynchronous lanes


def serve_desc(win):
    nvs = [r.qp.nv for r in win.reqs if not r.followup]
    nf = sum(r.followup for r in win.reqs)
    return (f"serving stream window of {len(win.reqs)} requests, Poisson arrivals: {len(nvs)} new "
            f"beams log-uniform 4x4x4..32x32x64 cubes ({min(nvs)}..{max(nvs)} vertices, "
            f"{3 * sum(nvs)} DOF total; floor + 0-2 walls, 1-3 planes per vertex; "
            f"v0 ~ N(0, 0.2^2)) and {nf} follow-up timesteps of live scenes (warm start, "
            f"A/x/active set resident); tol 1e-8*||b|| each")


def serve_chains(win):
    """The window's requests grouped by scene: each chain is a new scene
    followed by its follow-up timesteps, in arrival order."""
    chains = {}
    for i, r in enumerate(win.reqs):
        chains.setdefault(r.scene, []).append(i)
    return [chains[s] for s in sorted(chains)]


def oracle_helpers():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers as H
    return H


def cpu_chain(win, chain, fb=None):
    """Solves one scene chain with the CPU restatement of the reference MPRGP
    the way MprgpFemSolver steps a scene: the new scene from P(x0), each
    follow-up warm-started from the previous solution (no projection) and the
    stored power-method vector (MprgpFemSolver.cpp:533 passes &power_ev).
    Follow-up right-hand sides come from `fb` (request index -> b) when given,
    else from this chain's own solutions (workloads.next_step_rhs).
    Returns {request index: (x, stats)}."""
    from mprgp_gb300 import workloads as W
    H = oracle_helpers()
    qp = win.reqs[chain[0]].qp
    A, b, J, c = H.qp_from_beam(qp)
    out = {}
    ev, x_prev, v_prev, x_new, b_cur = None, qp.x0, np.zeros_like(qp.x0), None, b
    for i in chain:
        if win.reqs[i].followup:
            if fb is not None:
                b_next = fb[i]
                v_new = (x_new - x_prev) / qp.params["dt"]
            else:
                b_next, v_new = W.next_step_rhs(qp, b_cur, x_prev, x_new, v_prev,
                                                qp.params["dt"])
            x_prev, v_prev, b_cur = x_new, v_new, b_next
            start, proj = x_new, False
        else:
            start, proj = qp.x0, True
        tol = REL_TOL * float(np.linalg.norm(b_cur))
        x, _, st, ev = H.oracle_solve_warm("general", A, b_cur, start, J, c, ev=ev, tol=tol,
                                           max_it=20000, seed=SEED, project_x0=proj)
        out[i] = (x, st)
        x_new = x
    return out


def cpu_chains(win, chains, threads, fb=None):
    """Solves scene chains concurrently, one chain per host thread (each solve
    single-threaded, as the reference's serial path), longest chains first.
    Returns (seconds, {request index: (x, stats)})."""
    from concurrent.futures import ThreadPoolExecutor
    H = oracle_helpers()
    H.oracle().oracle_set_threads(1)
    order = sorted(chains, key=lambda ch: -len(ch) * win.reqs[ch[0]].qp.nv)
    out = {}
    t = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for part in ex.map(lambda ch: cpu_chain(win, ch, fb), order):
            out.update(part)
    return time.perf_counter() - t, out


def serve_config(win):
    """The `config` both arms of the serving benchmark report (one dict, so
    the two lines describe the same workload)."""
    return {"workload": serve_desc(win), "config": "c4", "arrival_rate_hz": SERVE_RATE,
            "requests": len(win.reqs), "seed": SERVE_SEED,
            "l2": "GPU arm: flushed before every window (256 MB device write); CPU arm: the "
                  "window's QPs (about 2 GB) exceed every host cache"}


SERVE_REF_REQUESTS = 64    # requests per reference-arm step (whole scene chains)


def run_serve(args):
    """configs c4: a window of the serving stream through the continuous-
    batching server (mixed form by default), against the plain FP64 GPU solve
    one request at a time on the same stream."""
    import torch
    import mprgp_gb300 as M
    from mprgp_gb300 import workloads as W
    from mprgp_gb300.stream import StreamPlayer
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    M.build()
    # replicas: each rank serves its own window of the stream (weak scaling)
    win = W.serving_window(SERVE_COUNT, SERVE_SEED + rank)
    ctx = M.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush_buf = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.fill_(1.0)

    mixed = args.form != "plain"
    prec = M.PREC_MIXED if mixed else M.PREC_FP64
    # Serving keeps the cluster solver (one item per CTA), the power-step
    # loop and the persistent engine: measured on this stream, they give the
    # best solves/s at the lowest median latency.  The tuner's sample (one
    # batched solve) measures batch throughput alone -- without the cluster
    # solver the small requests wait for the batched runs, about doubling
    # their median latency -- so only the remaining knobs are tuned.
    tuning = autotune_ctx(args, ctx, [r.qp for r in win.reqs if not r.followup][:48], prec,
                          fixed={"cluster": 16, "cluster_items": 1, "power": "step",
                                 "power_regs": 40, "engine": "persistent"})
    pl = StreamPlayer(ctx, win, rel_tol=REL_TOL, seed=SEED)
    served = dict(max_slots=512, quantum=512, power_launches=1003, cluster_quantum=0,
                  lanes=args.lanes)
    plain = dict(max_slots=1, quantum=-1, power_launches=1003)

    def check(res, what):
        bad = [(i, c) for i, c in enumerate(res.codes) if c != 0]
        if bad:
            raise RuntimeError(f"{what}: {len(bad)} requests did not converge: {bad[:4]}")
        return res

    # warm-up 1 records the follow-up right-hand sides (host-copy submission)
    check(pl.play(SERVE_RATE, prec, mode="host", **served), "record")
    pl.stage()
    for _ in range(max(0, args.warmup - 1)):
        check(pl.play(SERVE_RATE, prec, "device", flush=flush, stream=stream, **served), "warm-up")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    timed = []
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            timed.append(check(pl.play(SERVE_RATE, prec, "device", flush=flush, stream=stream,
                                       keep_x=(k == 0), **served), "served"))
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    from mprgp_gb300 import replicas
    n_req = len(win.reqs)
    local_ms = sum(r.event_ms for r in timed)
    value = replicas.aggregate_throughput(n_req * args.steps, local_ms / 1e3)
    total_ms = replicas.max_over_ranks(local_ms)
    lat = np.concatenate([r.latency_s for r in timed]) * 1e3
    # e2e right after the device-resident plays, in the same state of the
    # device: the same window submitted by reference to pinned host buffers
    e2e_line = None
    if not args.no_e2e:
        check(pl.play(SERVE_RATE, prec, "pinned", flush=flush, stream=stream, **served), "e2e warm-up")
        e2e = [check(pl.play(SERVE_RATE, prec, "pinned", flush=flush, stream=stream, **served), "e2e")
               for _ in range(args.steps)]
        ems = sum(r.event_ms for r in e2e)
        elat = np.concatenate([r.latency_s for r in e2e]) * 1e3
        e2e_line = {"value": round(replicas.aggregate_throughput(n_req * args.steps, ems / 1e3), 3),
                    "unit": "solves/s",
                    "h2d_bytes_per_step": int(e2e[0].h2d_bytes),
                    "d2h_bytes_per_step": int(e2e[0].d2h_bytes),
                    "p50_ms": round(float(np.percentile(elat, 50)), 3),
                    "p99_ms": round(float(np.percentile(elat, 99)), 3),
                    "path": "mprgp_server_submit (C ABI) by reference to pinned host buffers, "
                            "copied at admission; x and face read back at completion"}
    # plain FP64, one request at a time, same stream and arrivals
    base, errs, same_face = None, [float("nan")], 0
    if not args.no_plain:
        base = check(pl.play(SERVE_RATE, M.PREC_FP64, "device", flush=flush, stream=stream,
                             keep_x=True, **plain), "plain FP64")
        # error of every served result against the plain FP64 GPU solve of the same QP
        errs = []
        for i in range(n_req):
            xs, xp = timed[0].xs[i], base.xs[i]
            errs.append(float(np.linalg.norm(xs - xp) / max(np.linalg.norm(xp), 1e-300)))
            same_face += int(np.array_equal(timed[0].faces[i], base.faces[i]))
    # the served form in plain FP64 (same server, same stream): separates the
    # gain of serving/batching from the gain of the mixed precision
    served64 = None
    if mixed and not args.no_plain:
        r64 = [check(pl.play(SERVE_RATE, M.PREC_FP64, "device", flush=flush, stream=stream,
                             **served), "served FP64") for _ in range(max(1, min(args.steps, 3)))]
        ms64 = sum(r.event_ms for r in r64)
        lat64 = np.concatenate([r.latency_s for r in r64]) * 1e3
        served64 = {"value": round(n_req * len(r64) / (ms64 / 1e3), 3), "unit": "solves/s",
                    "windows": len(r64),
                    "p50_ms": round(float(np.percentile(lat64, 50)), 3),
                    "p99_ms": round(float(np.percentile(lat64, 99)), 3)}
    # arrival-rate sweep (one window each)
    sweep = []
    for rate in (() if args.no_sweep else SERVE_SWEEP):
        a = check(pl.play(rate, prec, "device", flush=flush, stream=stream, **served), "sweep")
        b = check(pl.play(rate, M.PREC_FP64, "device", flush=flush, stream=stream, **plain),
                  "sweep plain")
        sweep.append({"rate_hz": rate,
                      "served": {"solves_per_s": round(a.solves_per_s, 2),
                                 "p50_ms": round(float(np.percentile(a.latency_s, 50)) * 1e3, 3),
                                 "p99_ms": round(float(np.percentile(a.latency_s, 99)) * 1e3, 3)},
                      "plain_fp64": {"solves_per_s": round(b.solves_per_s, 2),
                                     "p50_ms": round(float(np.percentile(b.latency_s, 50)) * 1e3, 3),
                                     "p99_ms": round(float(np.percentile(b.latency_s, 99)) * 1e3, 3)}})
    # roofline of the solver kernels over the timed plays
    scene = {r.scene: r.qp for r in win.reqs if not r.followup}
    alg = vec = 0
    for res in timed:
        for i, st in enumerate(res.stats):
            q = scene[win.reqs[i].scene]
            alg += st.spmv_fp64 * spmv_bytes(q, 8) + st.spmv_fp32 * spmv_bytes(q, 4)
            vec += vector_bytes(st, q, mixed)
    # device time of the solver runs; concurrent lanes overlap, so their sum
    # is capped by the windows' own device time
    solver_ms = min(sum(r.solver_ms for r in timed), local_ms)
    peak, peak_kind = measured_peaks()
    read_peak = read_stream_peak()
    achieved = (alg + vec) / (solver_ms / 1e3) / 1e9
    launches = sum(r.launches for r in timed)
    its = [st.iterations for st in timed[0].stats]
    line = {
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 A (f32 accumulate) + f64 steps/projection/residual" if mixed else "f64",
        "data": "synthetic (seeded beam QPs, no dataset)",
        "config": serve_config(win),
        "setup": {"form": "served-" + ("mixed" if mixed else "fp64"),
                  "server": {"slots": served["max_slots"], "quantum_phases": served["quantum"],
                             "power_loop_per_step": served["power_launches"],
                             "small_instances": "cluster solver, to completion within a run",
                             "lanes": {0: "one synchronous run per step",
                                       2: "two asynchronous lanes (small, large)"}.get(
                                 args.lanes, f"{args.lanes} asynchronous lanes (small, large, "
                                             f"{args.lanes - 2} for the large requests' power "
                                             f"method)")},
                  "inputs": "staged in device memory before the timed region (e2e: pinned host)",
                  "autotune": tuning,
                  "parallelism": "replicas" if world > 1 else "single GPU"},
        "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3),
                       "p99": round(float(np.percentile(lat, 99)), 3)},
        "plain_fp64_one_at_a_time": None if base is None else {
            "value": round(base.solves_per_s, 3), "unit": "solves/s",
            "p50_ms": round(float(np.percentile(base.latency_s, 50)) * 1e3, 3),
            "p99_ms": round(float(np.percentile(base.latency_s, 99)) * 1e3, 3),
            "speedup_of_value": round(value / world / base.solves_per_s, 2)},
        "served_fp64": served64,
        "error_vs_fp64": {"max_rel_x": float(max(errs)), "median_rel_x": float(np.median(errs)),
                          "identical_active_sets": same_face, "of": n_req},
        "sweep": sweep,
        "solve": {"iterations_max": int(max(its)), "iterations_mean": round(float(np.mean(its)), 1)},
        "roofline": {"bound": "hbm",
                     "kernel": "all solver kernels (cluster_kernel, the power-method loop, the "
                               "engine's MPRGP phases; no single one dominates the stream)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "read_peak": read_peak, "frac_of_read_peak": round(achieved / read_peak, 4),
                     "traffic": committed_traffic("c4", "mixed" if mixed else "plain", "window"),
                     "traffic_unit": "DRAM bytes read + written per window (ncu launch list, "
                                     "profiles/dram_traffic_c4_serving.md)",
                     "bytes_per_window": int((alg + vec) / len(timed)),
                     "bytes_per_launch": int((alg + vec) / max(1, launches)),
                     "launch_ms": round(solver_ms / max(1, launches), 5),
                     "bytes_matrix_per_step": int(alg / len(timed)),
                     "bytes_vectors_per_step": int(vec / len(timed)),
                     "achieved_matrix_only": round(alg / (solver_ms / 1e3) / 1e9, 2),
                     "bytes_rule": "per matrix pass: nnzb*(9*s+2) + (nv+1)*4 + 2*n*s, s = 8 (FP64) "
                                   "or 4 (FP32); plus k*n*8 of vector traffic per phase (VEC_K "
                                   "in bench.py) and 49 B per constraint row read"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if e2e_line is not None:
        line["e2e"] = e2e_line
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # The oracle, single-threaded, on whole scene chains of the window
        # (follow-ups with the served right-hand sides, so that both sides
        # solve the same QPs), about 15 s of host time; its solutions are
        # the served results' reference (error_vs_oracle).
        spent, solved = 0.0, {}
        chains = serve_chains(win)
        for k in np.random.default_rng(SERVE_SEED).permutation(len(chains)):
            ch = chains[k]
            dt, part = cpu_chains(win, [ch], 1, fb=pl.fb)
            spent += dt
            solved.update(part)
            if spent > 15.0:
                break
        nf = sum(win.reqs[i].followup for i in solved)
        line["cpu_baseline"] = {
            "value": round(len(solved) / spent, 4), "unit": "solves/s", "cores": 1,
            "kind": "port",
            "sample": f"whole scene chains of the window in a seeded random order: {len(solved)} "
                      f"requests "
                      f"({nf} follow-up timesteps warm-started from the previous solution and "
                      f"power vector), solved one after another by the CPU restatement of the "
                      f"reference MPRGP (oracle/), single-threaded; {spent:.1f} s"}
        line["error_vs_oracle"] = oracle_errors(win, solved, timed[0])
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def oracle_errors(win, solved, served):
    """Served x and active sets against the oracle's FP64 solutions of the same
    requests: ||x - x_oracle|| / ||x_oracle|| and DECIDE_FACE of both."""
    from mprgp_gb300 import planes_to_J
    H = oracle_helpers()
    scene_qp = {r.scene: r.qp for r in win.reqs if not r.followup}
    errs, same, kkt = [], 0, []
    for i, (xo, st) in sorted(solved.items()):
        qp = scene_qp[win.reqs[i].scene]
        jptr, jidx, jval, c = planes_to_J(qp.nv, qp.plane_ptr, qp.planes)
        J = H.Csr(jptr, jidx, jval, len(c), qp.n)
        xs = served.xs[i]
        errs.append(float(np.linalg.norm(xs - xo) / max(np.linalg.norm(xo), 1e-300)))
        same += int(np.array_equal(H.decide_face_planes(J, c, xs), H.decide_face_planes(J, c, xo)))
        kkt.append(int(st["code"]) == 0)
    return {"max_rel_x": max(errs), "median_rel_x": float(np.median(errs)),
            "identical_active_sets": same, "of": len(errs), "oracle_converged": int(sum(kkt)),
            "requests": "the cpu_baseline sample; served mixed form at 1e-8||b|| vs the oracle "
                        "(reference MPRGP restatement, FP64) at 1e-8||b||"}


    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def run_reference_serve(args):
    """Reference arm of c4: the CPU restatement of the reference MPRGP serving
    the same window on every host core.  The window's beams come from the
    oracle's generator (bitwise the library's; the GPU library is not
    loaded).  A scene chain -- a new scene and its follow-up timesteps, each
    warm-started from the previous solution and power vector, its right-hand
    side from that solution -- runs on one thread; chains run concurrently.
    Each step solves the next whole chains of the window, in rotation, until
    it holds SERVE_REF_REQUESTS requests, so that --steps K --warmup W
    covers the window in a few minutes."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    from mprgp_gb300 import workloads as W
    H = oracle_helpers()
    win = W.serving_window(SERVE_COUNT, SERVE_SEED, builder=H.oracle_beam)
    chains = serve_chains(win)
    threads = os.cpu_count() or 1
    cursor = 0

    def next_sample():
        nonlocal cursor
        out, n = [], 0
        while n < SERVE_REF_REQUESTS:
            ch = chains[cursor % len(chains)]
            cursor += 1
            out.append(ch)
            n += len(ch)
        return out

    for _ in range(args.warmup):
        cpu_chains(win, next_sample(), threads)
    times, counts, conv, nfol = [], [], 0, 0
    for _ in range(args.steps):
        sample = next_sample()
        dt, out = cpu_chains(win, sample, threads)
        times.append(dt)
        counts.append(len(out))
        conv += sum(int(st["code"]) == 0 for _, st in out.values())
        nfol += sum(win.reqs[i].followup for i in out)
    total = sum(times)
    v = sum(counts) / total
    line = {
        "impl": "reference",
        "metric": "QP solves/s + p50/p99 latency at ||g_P||<=1e-8||b||: served vs plain FP64, 1 GB300",
        "value": round(v, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded beam QPs, no dataset)",
        "config": serve_config(win),
        "cpu_baseline": {"value": round(v, 4), "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"each step: the next whole scene chains of the same window "
                                   f"in rotation ({sum(counts)} requests over {args.steps} steps, "
                                   f"{nfol} of them follow-up timesteps warm-started from the "
                                   f"previous solution and power vector), chains concurrently on "
                                   f"{threads} host threads, each solve single-threaded, by the "
                                   f"CPU restatement of the reference MPRGP (oracle/)"},
        "e2e": {"value": round(v, 4), "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "solve": {"converged": conv, "of": sum(counts)},
    }
    print(json.dumps(line))


FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (non-tensor) nominal rate


def run_spmv(args):
    """The standalone y = A x of the config's beam (FixedSparseMatrix::multiply
    through mprgp_problem_spmv), one launch per step, L2 flushed before each;
    x and y FP64 at the API, A in FP64 and in FP32.  Reports HBM throughput on
    the algorithmic bytes and, for the FP64 matrix, the FP64 rate on the
    algorithmic flops (18 per 3x3 block): the FP64 product is bound by GB300's
    FP64 unit before HBM."""
    import torch
    import mprgp_gb300 as M
    M.build()
    name = args.config if args.config in ("c0", "c1", "c3") else "c1"
    qp = workload_qp(name)
    ctx = M.Context(0)
    pr = M.load_beam(ctx, qp, precisions=3)
    stream = torch.cuda.ExternalStream(ctx.stream)
    x = torch.from_numpy(np.random.default_rng(0).standard_normal(qp.n)).cuda()
    y = torch.empty_like(x)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peak, peak_src = measured_peaks()
    out = {}
    with ClockSampler(0) as clk:
        for prec, s_a, key in ((M.PREC_FP64, 8, "fp64"), (M.PREC_MIXED, 4, "fp32")):
            for _ in range(args.warmup):
                pr.spmv(x.data_ptr(), y.data_ptr(), prec)
            ctx.sync()
            ts = []
            for _ in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                pr.spmv(x.data_ptr(), y.data_ptr(), prec)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = float(np.median(ts))
            # x and y are FP64 at the API whatever the matrix precision
            byt = qp.nnzb * (9 * s_a + 4) + (qp.nv + 1) * 4 + 2 * qp.n * 8
            out[key] = {"ms": round(ms, 5), "GB/s": round(byt / ms / 1e6, 1),
                        "hbm_frac": round(byt / ms / 1e6 / peak, 4), "bytes": int(byt)}
            if s_a == 8:
                tf = 18.0 * qp.nnzb / ms / 1e9
                out[key]["fp64_tflops"] = round(tf, 4)
                out[key]["fp64_frac_of_nominal"] = round(tf / FP64_NOMINAL_TFLOPS, 4)
    pr.close()
    line = {"metric": "standalone y = A x throughput (FixedSparseMatrix::multiply, FP64 x and y)",
            "value": out["fp64"]["GB/s"], "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["fp64"]["ms"], "higher_is_better": True,
            "scaling": "none", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(name, qp)["workload"], "config": name,
                       "l2": "flushed before each launch (256 MB device write)"},
            "spmv": out,
            "roofline": {"bound": "fp64", "achieved": out["fp64"]["fp64_tflops"],
                         "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                         "frac": out["fp64"]["fp64_frac_of_nominal"],
                         "peak_source": "nominal (GB300 FP64 1.25 TFLOP/s)",
                         "hbm_frac": out["fp64"]["hbm_frac"], "hbm_peak_gbs": peak,
                         "hbm_peak_source": peak_src},
            "gpu_launches": 2 * args.steps, "clocks": clk.summary()}
    print(json.dumps(line))


def main():
    args = parse()
    if args.spmv:
        run_spmv(args)
        return
    if args.form is None:
        args.form = "mixed" if args.config in ("c2", "c3", "c4") else "plain"
    if args.impl == "reference":
        if args.config == "c4":
            run_reference_serve(args)
        else:
            run_reference(args)
    elif args.config == "c2":
        run_batch(args)
    elif args.config == "c4":
        run_serve(args)
    elif args.config == "c3" and not args.single:
        run_timesteps(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
