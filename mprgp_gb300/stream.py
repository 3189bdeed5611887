"""Plays a window of the serving stream through an mprgp_server.

The client side of the serving form: requests are submitted when their
(Poisson) arrival time has passed; a follow-up timestep of a scene is held
until that scene's previous request has completed (its right-hand side
depends on the previous solution), then submitted by reference to the
resident scene.  Latency is completion (as the client sees it) minus arrival.

Input modes of a play:
  "host"    arrays copied by the server at submit (mode 0); records the
            follow-up right-hand sides for later plays;
  "device"  every array staged in device memory beforehand (mode 1);
  "pinned"  every array in pinned host memory, copied at admission (mode 2).
A recorded play fixes each follow-up's b (from the served solutions), so later
plays -- any rate, any form -- solve exactly the same sequence of QPs.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import (KIND_PLANES, PREC_FP64, Server, default_options)
from . import workloads as W


@dataclass
class PlayResult:
    rate_hz: float
    wall_s: float
    event_ms: float
    latency_s: np.ndarray
    codes: list
    stats: list
    xs: dict = field(default_factory=dict)
    faces: dict = field(default_factory=dict)
    launches: int = 0
    solver_ms: float = 0.0
    h2d_bytes: int = 0
    d2h_bytes: int = 0

    @property
    def solves_per_s(self) -> float:
        return len(self.latency_s) / (self.event_ms / 1e3)


class StreamPlayer:
    def __init__(self, ctx, window: W.Window, rel_tol=1e-8, max_it=20000, seed=0x5EED,
                 use_ev=1):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.win = window
        self.rel_tol = rel_tol
        self.max_it = max_it
        self.seed = seed
        self.use_ev = use_ev
        self.scene_qp = {}
        for r in window.reqs:
            if not r.followup:
                self.scene_qp[r.scene] = r.qp
        self.fb = {}  # request index -> follow-up b (host), set by a recorded play
        self.dev = {}
        self.pin = {}

    # ------------------------------------------------------------ staging --
    def _arrays(self, i):
        r = self.win.reqs[i]
        if r.followup:
            return {"b": self.fb[i]}
        q = r.qp
        return {"row_ptr": q.row_ptr, "cols": q.cols, "vals": q.vals, "b": q.b,
                "plane_ptr": q.plane_ptr, "planes": q.planes, "x0": q.x0}

    def stage(self):
        """Device and pinned copies of every request's arrays (after record)."""
        torch = self.torch
        for i in range(len(self.win.reqs)):
            a = self._arrays(i)
            self.pin[i] = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory()
                           for k, v in a.items()}
            self.dev[i] = {k: v.cuda() for k, v in self.pin[i].items()}
        torch.cuda.synchronize()

    def input_bytes(self, i) -> int:
        return int(sum(np.asarray(v).nbytes for v in self._arrays(i).values()))

    # -------------------------------------------------------------- play --
    def options(self, i, precision):
        r = self.win.reqs[i]
        b = self.fb[i] if r.followup else r.qp.b
        return default_options(tol=self.rel_tol * float(np.linalg.norm(b)), max_it=self.max_it,
                               kind=KIND_PLANES, project_x0=0 if r.followup else 1,
                               seed=self.seed, precision=precision, use_ev=self.use_ev)

    def play(self, rate_hz: float, precision=PREC_FP64, mode="device", max_slots=128,
             quantum=256, power_launches=256, cluster_quantum=0, lanes=0, keep_x=False,
             stream=None, flush=None) -> PlayResult:
        torch = self.torch
        reqs = self.win.reqs
        arrive = self.win.arrivals(rate_hz)
        record = mode == "host"
        if not record and len(self.fb) != sum(r.followup for r in reqs):
            raise RuntimeError("play in host mode first to record the follow-up right-hand sides")
        srv = Server(self.ctx, max_slots=max_slots, quantum_phases=quantum,
                     power_launches=power_launches, cluster_quantum=cluster_quantum, lanes=lanes)
        # client-side scene state of the recording play (next_step_rhs)
        phys = {}
        pending = deque(range(len(reqs)))
        held = {}             # scene -> deque of follow-up request indices
        busy = set()          # scenes with a request in flight
        ticket_of = {}
        lat = np.zeros(len(reqs))
        codes, stats = [None] * len(reqs), [None] * len(reqs)
        xs, faces = {}, {}
        h2d = d2h = 0
        done = 0
        if flush is not None:
            flush()
        torch.cuda.synchronize()
        n0, ms0, _ = self.ctx.counters()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t0 = time.perf_counter()

        def submit(i):
            nonlocal h2d
            r = reqs[i]
            q = self.scene_qp[r.scene]
            if record and r.followup:
                st = phys[r.scene]
                b, v = W.next_step_rhs(q, st["b"], st["x"], st["x_new"], st["v"], q.params["dt"])
                phys[r.scene] = {"b": b, "x": st["x_new"], "v": v, "x_new": None}
                self.fb[i] = b
            opt = self.options(i, precision)
            if record:
                if r.followup:
                    t = srv.submit(r.scene, q, opt, b=self.fb[i], followup=True)
                else:
                    phys[r.scene] = {"b": q.b, "x": q.x0, "v": np.zeros_like(q.x0), "x_new": None}
                    t = srv.submit(r.scene, q, opt)
            else:
                src = self.dev[i] if mode == "device" else self.pin[i]
                ptr = {k: v.data_ptr() for k, v in src.items()}
                if r.followup:
                    t = srv.submit_ref(r.scene, q.nv, 0, len(q.planes), opt, ptr["b"],
                                       on_device=mode == "device")
                else:
                    t = srv.submit_ref(r.scene, q.nv, q.nnzb, len(q.planes), opt, ptr["b"],
                                       ptr["row_ptr"], ptr["cols"], ptr["vals"], ptr["plane_ptr"],
                                       ptr["planes"], ptr["x0"], on_device=mode == "device")
            if mode != "device":
                h2d += self.input_bytes(i)
            ticket_of[t] = i
            busy.add(r.scene)

        while done < len(reqs):
            now = time.perf_counter() - t0
            while pending and arrive[pending[0]] <= now:
                i = pending.popleft()
                sc = reqs[i].scene
                if reqs[i].followup and (sc in busy or held.get(sc)):
                    held.setdefault(sc, deque()).append(i)
                else:
                    submit(i)
            if ticket_of:
                srv.step()
                tnow = time.perf_counter() - t0
                for t in srv.poll():
                    i = ticket_of.pop(t)
                    state, x, face, st, _ = srv.result(t)
                    lat[i] = tnow - arrive[i]
                    codes[i] = st.code
                    stats[i] = st
                    d2h += x.nbytes + face.nbytes
                    sc = reqs[i].scene
                    busy.discard(sc)
                    if record:
                        phys[sc]["x_new"] = x
                    if keep_x:
                        xs[i], faces[i] = x, face
                    done += 1
                    if held.get(sc):
                        submit(held[sc].popleft())
            elif pending:
                wait = arrive[pending[0]] - (time.perf_counter() - t0)
                if wait > 2e-4:
                    time.sleep(wait - 1e-4)
        e1.record(stream)
        e1.synchronize()
        wall = time.perf_counter() - t0
        n1, ms1, _ = self.ctx.counters()
        srv.close()
        return PlayResult(rate_hz, wall, e0.elapsed_time(e1), lat, codes, stats, xs, faces,
                          n1 - n0, ms1 - ms0, h2d, d2h)
