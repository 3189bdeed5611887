"""Seeded synthetic QP streams of the measured configurations.

  batch(count=256)  uneven beams in one launch: cube counts a, b log-uniform
                    in [4, 24], c log-uniform in [4, 48]; floor plus 0-2 walls
                    (up to 3 planes per vertex); v0 ~ N(0, 0.2^2).
  serving_stream()  Poisson arrivals of beams log-uniform from 4x4x4 to
                    32x32x64 with 1-3 planes per vertex, 30 % of them
                    follow-up timesteps of a live scene (warm start);
  serving_window()  the same stream cut to a fixed number of requests.
Every instance is solved to ||g_P|| <= 1e-8 ||b||.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import beam, BeamQP


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def batch_dims(count=256, seed=2026, lo=(4, 4, 4), hi=(24, 24, 48)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        dims = tuple(log_uniform_int(rng, l, h) for l, h in zip(lo, hi))
        extra = int(rng.integers(0, 3))
        out.append((dims, extra, int(rng.integers(1, 2**31))))
    return out


def batch(count=256, seed=2026, v0_sigma=0.2):
    """The instances of the batched configuration, as BeamQPs."""
    return [beam(*dims, extra_planes_max=e, extra_planes_min=e, plane_mode=2,
                 v0_sigma=v0_sigma, seed=s)
            for dims, e, s in batch_dims(count, seed)]


def lumped_mass(qp: BeamQP) -> np.ndarray:
    """Per-vertex mass from A = M + h^2 K: K annihilates rigid translations, so
    the x-row sums of A's (0,0) block entries give M."""
    rows = np.repeat(np.arange(qp.nv), np.diff(qp.row_ptr))
    m = np.zeros(qp.nv)
    np.add.at(m, rows, np.asarray(qp.vals).reshape(-1, 9)[:, 0])
    return m


def next_step_rhs(qp: BeamQP, b_prev: np.ndarray, x_prev: np.ndarray, x_new: np.ndarray,
                  v_prev: np.ndarray, dt: float):
    """Right-hand side of the next implicit-Euler step after x_new was solved
    from (x_prev, v_prev): b' = b + M (x' + h v' - x - h v), v' = (x' - x)/h."""
    m = np.repeat(lumped_mass(qp), 3)
    v_new = (x_new - x_prev) / dt
    return b_prev + m * ((x_new + dt * v_new) - (x_prev + dt * v_prev)), v_new


@dataclass
class Request:
    t_arrive: float
    qp: BeamQP | None       # new scene (None for a follow-up)
    scene: int              # scene id (follow-ups refer to a live scene)
    followup: bool = False
    extra: dict = field(default_factory=dict)


@dataclass
class Window:
    """A fixed window of the serving stream: requests in arrival order and
    their arrival times at unit rate (divide by the rate for seconds)."""
    reqs: list
    t_unit: np.ndarray

    def arrivals(self, rate_hz: float) -> np.ndarray:
        return self.t_unit / rate_hz


def serving_window(count=128, seed=7, followup_frac=0.3, lo=(4, 4, 4), hi=(32, 32, 64),
                   v0_sigma=0.2, builder=None) -> Window:
    """`count` requests of the serving stream with Poisson arrival gaps: beams
    log-uniform from lo to hi cubes, floor plus 0-2 walls (1-3 planes per
    vertex), 30 % follow-up timesteps of an earlier scene of the window.
    `builder(a, b, c, **kw)` makes each beam (default: the library's
    generator, mprgp_beam_build)."""
    build = beam if builder is None else builder
    rng = np.random.default_rng(seed)
    t, reqs, times, scenes = 0.0, [], [], 0
    while len(reqs) < count:
        t += rng.exponential(1.0)
        times.append(t)
        if scenes > 0 and rng.uniform() < followup_frac:
            reqs.append(Request(t, None, int(rng.integers(0, scenes)), followup=True))
            continue
        dims = tuple(log_uniform_int(rng, l, h) for l, h in zip(lo, hi))
        extra = int(rng.integers(0, 3))
        qp = build(*dims, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2,
                   v0_sigma=v0_sigma, seed=int(rng.integers(1, 2**31)))
        reqs.append(Request(t, qp, scenes, extra={"dims": dims, "walls": extra}))
        scenes += 1
    return Window(reqs, np.asarray(times))


def serving_stream(rate_hz: float, duration_s: float, seed=7, followup_frac=0.3,
                   lo=(4, 4, 4), hi=(32, 32, 64), v0_sigma=0.2, max_live=64):
    """Seeded Poisson arrivals; follow-ups pick a random earlier scene."""
    rng = np.random.default_rng(seed)
    t, reqs, scenes = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > duration_s:
            break
        if scenes > 0 and rng.uniform() < followup_frac:
            reqs.append(Request(t, None, int(rng.integers(max(0, scenes - max_live), scenes)),
                                followup=True))
            continue
        dims = tuple(log_uniform_int(rng, l, h) for l, h in zip(lo, hi))
        extra = int(rng.integers(0, 3))
        qp = beam(*dims, extra_planes_max=extra, extra_planes_min=extra, plane_mode=2,
                  v0_sigma=v0_sigma, seed=int(rng.integers(1, 2**31)))
        reqs.append(Request(t, qp, scenes))
        scenes += 1
    return reqs
