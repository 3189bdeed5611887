"""Autotuner of the solver's launch shapes.

The knobs change how the work is laid onto the GPU, never what is computed:
every setting gives bitwise the same solutions (the per-item and
per-instance reductions run in a fixed order whatever the launch shape), and
the tuner checks that for the setting it picks.

  cluster      largest cluster of the small-instance solver (CTAs of 256
               vertex rows; instances up to that many items take it)
  cluster_items  items per CTA allowed in the largest cluster (larger
               instances then also run as independent clusters)
  power        the power method's loop: the power-step loop (each launch
               advances the states the previous one left while its rows form
               their products; CUDA-graph WHILE loop or plain stream
               launches; the default), the phase kernel whose last CTA
               finalizes each launch (graph or stream), phases of the
               persistent engine, or one persistent cooperative launch of its
               own (grid barrier per phase; synchronous runs whose items fit,
               else the power-step graph loop)
  power_regs   the phase kernel's register budget: 40 (6 CTAs per SM) or
               64 (4 CTAs per SM, more loads in flight per thread)
  engine       the large instances' MPRGP phases: the persistent cooperative
               engine, or a CUDA-graph loop of one launch per phase
  ctas_per_sm  resident CTAs per SM of the persistent engine (0 = all)
  stage        FP32 matrix slices staged in shared memory by bulk copies

The tuner times batched solves of a sample of the workload (device time of
the solver runs, best of `reps`), walks the knobs one at a time from the
default (coordinate descent; the power form and register budget together),
and caches the winner per device and workload signature (JSON;
MPRGP_TUNING_CACHE overrides the path).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import KIND_PLANES, PREC_MIXED, Context, default_options, load_beam

DEFAULT = {"cluster": 16, "cluster_items": 1, "power": "step", "power_regs": 40,
           "engine": "persistent", "ctas_per_sm": 0, "stage": 0}
SPACE = {
    "cluster": [16, 8, 4, 0],
    "cluster_items": [1, 2, 4],
    "power": ["step", "step-stream", "graph", "stream", "engine", "persistent"],
    "power_regs": [40, 64],
    "engine": ["persistent", "graph"],
    "ctas_per_sm": [0, 3, 2],
    "stage": [0, 1],
}
_POWER_BITS = {"step": 0, "step-stream": 4, "graph": 64, "stream": 64 | 4, "engine": 2,
               "persistent": 32}


def cache_path() -> str:
    return os.environ.get("MPRGP_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mprgp_gb300",
                                       "tuning.json"))


def apply(ctx: Context, cfg: dict) -> None:
    """Sets a tuning on a context (falls back to a smaller cluster size when
    the device does not offer the requested one)."""
    cl = cfg["cluster"]
    while True:
        try:
            ctx.set_cluster(cl)
            break
        except Exception:
            if cl == 0:
                raise
            cl //= 2
            cl = cl if cl >= 2 else 0
    ctx.set_cluster_items(cfg.get("cluster_items", 1))
    bits = _POWER_BITS[cfg["power"]] | (1 if cfg["stage"] else 0)
    bits |= 8 if cfg.get("power_regs", 40) == 64 else 0
    bits |= 16 if cfg.get("engine", "persistent") == "graph" else 0
    ctx.set_tuning(bits, cfg["ctas_per_sm"])


def signature(ctx: Context, qps, precision) -> str:
    nsm, bps = ctx.info()
    items = [math.ceil(q.nv / 256) for q in qps]
    hist = np.bincount([min(12, int(math.log2(max(1, i)))) for i in items], minlength=13)
    return f"sm{nsm}-bps{bps}-p{precision}-n{len(qps)}-h" + ".".join(str(int(h)) for h in hist)


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time(ctx, probs, opts, x0s, reps):
    best, xs = None, None
    for _ in range(reps):
        for pr, x0 in zip(probs, x0s):
            pr.set_x(x0)
        st = ctx.solve_batch(probs, opts)
        if any(s.code != 0 for s in st):
            raise RuntimeError("autotune: a sample solve did not converge")
        ms = st[0].device_ms
        best = ms if best is None else min(best, ms)
    xs = [pr.get_x() for pr in probs]
    return best, xs


def tune(ctx: Context, qps, precision=PREC_MIXED, reps=2, rel_tol=1e-8, seed=0x5EED,
         use_cache=True, verbose=False, power_cache=False, fixed=None) -> dict:
    """Picks and applies the fastest launch shapes for batched solves of
    `qps`; returns {"config", "ms", "default_ms", "tried", "seconds", "cached"}.
    `fixed` pins knobs to given values (they are not searched).
    power_cache=True tunes the solves that follow a first one on the same
    matrices (a timestep loop): the power method's result is reused, so the
    timed solves are the MPRGP phases alone."""
    t0 = time.perf_counter()
    fixed = dict(fixed or {})
    sig = signature(ctx, qps, precision) + ("-pc" if power_cache else "") + \
        "".join(f"-{k}{v}" for k, v in sorted(fixed.items()))
    path = cache_path()
    if use_cache:
        hit = _load(path).get(sig)
        if hit:
            apply(ctx, hit["config"])
            return dict(hit, cached=True, seconds=time.perf_counter() - t0)
    probs, opts, x0s = [], [], []
    for q in qps:
        pr = load_beam(ctx, q, precisions=3)
        pr.set_power_cache(power_cache)  # off: every timed solve runs its power method
        probs.append(pr)
        opts.append(default_options(tol=rel_tol * float(np.linalg.norm(q.b)), max_it=20000,
                                    kind=KIND_PLANES, project_x0=1, seed=seed,
                                    precision=precision))
        x0s.append(q.x0)
    tried = {}
    try:
        def run(cfg):
            key = json.dumps(cfg, sort_keys=True)
            if key not in tried:
                apply(ctx, cfg)
                tried[key] = _time(ctx, probs, opts, x0s, reps)
                if verbose:
                    print(f"autotune {cfg} {tried[key][0]:.3f} ms", flush=True)
            return tried[key]

        best = dict(DEFAULT, **fixed)
        if power_cache:  # an untimed first solve computes the power method once
            apply(ctx, best)
            _time(ctx, probs, opts, x0s, 1)
        best_ms, ref_x = run(best)
        default_ms = best_ms
        # coordinate descent; the power form and the power kernel's register
        # budget interact, so they are searched together
        steps = [[{"cluster": v} for v in SPACE["cluster"]],
                 [{"cluster_items": v} for v in SPACE["cluster_items"]],
                 [{"power": f, "power_regs": r} for f in SPACE["power"]
                  for r in (SPACE["power_regs"] if f in ("graph", "stream") else [40])],
                 [{"engine": v} for v in SPACE["engine"]],
                 [{"ctas_per_sm": v} for v in SPACE["ctas_per_sm"]],
                 [{"stage": v} for v in SPACE["stage"]]]
        steps = [st for st in steps if not any(k in fixed for k in st[0])]
        for step in steps:
            for change in step:
                cand = dict(best, **change)
                try:
                    ms, _ = run(cand)
                except Exception:  # a shape the device does not offer
                    continue
                if ms < best_ms * 0.98:  # keep the incumbent unless clearly faster
                    best, best_ms = cand, ms
        # every knob keeps the results bitwise: check the pick
        _, xs = run(best)
        for a, b in zip(xs, ref_x):
            if not np.array_equal(a, b):
                raise RuntimeError("autotune: launch shape changed a solution")
        apply(ctx, best)
    finally:
        for pr in probs:
            pr.close()
    out = {"config": best, "ms": best_ms, "default_ms": default_ms,
           "tried": {k: round(v[0], 4) for k, v in tried.items()}}
    if use_cache:
        db = _load(path)
        db[sig] = out
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(db, f, indent=1)
    return dict(out, cached=False, seconds=time.perf_counter() - t0)
