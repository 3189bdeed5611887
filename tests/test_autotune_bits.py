"""Host logic of the autotuner (no GPU): the launch-form bits each setting
maps to (mprgp_context_set_tuning, include/mprgp_gpu.h), the cluster-size
fallback, and the knobs a caller pins."""
import numpy as np
import pytest

from mprgp_gb300 import autotune


class FakeCtx:
    """Records the calls autotune.apply makes; rejects cluster sizes above
    `max_cluster` as a device without them would."""

    def __init__(self, max_cluster=16):
        self.max_cluster = max_cluster
        self.calls = []

    def set_cluster(self, c):
        if c > self.max_cluster:
            raise RuntimeError("cluster size not offered")
        self.calls.append(("cluster", c))

    def set_cluster_items(self, n):
        self.calls.append(("items", n))

    def set_tuning(self, bits, ctas_per_sm):
        self.calls.append(("tuning", bits, ctas_per_sm))


def bits_of(cfg, **kw):
    ctx = FakeCtx(**kw)
    autotune.apply(ctx, dict(autotune.DEFAULT, **cfg))
    return [c for c in ctx.calls if c[0] == "tuning"][0][1], ctx.calls


@pytest.mark.parametrize("power,bits", [
    ("step", 0),            # the power-step loop: the default
    ("step-stream", 4),     # ... as host-stream launches
    ("graph", 64),          # the phase kernel with a finalize per launch
    ("stream", 64 | 4),
    ("engine", 2),          # power phases inside the persistent engine
    ("persistent", 32),     # one cooperative launch where it applies
])
def test_power_forms_map_to_bits(power, bits):
    assert bits_of({"power": power})[0] == bits


def test_other_knobs():
    assert bits_of({"power": "graph", "power_regs": 64})[0] == 64 | 8
    assert bits_of({"engine": "graph"})[0] == 16
    assert bits_of({"stage": 1})[0] == 1
    b, calls = bits_of({"ctas_per_sm": 3, "cluster_items": 2})
    assert ("tuning", 0, 3) in calls and ("items", 2) in calls


def test_default_is_the_power_step_loop_with_every_knob_at_zero_bits():
    assert autotune.DEFAULT["power"] == "step"
    assert bits_of({})[0] == 0


def test_cluster_falls_back_to_offered_sizes():
    _, calls = bits_of({"cluster": 16}, max_cluster=4)
    assert ("cluster", 4) in calls and ("cluster", 16) not in calls


class FakeProblem:
    def __init__(self):
        self.cache = None

    def set_power_cache(self, on):
        self.cache = on

    def close(self):
        pass


class FakeQP:
    nv = 4000
    b = np.ones(12)
    x0 = np.zeros(12)


def _tune_with_fake_times(monkeypatch, cost, **kw):
    """tune() over a fake context whose timed solves cost cost(cluster, bits)."""
    ctx = FakeCtx()
    ctx.info = lambda: (152, 4)
    timed = []

    def fake_time(c, probs, opts, x0s, reps):
        cl = [k[1] for k in c.calls if k[0] == "cluster"][-1]
        bits = [k[1] for k in c.calls if k[0] == "tuning"][-1]
        timed.append((cl, bits, reps))
        return cost(cl, bits), [np.zeros(3) for _ in probs]

    monkeypatch.setattr(autotune, "load_beam", lambda c, q, precisions=3: FakeProblem())
    monkeypatch.setattr(autotune, "_time", fake_time)
    r = autotune.tune(ctx, [FakeQP(), FakeQP()], use_cache=False, **kw)
    return r, ctx, timed


def test_tuner_keeps_pinned_knobs_and_takes_clear_wins(monkeypatch):
    # the graph-loop engine (bit 16) is 10 % faster, cluster 8 would be too
    cost = lambda cl, bits: 100.0 * (0.9 if bits & 16 else 1.0) * (0.9 if cl == 8 else 1.0)
    r, ctx, timed = _tune_with_fake_times(monkeypatch, cost, fixed={"cluster": 16})
    assert r["config"]["cluster"] == 16 and r["config"]["engine"] == "graph"
    assert {cl for cl, _, _ in timed} == {16}  # the pinned knob was never searched
    # a 1 % difference is not a clear win: the incumbent stays
    cost2 = lambda cl, bits: 100.0 * (0.99 if bits & 16 else 1.0)
    r2, _, _ = _tune_with_fake_times(monkeypatch, cost2)
    assert r2["config"]["engine"] == autotune.DEFAULT["engine"]


def test_tuner_power_cache_runs_one_untimed_solve_first(monkeypatch):
    r, ctx, timed = _tune_with_fake_times(monkeypatch, lambda cl, bits: 100.0, power_cache=True,
                                          reps=2)
    assert timed[0][2] == 1 and all(t[2] == 2 for t in timed[1:])


def test_bench_names_the_power_loop_of_a_tuning():
    """bench.py labels the c1 roofline by the power-method loop a tuning
    selects (autotuner config or explicit bits)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.power_form(None) == "step"
    assert bench.power_form({"config": dict(autotune.DEFAULT)}) == "step"
    assert bench.power_form({"config": dict(autotune.DEFAULT, power="stream")}) == "graph"
    assert bench.power_form({"explicit_tuning_bits": 0}) == "step"
    assert bench.power_form({"explicit_tuning_bits": 64 | 4}) == "graph"
    assert bench.power_form({"explicit_tuning_bits": 32}) == "persistent"
    assert bench.power_form({"explicit_tuning_bits": 2}) == "engine"
