"""Host logic of the autotuner (no GPU): the launch-form bits each setting
maps to (mprgp_context_set_tuning, include/mprgp_gpu.h), the cluster-size
fallback, and the knobs a caller pins."""
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
