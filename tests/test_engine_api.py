"""Host-side surface of the engine (no GPU): the methods the driver, the
server and the bench call exist, and analytic biases map onto zg_bias the way
the Python callbacks evaluate them."""
import math

import pytest

from zandpack_gb300 import _lib
from zandpack_gb300.engine import Propagator, Trajectory, native_bias
from zandpack_gb300.workloads import bias_value


def test_trajectory_methods():
    for m in ("set_slot", "get_slot", "set_y", "get_y", "stage_input", "stage_sigma", "set_dH", "rhs",
              "error_norm2", "step_fourth", "attempt_native", "get_sigma", "set_tableau", "close"):
        assert callable(getattr(Trajectory, m)), m
    for m in ("attempt", "run", "set_state"):
        assert callable(getattr(Propagator, m)), m


@pytest.mark.parametrize("spec", [
    {"kind": "exp_ramp", "V0": 0.5, "tau": 5.0},
    {"kind": "gauss", "V0": 0.3, "tc": 20.0, "sigma": 5.0},
    {"kind": "sin", "V0": 0.2, "f": 0.05},
    {"kind": "step_lead0", "V0": 0.4},
    {"kind": "zero"}])
def test_native_bias_matches_python(spec):
    b = native_bias(spec, 3)
    for t in (0.0, 0.7, 13.0, 21.5):
        for a in range(3):
            V = 0.0
            if b.kind == _lib.ZG_BIAS["exp_ramp"]:
                V = b.V0 * (1 - math.exp(-t / b.tau))
            elif b.kind == _lib.ZG_BIAS["gauss"]:
                V = b.V0 * math.exp(-(t - b.tc) ** 2 / (2 * b.sigma ** 2))
            elif b.kind == _lib.ZG_BIAS["sin"]:
                V = b.V0 * math.sin(2 * math.pi * b.f * t)
            elif b.kind == _lib.ZG_BIAS["step"]:
                V = b.V0 if t > 0 else 0.0
            assert abs(b.w[a] * V - bias_value(spec, t, a)) < 1e-15
