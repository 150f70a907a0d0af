"""Extrapolation weights of the pressure initial guess against the reference's unit tests
(tests/time_integration/extrapolation_constants_0{1,2}: orders 1-4, every start-up order, constant
and adaptive time steps {0.1, 0.2, 0.3, 0.4, 0.5}) and the constant-step values."""
import json
import os

import pytest

from exadg_gb300.learned_guess import extrapolation_constants

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "extrapolation_constants.json")))


def _transcript(time_steps):
    # the reference test prints, per order and start-up order, the sum of the `order` weights
    lines = []
    for order in (1, 2, 3, 4):
        lines.append("ExtrapolationConstants of oder %d" % order)
        for cur in range(1, order + 1):
            lines.append("Current order %d" % cur)
            s = sum(extrapolation_constants(order, time_steps, cur))
            lines.append("Sum: %.6g" % s)
    return lines


def test_constant_steps_golden():
    assert _transcript(None) == GOLD["extrapolation_constants_01"]


def test_adaptive_steps_golden():
    assert _transcript([0.1, 0.2, 0.3, 0.4, 0.5]) == GOLD["extrapolation_constants_02"]


@pytest.mark.parametrize("order,beta", [(1, [1.0]), (2, [2.0, -1.0]), (3, [3.0, -3.0, 1.0]), (4, [4.0, -6.0, 4.0, -1.0])])
def test_constant_step_values(order, beta):
    assert extrapolation_constants(order) == pytest.approx(beta, abs=1e-13)


def test_adaptive_steps_reproduce_polynomials():
    # order-q extrapolation is exact for polynomials of degree < q on any step sequence
    dts = [0.3, 0.1, 0.45, 0.2]
    for q in (1, 2, 3, 4):
        beta = extrapolation_constants(4, dts, q)
        times = [0.0]
        for i in range(1, 4):
            times.append(times[-1] - dts[i])
        for deg in range(q):
            f = lambda t: (t + 0.7) ** deg
            assert sum(b * f(t) for b, t in zip(beta, times)) == pytest.approx(f(dts[0]), rel=1e-12)


def test_adaptive_values():
    # steps {0.1, 0.2, 0.3, ...}: order 2 -> (1.5, -0.5); order 3 -> (1.8, -1.0, 0.2)
    d = [0.1, 0.2, 0.3, 0.4, 0.5]
    assert extrapolation_constants(2, d) == pytest.approx([1.5, -0.5], rel=1e-13)
    assert extrapolation_constants(3, d) == pytest.approx([1.8, -1.0, 0.2], rel=1e-13)
