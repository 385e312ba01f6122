"""The explicit integrators of af_advance as forward_euler stages.

The host step driver and the CPU restatement each restate the stage table
(afivo/src/m_af_advance.f90:150-199); both must agree, and applied to the
scalar ODE y' = k y the stages must show each method's order of accuracy
(forward Euler 1, midpoint and Heun 2, SSPRK3(3) and SSPRK3(4) 3, RK4 4)."""
import numpy as np
import pytest

import streamer_model as sm
from oracle_streamer import STAGES

ORDER = {"forward_euler": 1, "midpoint": 2, "heun": 2, "ssprk33": 3, "ssprk43": 3, "rk4": 4}


def test_tables_agree():
    assert set(STAGES) == set(sm.INTEGRATORS) == set(ORDER)
    for name, stages in sm.INTEGRATORS.items():
        assert stages == STAGES[name]


def advance(name, k, dt, y0=1.0):
    """States y[s]; each stage: y[s_out] = sum w y[s_prev] + f dt k y[s_deriv]."""
    stages = sm.INTEGRATORS[name]
    y = np.zeros(len(stages) + 1)
    y[0] = y0
    for f, s_deriv, s_prev, w_prev, s_out in stages:
        deriv = k * y[s_deriv]
        y[s_out] = sum(w * y[s] for s, w in zip(s_prev, w_prev)) + f * dt * deriv
    return y[0]


@pytest.mark.parametrize("name", sorted(ORDER))
def test_order_of_accuracy(name):
    k = -1.3
    errs = []
    for n in (20, 40):
        dt = 1.0 / n
        y = 1.0
        for _ in range(n):
            y = advance(name, k, dt, y)
        errs.append(abs(y - np.exp(k)))
    order = np.log2(errs[0] / errs[1])
    assert abs(order - ORDER[name]) < 0.15, (name, order)
    assert sm.states_needed(name) == len(sm.INTEGRATORS[name]) + 1
