"""The project's FP64 exp, log and pow (afivo-streamer_gb300/csrc/afg_math.h),
which the analytic rate forms of the FP64 transport path use on the GPU and
in the CPU restatement alike (so both evaluate them bit for bit the same).
Here the host build is checked against 60-digit values: exp and log within
2 units in the last place, pow within |y log x| + 4, over the arguments the
rate forms see and the edge cases (zero, subnormals, overflow, NaN)."""
import math

import numpy as np
import pytest

import oracle

mpmath = pytest.importorskip("mpmath")
mpmath.mp.dps = 60


def ulps(got, want):
    """|got - want| in units of the last place of want (doubles)."""
    out = np.empty(len(got))
    for q, (g, w) in enumerate(zip(got, want)):
        wf = float(w)
        if wf == 0.0 or math.isinf(wf):
            out[q] = 0.0 if g == wf else np.inf
            continue
        out[q] = float(abs(mpmath.mpf(g) - w) / mpmath.mpf(math.ulp(wf)))
    return out


def test_exp_within_two_ulp():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-745, 709.7, 4000), rng.uniform(-1, 1, 2000), rng.uniform(-1e-8, 1e-8, 500),
                        rng.uniform(-60, 0, 2000)])
    got = oracle.math_eval(0, x)
    want = [mpmath.exp(mpmath.mpf(v)) for v in x]
    u = ulps(got, want)
    assert u.max() <= 2.0, u.max()


def test_log_within_two_ulp():
    rng = np.random.default_rng(2)
    x = np.concatenate([np.exp(rng.uniform(-740, 709, 4000)), rng.uniform(0.5, 2.0, 2000),
                        1 + rng.uniform(-1e-6, 1e-6, 500), np.array([5e-324, 1e-310, 2.2e-308])])
    got = oracle.math_eval(1, x)
    want = [mpmath.log(mpmath.mpf(v)) for v in x]
    u = ulps(got, want)
    assert u.max() <= 2.0, u.max()


def test_pow_within_bound():
    rng = np.random.default_rng(3)
    x = np.exp(rng.uniform(-20, 20, 4000))
    y = rng.uniform(-4, 4, 4000)
    got = oracle.math_eval(2, x, y)
    want = [mpmath.power(mpmath.mpf(a), mpmath.mpf(b)) for a, b in zip(x, y)]
    u = ulps(got, want)
    bound = np.abs(y * np.log(x)) + 4
    assert np.all(u <= bound), float(np.max(u - bound))


def test_edge_cases():
    inf, nan = np.inf, np.nan
    e = oracle.math_eval(0, np.array([0.0, -0.0, 709.782712893384, 709.79, -745.14, -745.13, -inf, inf, nan]))
    assert e[0] == 1.0 and e[1] == 1.0
    assert np.isfinite(e[2]) and e[2] > 1.7e308
    assert e[3] == inf and e[4] == 0.0 and 0.0 < e[5] < 1e-323
    assert e[6] == 0.0 and e[7] == inf and np.isnan(e[8])
    lg = oracle.math_eval(1, np.array([1.0, 0.0, -1.0, inf, nan]))
    assert lg[0] == 0.0 and lg[1] == -inf and np.isnan(lg[2]) and lg[3] == inf and np.isnan(lg[4])
    x = np.array([2.5, 7.0, 0.0, 0.0, -2.0, -2.0, -2.0, 1.0, 3.0, inf])
    y = np.array([1.0, 2.0, 3.0, -1.0, 3.0, 2.0, 0.5, nan, 0.0, -1.0])
    p = oracle.math_eval(2, x, y)
    assert p[0] == 2.5 and p[1] == 49.0 and p[2] == 0.0 and p[3] == inf
    assert abs(p[4] + 8.0) <= 8 * 4e-16 and abs(p[5] - 4.0) <= 4e-15 and np.isnan(p[6])
    assert p[7] == 1.0 and p[8] == 1.0 and p[9] == 0.0


def test_rate_form_arguments_match_libm_closely():
    """The k13 form c1 exp(-(c2/(c3+Td))^c4) over reduced fields 1-1000 Td:
    the project's functions and the C library's differ by the rounding of
    q = (c2/Td)^c4 carried through exp(-q), i.e. within
    (q (|c4 log(c2/Td)| + 8) + 8) units of 2^-52 relative."""
    rng = np.random.default_rng(4)
    td = rng.uniform(1, 1000, 3000)
    c2, c4 = rng.uniform(50, 2000, 3000), rng.uniform(0.5, 3, 3000)
    q = oracle.math_eval(2, c2 / td, c4)
    k = oracle.math_eval(0, -q)
    ref = np.exp(-np.power(c2 / td, c4))
    ok = ref > 1e-300
    bound = (q * (np.abs(c4 * np.log(c2 / td)) + 8) + 8) * 2.0 ** -52
    assert np.all(np.abs(k[ok] - ref[ok]) / ref[ok] <= bound[ok])
