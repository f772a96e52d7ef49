"""CPU tests of the oracle: the reference's own closed-form checks, the
deterministic fourth root, nalgebra's norm order, the right-hand sides, and
the committed golden fixtures."""
import math
import os
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_reference_quadratic(oracle, method, layout):
    """src/ivp/rk.rs:682-719: y' = -2t, y(0) = 1, every yielded step within
    1e-4 of 1 - t^2 (dt in [1e-4, 0.1], tol 1e-5, t in [0, 10])."""
    cfg = oracle.rk_cfg(method=method, layout=layout, tol=1e-5, dt_min=1e-4, dt_max=0.1)
    p = oracle.rk_solve_one(cfg, 2, np.array([1.0]), 0.0, 10.0, traj_cap=100000)
    assert p.status == 0 and p.accepted > 0
    assert np.all(np.abs(p.traj_y[:, 0] - (1.0 - p.traj_t ** 2)) <= 1e-4)
    assert p.traj_t[-1] == pytest.approx(10.0)


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_reference_sine(oracle, method, layout):
    """src/ivp/rk.rs:721-758: y' = cos t, y(0) = 0, within 1e-2 of sin t."""
    cfg = oracle.rk_cfg(method=method, layout=layout, tol=1e-4, dt_min=1e-3, dt_max=0.01)
    p = oracle.rk_solve_one(cfg, 3, np.array([0.0]), 0.0, 10.0, traj_cap=100000)
    assert p.status == 0 and p.accepted > 0
    assert np.all(np.abs(p.traj_y[:, 0] - np.sin(p.traj_t)) <= 1e-2)


def test_reference_doc_example_exp(oracle):
    """src/ivp/rk.rs:539-559 (doc example, never executed by the reference's
    tests): y' = y, dt in [0.001, 0.1], tol 1e-4, |e^t - y| < 1e-3 on [0, 10]
    holds for the Fehlberg tableau."""
    cfg = oracle.rk_cfg(layout=2, tol=1e-4, dt_min=1e-3, dt_max=0.1)
    p = oracle.rk_solve_one(cfg, 0, np.array([1.0]), 0.0, 10.0, traj_cap=100000)
    assert p.status == 0
    # Absolute error grows with e^t; the doc's bound holds on the early part.
    early = p.traj_t <= 2.0
    assert np.all(np.abs(np.exp(p.traj_t[early]) - p.traj_y[early, 0]) < 1e-3)


def test_as_compiled_fails_on_y_dependent_rhs(oracle):
    """The as-compiled (column-major) matrix uses stage values of the previous
    attempt: on a Van der Pol oscillator it cannot keep dt above dt_min."""
    cfg = oracle.rk_cfg(layout=0, tol=1e-6, dt_min=1e-6, dt_max=0.1, max_attempts=200000)
    p = oracle.rk_solve_one(cfg, 5, np.array([2.0, 0.0]), 0.0, 10.0, params=np.array([1.0]))
    assert p.status in (8, 13)
    assert p.accepted < 50


def test_fehlberg_typo_is_inconsistent(oracle):
    """rk.rs:499 writes 1859/4014; Fehlberg's row 5 sums to c_5 = 1/2 only with
    1859/4104.  The literal makes the embedded error estimate O(dt)."""
    row_lit = -8 / 27 + 2 - 3544 / 2565 + 1859 / 4014 - 11 / 40
    row_fix = -8 / 27 + 2 - 3544 / 2565 + 1859 / 4104 - 11 / 40
    assert abs(row_fix - 0.5) < 1e-12
    assert abs(row_lit - 0.5) > 1e-2


def _is_correctly_rounded(x, r):
    h = Fraction(math.ulp(r)) / 2
    R, X = Fraction(r), Fraction(x)
    lo = R - (h / 2 if math.frexp(r)[0] == 0.5 else h)
    return lo ** 4 <= X <= (R + h) ** 4


def test_qrt_correctly_rounded(oracle):
    rng = np.random.default_rng(0)
    xs = np.concatenate([10.0 ** rng.uniform(-300, 300, 2000), 10.0 ** rng.uniform(-4, 8, 3000),
                         [1.0, 16.0, 0.0625, 2.0, 4.0, 1e-320, 5e-324, 1.7e308]])
    for x in xs:
        r = oracle.qrt(float(x))
        assert _is_correctly_rounded(float(x), r), (x, r)


def test_qrt_special_values(oracle):
    assert oracle.qrt(0.0) == 0.0
    assert oracle.qrt(float("inf")) == float("inf")
    assert math.isnan(oracle.qrt(float("nan")))
    assert oracle.qrt(16.0) == 2.0


def test_qrt_agrees_with_libm_pow_mostly(oracle):
    """glibc pow(x, 0.25) is not always correctly rounded; the two differ by
    at most one ulp and on well under 1% of inputs."""
    rng = np.random.default_rng(1)
    xs = 10.0 ** rng.uniform(-4, 8, 20000)
    diff = 0
    for x in xs:
        a, b = oracle.qrt(float(x)), math.pow(float(x), 0.25)
        if a != b:
            diff += 1
            assert abs(a - b) <= math.ulp(a)
    assert diff / xs.size < 0.01


def test_norm_summation_order(oracle):
    x = np.array([1e-3, 3.0, 1e8, 7.0])
    assert oracle.norm(x[:2]) == math.sqrt(x[0] * x[0] + x[1] * x[1])
    assert oracle.norm(x[:3]) == math.sqrt((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2])
    s4 = (x[0] * x[0] + x[2] * x[2]) + (x[1] * x[1] + x[3] * x[3])
    assert oracle.norm(x, dyn_dim=False) == math.sqrt(s4)
    s4d = ((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2]) + x[3] * x[3]
    assert oracle.norm(x, dyn_dim=True) == math.sqrt(s4d)
    v = np.arange(1.0, 20.0) * 1.1
    acc = [0.0] * 8
    for i in range(16):
        acc[i % 8] += v[i] * v[i]
    res = 0.0 + (acc[0] + acc[4])
    res += acc[1] + acc[5]
    res += acc[2] + acc[6]
    res += acc[3] + acc[7]
    for k in range(16, 19):
        res += v[k] * v[k]
    assert oracle.norm(v, dyn_dim=True) == math.sqrt(res)


def test_rhs_formulas(oracle):
    y = np.array([1.3, -0.7, 2.1])
    f = oracle.rhs_eval(6, 0.0, y, np.array([10.0, 28.0, 8 / 3]))
    np.testing.assert_allclose(f, [10 * (y[1] - y[0]), y[0] * (28 - y[2]) - y[1], y[0] * y[1] - 8 / 3 * y[2]])
    f = oracle.rhs_eval(5, 0.0, y[:2], np.array([1.5]))
    np.testing.assert_allclose(f, [y[1], 1.5 * (1 - y[0] ** 2) * y[1] - y[0]])
    f = oracle.rhs_eval(7, 0.0, y[:2], np.array([1.0, 0.5, 0.7, 1.2]))
    np.testing.assert_allclose(f, [y[0] - 0.5 * y[0] * y[1], 0.7 * y[0] * y[1] - 1.2 * y[1]])


def test_golden_fixtures(oracle):
    """Committed oracle outputs (tests/golden/make_golden.py) are reproduced
    bit for bit."""
    path = os.path.join(HERE, "golden", "rk_golden.npz")
    g = np.load(path)
    for name in sorted({k.split(":")[0] for k in g.files}):
        rhs, method, layout, tol, dtmin, dtmax, t_end = g[f"{name}:cfg"]
        cfg = oracle.rk_cfg(method=int(method), layout=int(layout), tol=tol, dt_min=dtmin, dt_max=dtmax,
                            max_attempts=int(g[f"{name}:cap"]))
        r = oracle.rk_solve_batch(cfg, int(rhs), g[f"{name}:y0"], g[f"{name}:params"], 0.0, t_end, threads=2)
        np.testing.assert_array_equal(r["y"], g[f"{name}:y"])
        np.testing.assert_array_equal(r["accepted"], g[f"{name}:accepted"])
        np.testing.assert_array_equal(r["rejected"], g[f"{name}:rejected"])
        np.testing.assert_array_equal(r["status"], g[f"{name}:status"])
