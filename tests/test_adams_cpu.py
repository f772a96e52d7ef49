"""CPU restatement of the reference's Adams predictor-corrector and Euler
solvers (src/ivp/adams.rs, src/ivp.rs:240-485), checked against the
reference's own unit tests (the same problems, builder values and
epsilon = 0.01 closed-form bounds on every yielded item) and the step-factor
root against libm pow."""
import math

import numpy as np
import pytest

EXP, DECAY, QUADRATIC, SINE, HARMONIC = 0, 1, 2, 3, 4


def _adams(O, order, rhs, y0, t0, t1, dt_min, dt_max, tol):
    cfg = O.adams_cfg(order=order, tol=tol, dt_min=dt_min, dt_max=dt_max)
    p = O.adams_solve_one(cfg, rhs, np.array(y0, float), t0, t1, traj_cap=200000)
    assert p.status == 0
    return p


# src/ivp/adams.rs tests: (order, rhs, y0, t_final, dt_min, dt_max, tol, exact)
ADAMS_CASES = [
    (5, EXP, [1.0], 2.0, 1e-5, 0.1, 0.0005, np.exp),
    (5, QUADRATIC, [1.0], 5.0, 1e-7, 0.001, 0.01, lambda t: 1.0 - t * t),
    (5, SINE, [0.0], 2 * math.pi, 1e-5, 0.001, 0.01, np.sin),
    (3, EXP, [1.0], 2.0, 1e-5, 0.1, 0.001, np.exp),
    (3, SINE, [0.0], 2 * math.pi, 1e-5, 0.001, 0.01, np.sin),
]


@pytest.mark.parametrize("order,rhs,y0,t1,dmin,dmax,tol,exact", ADAMS_CASES)
def test_adams_reference_unit_tests(oracle, order, rhs, y0, t1, dmin, dmax, tol, exact):
    p = _adams(oracle, order, rhs, y0, 0.0, t1, dmin, dmax, tol)
    assert p.accepted > 0
    assert np.abs(p.traj_y[:, 0] - exact(p.traj_t)).max() <= 0.01


def test_adams_yields_bootstrap_states_in_time_order(oracle):
    """After the RK4 bootstrap the iterator re-emits the bootstrap states,
    then the accepted PECE state (the yield machine of adams.rs:417-441)."""
    p = _adams(oracle, 5, EXP, [1.0], 0.0, 2.0, 1e-5, 0.1, 0.0005)
    assert np.all(np.diff(p.traj_t) > 0)
    assert p.t == pytest.approx(2.0)


# src/ivp.rs tests: (rhs, y0, dt, exact of component 0)
EULER_CASES = [
    (HARMONIC, [1.0, 0.0], 0.01, np.cos),
    (EXP, [1.0], 0.005, np.exp),
    (QUADRATIC, [1.0], 0.01, lambda t: 1.0 - t * t),
    (SINE, [0.0], 0.01, np.sin),
]


@pytest.mark.parametrize("rhs,y0,dt,exact", EULER_CASES)
def test_euler_reference_unit_tests(oracle, rhs, y0, dt, exact):
    p = oracle.euler_solve_one(rhs, np.array(y0, float), 0.0, 1.0, dt, traj_cap=100000)
    assert p.status == 0
    assert np.abs(p.traj_y[:, 0] - exact(p.traj_t)).max() <= 0.01
    # the iterator yields the state each step starts from: t = 0 first, and
    # the state reached at t = 1 is never yielded
    assert p.traj_t[0] == 0.0 and p.t < 1.0


@pytest.mark.parametrize("n", [3, 5])
def test_rootn_matches_libm_pow(oracle, n):
    """The step factor is x^RN(1/n) (the reference's powf(order.recip()));
    the engine's fixed-sequence root agrees with glibc's pow bit for bit on
    ~99.9 % of inputs and is never more than one ulp away."""
    rng = np.random.default_rng(7 + n)
    xs = 10.0 ** rng.uniform(-12, 12, 20000)
    same = far = 0
    for x in xs:
        r, p = oracle.rootn(x, n), x ** (1.0 / n)
        same += r == p
        far += abs(r - p) > 2.3e-16 * abs(p)
    assert same / xs.size >= 0.995 and far == 0
    assert oracle.rootn(0.0, n) == 0.0 and math.isinf(oracle.rootn(math.inf, n))
    assert math.isnan(oracle.rootn(-1.0, n))
    # x^RN(1/n), not the true root: 512^RN(1/3) is 8 - 1 ulp, as pow says
    assert oracle.rootn(2.0 ** (3 * n), n) == (2.0 ** (3 * n)) ** (1.0 / n)
