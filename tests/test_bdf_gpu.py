"""GPU batched BDF6 / BDF2 against the CPU oracle, bit for bit.

As-compiled mode reproduces the reference's BDFSolver (src/ivp/bdf.rs:495-634)
including its failure modes (no yielded items on its own test problems,
MaximumIterationsExceeded on Robertson); corrected mode is the engine's
stiff BDF, checked bit for bit against the oracle's restatement and for
accuracy against scipy's Radau at rtol 1e-12.
"""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oracle(O, b, mode, method=0, max_steps=200000, t_end=None):
    cfg = O.bdf_cfg(method=method, mode=mode, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, max_steps=max_steps)
    out = {"y": np.zeros_like(b.y0), "t": np.zeros(b.n), "accepted": np.zeros(b.n, np.int64),
           "rejected": np.zeros(b.n, np.int64), "status": np.zeros(b.n, np.int32)}
    for i in range(b.n):
        te = b.t_end[i] if t_end is None else t_end
        p = O.bdf_solve_one(cfg, b.rhs, b.y0[:, i], b.t0[i], te, params=b.params[:, i] if b.params.size else None)
        out["y"][:, i] = p.y
        out["t"][i] = p.t
        out["accepted"][i] = p.accepted
        out["rejected"][i] = p.rejected
        out["status"][i] = p.status
    return out


def _gpu(E, b, mode, method=0, max_steps=200000):
    return E.bdf_solve(b.y0, b.params if b.params.size else None, b.t0, b.t_end, rhs=b.rhs, tol=b.tol,
                       dt_min=b.dt_min, dt_max=b.dt_max, method=method, mode=mode, max_steps=max_steps)


def _same(sol, ref):
    np.testing.assert_array_equal(sol.status, ref["status"])
    np.testing.assert_array_equal(sol.accepted, ref["accepted"])
    np.testing.assert_array_equal(sol.rejected, ref["rejected"])
    np.testing.assert_array_equal(sol.t, ref["t"])
    np.testing.assert_array_equal(sol.y.view(np.int64), ref["y"].view(np.int64))


def test_corrected_robertson_bit_exact(engine, oracle):
    b = W.robertson(n=256)
    sol = _gpu(engine, b, engine.BDF_CORRECTED)
    ref = _oracle(oracle, b, oracle.BDF_CORRECTED)
    assert (sol.status == 0).all()
    _same(sol, ref)


@pytest.mark.parametrize("masses", [2, 3, 4])
def test_corrected_spring_chain_bit_exact(engine, oracle, masses):
    b = W.spring_chains(n=64, masses=masses)
    sol = _gpu(engine, b, engine.BDF_CORRECTED)
    ref = _oracle(oracle, b, oracle.BDF_CORRECTED)
    assert (sol.status == 0).all()
    _same(sol, ref)


def test_corrected_bdf2_bit_exact(engine, oracle):
    b = W.robertson(n=64, seed=9)
    b.t_end = np.full(b.n, 10.0)
    sol = _gpu(engine, b, engine.BDF_CORRECTED, method=engine.BDF2)
    ref = _oracle(oracle, b, oracle.BDF_CORRECTED, method=oracle.BDF2)
    _same(sol, ref)


def test_corrected_robertson_accuracy_vs_radau(engine):
    from scipy.integrate import solve_ivp
    b = W.robertson(n=16, seed=12)
    sol = _gpu(engine, b, engine.BDF_CORRECTED)
    for i in range(b.n):
        k1, k2, k3 = b.params[:, i]

        def f(t, y):
            return [-k1 * y[0] + k3 * y[1] * y[2], k1 * y[0] - k2 * y[1] ** 2 - k3 * y[1] * y[2], k2 * y[1] ** 2]

        r = solve_ivp(f, (0, 1e4), b.y0[:, i], method="Radau", rtol=1e-12, atol=1e-14)
        assert np.abs(sol.y[:, i] - r.y[:, -1]).max() < 1e-4


def _unit(rhs, y0, t_end, n=4):
    y = np.full((1, n), y0)
    return W.Batch("unit", rhs, y, np.zeros((0, n)), np.zeros(n), np.full(n, t_end), 1e-5, 1e-5, 0.1, 0)


@pytest.mark.parametrize("case", [(W.RHS_EXP, 1.0, 7.0), (W.RHS_DECAY, 1.0, 10.0), (W.RHS_QUADRATIC, 1.0, 2.0)])
@pytest.mark.parametrize("method", [0, 1])
def test_as_compiled_reference_tests(engine, oracle, case, method):
    """src/ivp/bdf.rs:785-1063: the reference yields no items on its own test
    problems (its assertions never run); the engine reproduces that exactly."""
    b = _unit(*case)
    sol = _gpu(engine, b, engine.BDF_AS_COMPILED, method=method)
    ref = _oracle(oracle, b, oracle.BDF_AS_COMPILED, method=method)
    _same(sol, ref)
    assert (sol.accepted == 0).all()


def test_as_compiled_robertson(engine, oracle):
    b = W.robertson(n=32, seed=14)
    sol = _gpu(engine, b, engine.BDF_AS_COMPILED)
    ref = _oracle(oracle, b, oracle.BDF_AS_COMPILED)
    _same(sol, ref)
    assert (sol.status == 9).all()  # MaximumIterationsExceeded, as the reference


def test_corrected_reference_tests_via_builder(engine):
    """The reference's BDF6 tests (bdf.rs:820-923), run by the corrected
    solver through the builder mirror."""
    from bacon_gb300.ivp import BDF6, Rhs
    for rhs, y0, t_end, exact, eps in [(Rhs.DECAY, 1.0, 10.0, lambda t: np.exp(-t), 0.01),
                                       (Rhs.QUADRATIC, 1.0, 2.0, lambda t: 1 - t * t, 0.01),
                                       (Rhs.SINE, 0.0, 6.0, np.sin, 0.01)]:
        path = (BDF6.new(1).with_minimum_dt(1e-9).with_maximum_dt(0.1).with_tolerance(1e-5)
                .with_initial_time(0.0).with_ending_time(t_end).with_initial_conditions_slice([y0])
                .with_derivative(rhs).solve(()).collect_vec())
        assert len(path) > 0
        for t, y in path:
            assert abs(y[0] - exact(t)) <= eps


@pytest.mark.parametrize("kind", ["lorenz", "lotka_volterra"])
def test_as_compiled_secant_fallbacks(engine, oracle, kind):
    """The reference's secant on multi-dimensional systems: the "+" finite
    difference makes the Jacobian's columns nearly equal, its partial-pivot
    LU meets exactly zero pivots, and the full-pivot LU and QR fallbacks
    (src/ivp/bdf.rs:433-443) take over.  Bit for bit against the oracle,
    including the systems where all three fail (SingularMatrix)."""
    if kind == "lorenz":
        b = W.lorenz(n=64, seed=5)
        b.t_end = np.full(b.n, 2.0)
    else:
        b = W.lotka_volterra(n=64, seed=6)
        b.t_end = np.full(b.n, 5.0)
    sol = _gpu(engine, b, engine.BDF_AS_COMPILED, max_steps=20000)
    ref = _oracle(oracle, b, oracle.BDF_AS_COMPILED, max_steps=20000)
    _same(sol, ref)
