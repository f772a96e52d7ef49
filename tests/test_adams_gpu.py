"""GPU batched Adams5 / Adams3 and Euler against the CPU restatement, bit
for bit (states, times, yielded-item and Redo counts, statuses), on the
reference's unit-test problems and on the benchmark families."""
import math

import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oracle_adams(O, b, order, max_attempts=0, dyn=False):
    cfg = O.adams_cfg(order=order, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, max_attempts=max_attempts,
                      dyn_dim=dyn)
    out = {"y": np.zeros_like(b.y0), "t": np.zeros(b.n), "accepted": np.zeros(b.n, np.int64),
           "rejected": np.zeros(b.n, np.int64), "status": np.zeros(b.n, np.int32)}
    for i in range(b.n):
        p = O.adams_solve_one(cfg, b.rhs, b.y0[:, i], b.t0[i], b.t_end[i],
                              params=b.params[:, i] if b.params.size else None)
        out["y"][:, i], out["t"][i], out["accepted"][i], out["rejected"][i], out["status"][i] = (
            p.y, p.t, p.accepted, p.rejected, p.status)
    return out


def _same(sol, ref):
    np.testing.assert_array_equal(sol.status, ref["status"])
    np.testing.assert_array_equal(sol.accepted, ref["accepted"])
    np.testing.assert_array_equal(sol.rejected, ref["rejected"])
    np.testing.assert_array_equal(sol.t, ref["t"])
    np.testing.assert_array_equal(sol.y.view(np.int64), ref["y"].view(np.int64))


def _gpu_adams(E, b, order, **kw):
    return E.adams_solve(b.y0, b.params if b.params.size else None, b.t0, b.t_end, rhs=b.rhs, tol=b.tol,
                         dt_min=b.dt_min, dt_max=b.dt_max, order=order, **kw)


# The reference's Adams clears its history on every dt change and restarts
# with an RK4 bootstrap, so it takes ~10^5 step calls per Van der Pol system
# at tol 1e-6 (order 5) and ~10^6 (order 3): the horizons here are short.
@pytest.mark.parametrize("order", [5, 3])
def test_adams_vdp_bit_exact(engine, oracle, order):
    b = W.van_der_pol(n=256, seed=81)
    b.t_end = np.full(b.n, 2.0 if order == 5 else 0.5)
    _same(_gpu_adams(engine, b, order), _oracle_adams(oracle, b, order))


@pytest.mark.parametrize("order", [5, 3])
def test_adams_lotka_volterra_bit_exact(engine, oracle, order):
    b = W.lotka_volterra(n=256, seed=82)
    b.tol = 1e-6
    b.t_end = np.full(b.n, 3.0)
    _same(_gpu_adams(engine, b, order), _oracle_adams(oracle, b, order))


def test_adams_lorenz_short_bit_exact(engine, oracle):
    """Adams5 cannot hold dt above 1e-8 on these Lorenz systems: every one
    ends with MinimumTimeDeltaExceeded, some only after millions of step
    calls, so both sides get the same cap."""
    b = W.lorenz(n=32, seed=83)
    b.t_end = np.minimum(b.t_end, 1.0)
    _same(_gpu_adams(engine, b, 5, max_attempts=2_000_000), _oracle_adams(oracle, b, 5, max_attempts=2_000_000))


def test_adams_reference_problems_and_paths(engine, oracle):
    """The reference's adams5_exp problem through the builder mirror: the
    whole yielded path equals the restatement's and stays within 0.01 of
    exp(t)."""
    from bacon_gb300.ivp import Adams5, Rhs
    it = (Adams5.new(1).with_minimum_dt(1e-5).with_maximum_dt(0.1).with_tolerance(0.0005)
          .with_initial_time(0.0).with_ending_time(2.0).with_initial_conditions_slice([1.0])
          .with_derivative(Rhs.EXP).solve(()))
    path = it.collect_vec()
    ref = oracle.adams_solve_one(oracle.adams_cfg(order=5, tol=0.0005, dt_min=1e-5, dt_max=0.1), 0,
                                 np.array([1.0]), 0.0, 2.0, traj_cap=100000)
    assert len(path) == ref.accepted
    np.testing.assert_array_equal([t for t, _ in path], ref.traj_t)
    np.testing.assert_array_equal(np.array([y[0] for _, y in path]), ref.traj_y[:, 0])
    assert max(abs(y[0] - math.exp(t)) for t, y in path) <= 0.01


def test_adams_failures_retire_only_their_system(engine, oracle):
    """A NaN initial state (Redo forever: the cap) and an end before the
    start retire only their own systems.  The reference's Adams5 also fails
    on some clean Van der Pol systems (MinimumTimeDeltaExceeded), identically
    in both.  (Over t in [0, 0.2] the RK4 bootstrap lands exactly on the end
    and the reference returns Done without yielding anything, hence 0.5.)"""
    b = W.van_der_pol(n=64, seed=84)
    b.y0 = b.y0.copy()
    b.y0[0, 5] = np.nan
    b.t_end = b.t_end.copy()
    b.t_end[7] = -1.0
    b.t_end = np.where(b.t_end > 0, 0.5, b.t_end)
    sol = _gpu_adams(engine, b, 5, max_attempts=200_000)
    ref = _oracle_adams(oracle, b, 5, max_attempts=200_000)
    _same(sol, ref)
    assert sol.status[5] == 13 and sol.status[7] == 5
    assert (sol.status == 0).sum() >= 40


@pytest.mark.parametrize("rhs,y0,dt", [(4, [1.0, 0.0], 0.01), (0, [1.0], 0.005), (2, [1.0], 0.01),
                                       (3, [0.0], 0.01)])
def test_euler_reference_problems_bit_exact(engine, oracle, rhs, y0, dt):
    n = 8
    Y0 = np.tile(np.array(y0, float)[:, None], (1, n))
    te = np.linspace(0.5, 1.0, n)
    sol = engine.euler_solve(Y0, None, np.zeros(n), te, rhs=rhs, dt=dt)
    for i in range(n):
        p = oracle.euler_solve_one(rhs, Y0[:, i], 0.0, te[i], dt)
        assert sol.status[i] == p.status and sol.accepted[i] == p.accepted and sol.t[i] == p.t
        np.testing.assert_array_equal(sol.y[:, i].view(np.int64), p.y.view(np.int64))


def test_euler_builder_dt_averaging(engine):
    """Euler's with_maximum_dt / with_minimum_dt: the first value, then the
    mean with each later one (src/ivp.rs:395-423); tolerance is a no-op."""
    from bacon_gb300.ivp import Euler, Rhs
    it = (Euler.new(1).with_tolerance(-1.0).with_maximum_dt(0.02).with_minimum_dt(0.01)
          .with_initial_time(0.0).with_ending_time(1.0).with_initial_conditions_slice([1.0])
          .with_derivative(Rhs.EXP).solve(()))
    path = it.collect_vec()
    ts = np.array([t for t, _ in path])
    np.testing.assert_allclose(np.diff(ts[:5]), 0.015)


def test_adams5_vdp_config_full_4096(engine, oracle):
    """The benchmark's Adams5 workload in full: 4,096 Van der Pol systems to
    t = 10, ~2.8e9 step calls and ~3e8 fifth roots.  The oracle runs
    each system on its own host thread pool."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    b = W.van_der_pol()
    cfg = oracle.adams_cfg(order=5, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)

    def one(i):
        return oracle.adams_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, 10.0, params=b.params[:, i])

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        paths = list(ex.map(one, range(b.n)))
    ref = {"y": np.stack([p.y for p in paths], axis=1), "t": np.array([p.t for p in paths]),
           "accepted": np.array([p.accepted for p in paths]), "rejected": np.array([p.rejected for p in paths]),
           "status": np.array([p.status for p in paths], np.int32)}
    _same(_gpu_adams(engine, b, 5), ref)
