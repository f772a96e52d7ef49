"""GPU discrete adjoint (batched solve_ivp_adjoint) against the CPU oracle's
reverse sweep (bit-identical), frozen-step central differences (h = 1e-6,
1e-6 relative) and forward sensitivities.  Calls go through the C ABI."""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _gpu(E, b, target, **kw):
    return E.rk_solve_adjoint(b.y0, b.params, b.t0, b.t_end, target, rhs=b.rhs, tol=b.tol,
                              dt_min=b.dt_min, dt_max=b.dt_max, **kw)


@pytest.mark.parametrize("every", [32, 7, 1])
def test_lotka_volterra_adjoint_bit_exact(engine, oracle, every):
    b = W.lotka_volterra(n=256)
    tg = b.extra["target"]
    sol = _gpu(engine, b, tg, layout=2, checkpoint_every=every)
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    for i in range(0, b.n, 17):
        st, L, gy, gp = oracle.rk_adjoint_one(cfg, b.rhs, b.y0[:, i], b.params[:, i], 0.0, 15.0, tg[:, i],
                                              checkpoint_every=every)
        assert st == 0
        assert sol.loss[i] == L
        np.testing.assert_array_equal(sol.dl_dy0[:, i], gy)
        np.testing.assert_array_equal(sol.dl_dp[:, i], gp)


def test_adjoint_vs_frozen_fd_and_forward_sensitivities(engine, oracle):
    b = W.lotka_volterra(n=64, seed=31)
    tg = b.extra["target"]
    sol = _gpu(engine, b, tg, layout=2)
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    worst_fd = worst_fs = 0.0
    for i in range(b.n):
        g = np.concatenate([sol.dl_dy0[:, i], sol.dl_dp[:, i]])
        _, fy, fp = oracle.rk_frozen_fd_one(cfg, b.rhs, b.y0[:, i], b.params[:, i], 0.0, 15.0, tg[:, i], 1e-6)
        _, sy, sp = oracle.rk_fwdsens_one(cfg, b.rhs, b.y0[:, i], b.params[:, i], 0.0, 15.0, tg[:, i])
        scale = np.abs(g).max()
        worst_fd = max(worst_fd, np.abs(g - np.concatenate([fy, fp])).max() / scale)
        worst_fs = max(worst_fs, np.abs(g - np.concatenate([sy, sp])).max() / scale)
    assert worst_fd <= 1e-6, worst_fd
    assert worst_fs <= 1e-12, worst_fs


@pytest.mark.parametrize("rhs_case", ["vdp", "lorenz"])
def test_other_rhs_adjoint(engine, oracle, rhs_case):
    if rhs_case == "vdp":
        b = W.van_der_pol(n=64, seed=41)
    else:
        b = W.lorenz(n=64, seed=42)
        b.t_end = np.minimum(b.t_end, 2.0)
    rng = np.random.default_rng(5)
    tg = rng.normal(size=b.y0.shape)
    sol = _gpu(engine, b, tg, layout=2, max_steps=4096)
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    for i in range(0, b.n, 9):
        st, L, gy, gp = oracle.rk_adjoint_one(cfg, b.rhs, b.y0[:, i], b.params[:, i], 0.0, b.t_end[i], tg[:, i])
        assert st == 0
        np.testing.assert_array_equal(sol.dl_dy0[:, i], gy)
        np.testing.assert_array_equal(sol.dl_dp[:, i], gp)


def test_adjoint_capacity_and_failures(engine):
    b = W.lotka_volterra(n=32, seed=51)
    tg = b.extra["target"]
    sol = _gpu(engine, b, tg, layout=2, max_steps=16)
    assert (sol.forward.status == 17).all()            # step log too small
    assert np.isnan(sol.loss).all()
    b.y0 = b.y0.copy()
    b.y0[0, 3] = np.nan
    sol = _gpu(engine, b, tg, layout=2, max_attempts=2000)
    assert sol.forward.status[3] == 13 and np.isnan(sol.dl_dy0[:, 3]).all()
    ok = np.arange(32) != 3
    assert (sol.forward.status[ok] == 0).all() and np.isfinite(sol.dl_dp[:, ok]).all()


def test_adjoint_device_path_matches_host(engine):
    import torch
    b = W.lotka_volterra(n=1024, seed=61)
    tg = b.extra["target"]
    host = _gpu(engine, b, tg, layout=2)
    dev = torch.device("cuda")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    sol = engine.rk_solve_adjoint(T(b.y0), T(b.params), 0.0, 15.0, T(tg), rhs=b.rhs, tol=b.tol,
                                  dt_min=b.dt_min, dt_max=b.dt_max, layout=2)
    np.testing.assert_array_equal(sol.dl_dp.cpu().numpy(), host.dl_dp)
    np.testing.assert_array_equal(sol.loss.cpu().numpy(), host.loss)
