"""Dense output: every (t, y) item the reference iterator yields
(src/ivp.rs:209-238, collect_vec), packed into one stream with CSR offsets,
bit for bit against the oracle's per-system paths.  Also the fixed per-system
slabs: a system whose slab is full ends with BACON_CAPACITY_EXCEEDED (17)
instead of dropping items."""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _check_packed(sol, paths, dim):
    off = np.asarray(sol.traj_off)
    assert off[0] == 0 and np.all(np.diff(off) == np.asarray(sol.accepted))
    for i, p in enumerate(paths):
        a, b = int(off[i]), int(off[i + 1])
        assert b - a == p.accepted == len(p.traj_t)
        np.testing.assert_array_equal(sol.traj_t[a:b], p.traj_t)
        np.testing.assert_array_equal(sol.traj_y[a:b].reshape(-1, dim), p.traj_y.reshape(-1, dim))


def test_rk45_dense_lorenz_uneven_end_times(engine, oracle):
    """1,024 Lorenz systems of the headline workload (T ~ U[1, 20]):
    ~2.4 million items, bit-identical to the oracle's paths."""
    b = W.lorenz(n=1 << 20).subset(np.arange(0, 1 << 20, 1024))
    sol = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min,
                          dt_max=b.dt_max, layout=2, dense=True)
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    paths = []
    for i in range(b.n):
        p = oracle.rk_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, float(b.t_end[i]), params=b.params[:, i],
                                traj_cap=8192)
        assert p.accepted <= 8192
        paths.append(p)
    assert int(sol.traj_off[-1]) == sum(p.accepted for p in paths) > 1_000_000
    _check_packed(sol, paths, 3)


def test_rk45_dense_device_resident_matches_host(engine):
    import torch
    b = W.lorenz(n=1 << 20).subset(np.arange(0, 1 << 20, 4096))
    host = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min,
                           dt_max=b.dt_max, layout=2, dense=True)
    dev = torch.device("cuda")
    d = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (b.y0, b.params, b.t0, b.t_end)]
    sol = engine.rk_solve(*d, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, layout=2, dense=True)
    np.testing.assert_array_equal(sol.traj_off.cpu().numpy(), host.traj_off)
    np.testing.assert_array_equal(sol.traj_t.cpu().numpy(), host.traj_t)
    np.testing.assert_array_equal(sol.traj_y.cpu().numpy(), host.traj_y)


def test_dense_capacity_too_small_reports_the_total(engine):
    """capacity < total: BACON_CAPACITY_EXCEEDED after the counting pass,
    with the total and the offsets filled."""
    import ctypes
    from bacon_gb300 import _capi
    b = W.van_der_pol(n=64, seed=12)
    prob = engine.make_problem(b.y0, b.params, 0.0, 10.0, b.tol, b.dt_min, b.dt_max, b.rhs)
    opts = engine.rk_options(layout=2)
    out = engine.alloc_outputs(2, b.n, device=False)
    res = engine.make_result(out)
    off = np.zeros(b.n + 1, np.int64)
    t = np.zeros(10)
    y = np.zeros((10, 2))
    dz = _capi.DenseOutput()
    dz.capacity, dz.t, dz.y, dz.offsets = 10, t.ctypes.data, y.ctypes.data, off.ctypes.data
    code = _capi.load().bacon_rk_solve_dense(engine.default_context().handle, ctypes.byref(prob),
                                             ctypes.byref(opts), ctypes.byref(res), ctypes.byref(dz))
    assert code == 17
    assert dz.total == int(out["accepted"].sum()) == off[-1] > 10
    np.testing.assert_array_equal(np.diff(off), out["accepted"])
    assert not t.any()


def test_bdf_dense_robertson(engine, oracle):
    rob = W.robertson(n=64, seed=23)
    sol = engine.bdf_solve(rob.y0, rob.params, 0.0, 1e4, rhs=rob.rhs, tol=rob.tol, dt_min=rob.dt_min,
                           dt_max=rob.dt_max, dense=True)
    assert sol.code == 0
    cfg = oracle.bdf_cfg(mode=oracle.BDF_CORRECTED, tol=rob.tol, dt_min=rob.dt_min, dt_max=rob.dt_max)
    paths = [oracle.bdf_solve_one(cfg, rob.rhs, rob.y0[:, i], 0.0, 1e4, params=rob.params[:, i], traj_cap=4096)
             for i in range(rob.n)]
    _check_packed(sol, paths, 3)


def test_adams5_dense_van_der_pol(engine, oracle):
    """t in [0, 2]: the reference's Adams5 takes ~10^5 step calls per unit
    time here."""
    b = W.van_der_pol(n=32, seed=29)
    sol = engine.adams_solve(b.y0, b.params, 0.0, 2.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                             order=5, dense=True)
    cfg = oracle.adams_cfg(order=5, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    paths = [oracle.adams_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, 2.0, params=b.params[:, i], traj_cap=1 << 22)
             for i in range(b.n)]
    np.testing.assert_array_equal(sol.status, [p.status for p in paths])
    _check_packed(sol, paths, 2)


def test_full_slab_ends_with_capacity_status(engine, oracle):
    """A slab of 50 items: systems with more items stop with status 17 at
    the item that does not fit; their first 50 items and final state are
    those of the oracle's path at item 50."""
    b = W.van_der_pol(n=256, seed=31)
    cap = 50
    sol = engine.rk_solve(b.y0, b.params, 0.0, 10.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, traj_cap=cap)
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    full = 0
    for i in range(b.n):
        p = oracle.rk_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, 10.0, params=b.params[:, i], traj_cap=4096)
        k = min(p.accepted, cap)
        np.testing.assert_array_equal(sol.traj_t[i, :k], p.traj_t[:k])
        np.testing.assert_array_equal(sol.traj_y[i, :k], p.traj_y[:k])
        if p.accepted > cap:
            full += 1
            assert sol.status[i] == 17 and sol.accepted[i] == cap
            assert sol.t[i] == p.traj_t[cap - 1]
            np.testing.assert_array_equal(sol.y[:, i], p.traj_y[cap - 1])
        else:
            assert sol.status[i] == 0 and sol.accepted[i] == p.accepted
    assert full > 0


def test_dense_output_of_failing_systems(engine, oracle):
    """A system that fails keeps the items it yielded before the failure:
    the attempt cap (NaN state, no item), MinimumTimeDeltaExceeded (stiff),
    end <= start (no item); the rest are complete."""
    b = W.van_der_pol(n=48, seed=61)
    b.y0 = b.y0.copy()
    b.y0[0, 3] = np.nan
    b.params = b.params.copy()
    b.params[0, 7] = 1e6
    b.t_end = b.t_end.copy()
    b.t_end[11] = -1.0
    sol = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, max_attempts=3000, dense=True)
    assert sol.status[3] == 13 and sol.status[7] == 8 and sol.status[11] == 5
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, max_attempts=3000)
    paths = [oracle.rk_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, float(b.t_end[i]), params=b.params[:, i],
                                 traj_cap=4096) for i in range(b.n)]
    np.testing.assert_array_equal(sol.status, [p.status for p in paths])
    _check_packed(sol, paths, 2)


def test_dense_fp32_stage_matches_its_slab(engine):
    """The FP32-stage kernel writes the same items packed as into slabs."""
    b = W.lorenz(n=1 << 20).subset(np.arange(0, 1 << 20, 8192))
    b.t_end = np.minimum(b.t_end, 3.0)
    kw = dict(rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, layout=2, precision=2)
    slab = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, traj_cap=4096, **kw)
    dense = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, dense=True, **kw)
    assert (slab.status == 0).all()
    off = dense.traj_off
    for i in range(b.n):
        k = int(slab.accepted[i])
        np.testing.assert_array_equal(dense.traj_t[off[i]:off[i + 1]], slab.traj_t[i, :k])
        np.testing.assert_array_equal(dense.traj_y[off[i]:off[i + 1]], slab.traj_y[i, :k])


def test_euler_dense_matches_oracle_path(engine, oracle):
    """Euler yields the state each step starts from (src/ivp.rs:318-339)."""
    b = W.van_der_pol(n=64, seed=67)
    sol = engine.euler_solve(b.y0, b.params, 0.0, 2.0, rhs=b.rhs, dt=0.01, dense=True)
    assert sol.code == 0
    paths = [oracle.euler_solve_one(b.rhs, b.y0[:, i], 0.0, 2.0, 0.01, params=b.params[:, i], traj_cap=4096)
             for i in range(b.n)]
    _check_packed(sol, paths, 2)


def test_linear_dense_exact_matches_oracle_paths(engine, oracle):
    """The lock-step linear engine (one shared A, dim 64, FP64 exact) yields
    every accepted (t, y) from its control kernel, bit-identical to the
    oracle's per-system paths; per-system end times leave systems running in
    different rounds."""
    b = W.linear_shared(n=37, dim=64, seed=41)
    t_end = np.random.default_rng(7).uniform(1.0, 5.0, b.n)
    sol = engine.rk_solve(b.y0, None, 0.0, t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, precision=0, shared=b.extra["A"], dense=True)
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    paths = [oracle.rk_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, float(t_end[i]), shared=b.extra["A"],
                                 traj_cap=4096) for i in range(b.n)]
    _check_packed(sol, paths, 64)


def test_linear_dense_tensor_core_path(engine):
    """The tensor-core engine's items: one per accepted attempt, times
    increasing to t_end, the last item the final state, and every state within
    the split's accuracy of the exact solution at its own time."""
    b = W.linear_shared(n=256, dim=128, seed=42)
    sol = engine.rk_solve(b.y0, None, 0.0, 5.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, precision=engine.TC_SPLIT, shared=b.extra["A"], dense=True)
    assert sol.code == 0
    off = np.asarray(sol.traj_off)
    assert np.all(np.diff(off) == sol.accepted)
    q, lam = b.extra["Q"], b.extra["lambda"]
    for i in range(0, b.n, 17):
        a, e = int(off[i]), int(off[i + 1])
        ts = sol.traj_t[a:e]
        assert np.all(np.diff(ts) > 0) and ts[-1] == sol.t[i]
        ys = sol.traj_y[a:e].reshape(-1, 128)
        np.testing.assert_array_equal(ys[-1], sol.y[:, i])
        exact = q @ (np.exp(-lam[:, None] * ts[None, :]) * (q.T @ b.y0[:, i])[:, None])
        assert np.abs(ys - exact.T).max() < 1e-7


def test_linear_slab_full_ends_with_capacity_status(engine, oracle):
    """A per-system slab too small for the path: the system ends with
    BACON_CAPACITY_EXCEEDED once the slab is full, its final state the last
    item it yielded, as the oracle's path says."""
    b = W.linear_shared(n=8, dim=64, seed=43)
    sol = engine.rk_solve(b.y0, None, 0.0, 5.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, precision=0, shared=b.extra["A"], traj_cap=40)
    assert (sol.status == 17).all() and (sol.accepted == 40).all() and sol.code == 17
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    for i in range(b.n):
        p = oracle.rk_solve_one(cfg, b.rhs, b.y0[:, i], 0.0, 5.0, shared=b.extra["A"], traj_cap=4096)
        np.testing.assert_array_equal(sol.traj_t[i], p.traj_t[:40])
        np.testing.assert_array_equal(sol.traj_y[i].reshape(-1, 64), p.traj_y.reshape(-1, 64)[:40])
        np.testing.assert_array_equal(sol.y[:, i], p.traj_y.reshape(-1, 64)[39])
