"""Ragged (uneven-size) stiff batches: one warp per spring-mass chain, and the
mixed Robertson + chains launch, bit for bit against the CPU oracle's
corrected BDF (each chain a dynamically sized system) and against the
one-thread-per-system kernel for the uniform part."""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# sizes around the 32-row chunk boundaries of the warp layout (dim = 2 m)
MASSES = [1, 2, 3, 5, 8, 15, 16, 17, 24, 31, 32, 33, 40, 47, 48, 49, 63, 64]


def _chains(masses, seed, t_end):
    rng = np.random.default_rng(seed)
    base = W.ragged_spring_chains(n=len(masses), min_masses=1, max_masses=1, seed=seed)
    ys, ps = [], []
    for m in masses:
        k = 10.0 ** rng.uniform(0.0, 6.0, m)
        ps.append(np.concatenate([k, [2.0 * np.sqrt(k.max())]]))
        y = np.zeros(2 * m)
        y[:m] = rng.uniform(-1.0, 1.0, m)
        ys.append(y)
    base.y_off = np.concatenate([[0], np.cumsum([len(y) for y in ys])]).astype(np.int64)
    base.p_off = np.concatenate([[0], np.cumsum([len(p) for p in ps])]).astype(np.int64)
    base.y0 = np.concatenate(ys)
    base.params = np.concatenate(ps)
    base.t_end = np.full(len(masses), t_end)
    base.t0 = np.zeros(len(masses))
    return base


def _oracle_ragged(O, r, method=0, max_steps=200000):
    cfg = O.bdf_cfg(method=method, mode=O.BDF_CORRECTED, dyn_dim=True, tol=r.tol, dt_min=r.dt_min,
                    dt_max=r.dt_max, max_steps=max_steps)
    out = {"y": np.zeros_like(r.y0), "t": np.zeros(r.n), "accepted": np.zeros(r.n, np.int64),
           "rejected": np.zeros(r.n, np.int64), "status": np.zeros(r.n, np.int32)}
    for i in range(r.n):
        y0, p = r.system(i)
        res = O.bdf_solve_one(cfg, r.rhs, y0, r.t0[i], r.t_end[i], params=p)
        out["y"][r.y_off[i]:r.y_off[i + 1]] = res.y
        out["t"][i] = res.t
        out["accepted"][i] = res.accepted
        out["rejected"][i] = res.rejected
        out["status"][i] = res.status
    return out


def _same(sol, ref):
    np.testing.assert_array_equal(sol.status, ref["status"])
    np.testing.assert_array_equal(sol.accepted, ref["accepted"])
    np.testing.assert_array_equal(sol.rejected, ref["rejected"])
    np.testing.assert_array_equal(sol.t, ref["t"])
    np.testing.assert_array_equal(sol.y.view(np.int64), ref["y"].view(np.int64))


def test_ragged_chains_bit_exact(engine, oracle):
    r = _chains(MASSES, seed=31, t_end=0.3)
    _, sol = engine.bdf_solve_mixed(None, r)
    ref = _oracle_ragged(oracle, r)
    assert (ref["status"] == 0).all()
    _same(sol, ref)


def test_ragged_chains_bdf2_bit_exact(engine, oracle):
    """BDF2's order-1/order-2 error estimate keeps dt near 1e-7 on these
    chains, so the horizon is short."""
    r = _chains([1, 3, 16, 17], seed=32, t_end=1e-3)
    _, sol = engine.bdf_solve_mixed(None, r, method=1)
    ref = _oracle_ragged(oracle, r, method=1)
    assert (ref["status"] == 0).all()
    _same(sol, ref)


def test_ragged_chains_full_horizon_sample(engine, oracle):
    """The workload's own distribution (m ~ U{2..64}) over t in [0, 10]."""
    r = W.ragged_spring_chains(n=12, seed=7)
    _, sol = engine.bdf_solve_mixed(None, r)
    ref = _oracle_ragged(oracle, r)
    _same(sol, ref)


def test_mixed_launch_matches_parts(engine, oracle):
    """Robertson (a thread each) and chains (a warp each) in one launch: the
    uniform part equals bacon_bdf_solve, the ragged part the oracle."""
    rob = W.robertson(n=300, seed=41)
    r = _chains(MASSES[::2], seed=42, t_end=0.2)
    us, rs = engine.bdf_solve_mixed(rob, r)
    alone = engine.bdf_solve(rob.y0, rob.params, rob.t0, rob.t_end, rhs=rob.rhs, tol=rob.tol,
                             dt_min=rob.dt_min, dt_max=rob.dt_max, mode=engine.BDF_CORRECTED)
    np.testing.assert_array_equal(us.status, alone.status)
    np.testing.assert_array_equal(us.accepted, alone.accepted)
    np.testing.assert_array_equal(us.rejected, alone.rejected)
    np.testing.assert_array_equal(us.y.view(np.int64), alone.y.view(np.int64))
    _same(rs, _oracle_ragged(oracle, r))


def test_mixed_device_arrays(engine, oracle):
    torch = pytest.importorskip("torch")
    r = _chains([4, 33, 64], seed=43, t_end=0.2)
    dev = torch.device("cuda")
    d = W.RaggedBatch(r.name, r.rhs, *(torch.from_numpy(x).to(dev) for x in (r.y_off, r.p_off, r.y0, r.params,
                                                                               r.t0, r.t_end)),
                      r.tol, r.dt_min, r.dt_max, r.seed)
    _, sol = engine.bdf_solve_mixed(None, d)
    ref = _oracle_ragged(oracle, r)
    np.testing.assert_array_equal(sol.y.cpu().numpy().view(np.int64), ref["y"].view(np.int64))
    np.testing.assert_array_equal(sol.accepted.cpu().numpy(), ref["accepted"])


def test_ragged_failures_retire_only_their_system(engine, oracle):
    r = _chains([3, 20, 40], seed=44, t_end=0.2)
    r.t_end = r.t_end.copy()
    r.t_end[1] = -1.0   # ends before it starts
    r.y0 = r.y0.copy()
    r.y0[r.y_off[2]] = np.nan
    _, sol = engine.bdf_solve_mixed(None, r, max_steps=500)
    ref = _oracle_ragged(oracle, r, max_steps=500)
    assert sol.status[0] == 0 and sol.status[1] == 5 and sol.status[2] != 0
    np.testing.assert_array_equal(sol.status, ref["status"])
    assert sol.code == 5


def test_mixed_dense_output_matches_oracle_paths(engine, oracle):
    """bacon_bdf_solve_mixed_dense: every item of both parts, packed.  The
    ragged chains' states go to one flat stream with value offsets (items x
    each chain's own dimension); chains and Robertson systems match the
    oracle's per-system paths bit for bit, and the final states equal the
    plain mixed solve's."""
    r = _chains(MASSES, seed=35, t_end=0.3)
    rob = W.robertson(n=48, seed=36)
    rob.t_end = np.full(rob.n, 10.0)
    us, rs = engine.bdf_solve_mixed(rob, r, dense=True)
    assert us.code == 0 and rs.code == 0
    off, voff = np.asarray(rs.traj_off), np.asarray(rs.traj_voff)
    dims = np.diff(r.y_off)
    np.testing.assert_array_equal(np.diff(off), rs.accepted)
    np.testing.assert_array_equal(np.diff(voff), rs.accepted * dims)
    cfg = oracle.bdf_cfg(mode=oracle.BDF_CORRECTED, dyn_dim=True, tol=r.tol, dt_min=r.dt_min, dt_max=r.dt_max)
    for i in range(r.n):
        y0, p = r.system(i)
        path = oracle.bdf_solve_one(cfg, r.rhs, y0, r.t0[i], r.t_end[i], params=p, traj_cap=100000)
        a, b = int(off[i]), int(off[i + 1])
        assert b - a == path.accepted
        np.testing.assert_array_equal(rs.traj_t[a:b], path.traj_t)
        np.testing.assert_array_equal(rs.traj_y[voff[i]:voff[i + 1]], path.traj_y.reshape(-1))
    rcfg = oracle.bdf_cfg(mode=oracle.BDF_CORRECTED, tol=rob.tol, dt_min=rob.dt_min, dt_max=rob.dt_max)
    uoff = np.asarray(us.traj_off)
    for i in range(0, rob.n, 5):
        path = oracle.bdf_solve_one(rcfg, rob.rhs, rob.y0[:, i], 0.0, 10.0, params=rob.params[:, i],
                                    traj_cap=100000)
        a, b = int(uoff[i]), int(uoff[i + 1])
        np.testing.assert_array_equal(us.traj_t[a:b], path.traj_t)
        np.testing.assert_array_equal(us.traj_y[a:b].reshape(-1), path.traj_y.reshape(-1))
    plain_u, plain_r = engine.bdf_solve_mixed(rob, r)
    np.testing.assert_array_equal(plain_r.y, rs.y)
    np.testing.assert_array_equal(plain_u.y, us.y)


def test_mixed_dense_capacity_short_reports_totals(engine):
    """With capacity 0 the call returns BACON_CAPACITY_EXCEEDED after the
    counting pass, with both totals and the offsets filled."""
    import ctypes
    from bacon_gb300 import _capi
    r = _chains([2, 5, 17], seed=37, t_end=0.2)
    rp = _capi.RaggedProblem()
    rp.n, rp.rhs = r.n, int(r.rhs)
    y_off, p_off = np.ascontiguousarray(r.y_off), np.ascontiguousarray(r.p_off)
    y0, prm = np.ascontiguousarray(r.y0), np.ascontiguousarray(r.params)
    t0, te = np.ascontiguousarray(r.t0), np.ascontiguousarray(r.t_end)
    rp.y_offsets, rp.p_offsets, rp.y0, rp.params = y_off.ctypes.data, p_off.ctypes.data, y0.ctypes.data, prm.ctypes.data
    rp.t0, rp.t_end = t0.ctypes.data, te.ctypes.data
    rp.tol, rp.dt_min, rp.dt_max = r.tol, r.dt_min, r.dt_max
    o = _capi.BdfOptions()
    o.method, o.mode, o.memory = 0, 1, 1
    yf, tf = np.zeros_like(y0), np.zeros(r.n)
    acc, rej, st = np.zeros(r.n, np.int32), np.zeros(r.n, np.int32), np.zeros(r.n, np.int32)
    rres = _capi.RaggedResult()
    rres.y_final, rres.t_final = yf.ctypes.data, tf.ctypes.data
    rres.accepted, rres.rejected, rres.status = acc.ctypes.data, rej.ctypes.data, st.ctypes.data
    off, voff = np.zeros(r.n + 1, np.int64), np.zeros(r.n + 1, np.int64)
    gd = _capi.RaggedDenseOutput()
    gd.capacity, gd.value_capacity, gd.t, gd.y = 0, 0, None, None
    gd.offsets, gd.value_offsets = off.ctypes.data, voff.ctypes.data
    code = _capi.load().bacon_bdf_solve_mixed_dense(engine.default_context().handle, None, ctypes.byref(rp),
                                                    ctypes.byref(o), None, ctypes.byref(rres), None,
                                                    ctypes.byref(gd))
    assert code == 17
    assert gd.total == acc.sum() == off[-1] > 0
    assert gd.total_values == (acc * np.diff(y_off)).sum() == voff[-1]


def test_mixed_dense_device_arrays_match_host(engine):
    """The mixed dense output with every array on the device equals the
    host-memory call's."""
    import torch
    r = _chains([3, 16, 33, 64], seed=38, t_end=0.2)
    rob = W.robertson(n=40, seed=39)
    rob.t_end = np.full(rob.n, 5.0)
    hu, hr = engine.bdf_solve_mixed(rob, r, dense=True)
    dev = torch.device("cuda")
    td = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    dr = W.RaggedBatch(r.name, r.rhs, td(r.y_off), td(r.p_off), td(r.y0), td(r.params), td(r.t0), td(r.t_end),
                       r.tol, r.dt_min, r.dt_max, r.seed)
    du = W.Batch(rob.name, rob.rhs, td(rob.y0), td(rob.params), td(rob.t0), td(rob.t_end), rob.tol, rob.dt_min,
                 rob.dt_max, rob.seed)
    us, rs = engine.bdf_solve_mixed(du, dr, dense=True)
    for a, b in ((rs.traj_off, hr.traj_off), (rs.traj_voff, hr.traj_voff), (rs.traj_t, hr.traj_t),
                 (rs.traj_y, hr.traj_y), (us.traj_off, hu.traj_off), (us.traj_t, hu.traj_t),
                 (us.traj_y, hu.traj_y)):
        np.testing.assert_array_equal(a.cpu().numpy(), b)


def test_mixed_dense_uniform_part_only(engine, oracle):
    """The mixed dense call with no ragged part records the uniform part's
    items exactly as bacon_bdf_solve_dense does."""
    rob = W.robertson(n=24, seed=44)
    rob.t_end = np.full(rob.n, 3.0)
    us, rs = engine.bdf_solve_mixed(rob, None, dense=True)
    assert rs is None and us.code == 0
    ref = engine.bdf_solve(rob.y0, rob.params, 0.0, 3.0, rhs=rob.rhs, tol=rob.tol, dt_min=rob.dt_min,
                           dt_max=rob.dt_max, dense=True)
    np.testing.assert_array_equal(np.asarray(us.traj_off), np.asarray(ref.traj_off))
    np.testing.assert_array_equal(us.traj_t, ref.traj_t)
    np.testing.assert_array_equal(us.traj_y, ref.traj_y)
