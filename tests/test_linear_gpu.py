"""Batched RKF45 on y' = A y with one shared A (the GEMM right-hand side).

FP64_EXACT stage GEMMs sum every matvec in the CPU oracle's order, so the
lock-step engine is bit-identical to the oracle's per-system solve; all
modes are checked against the exact solution Q exp(-Lambda t) Q^T y0."""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _solve(E, b, precision=0, layout=2):
    return E.rk_solve(b.y0, None, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                      layout=layout, precision=precision, shared=b.extra["A"])


@pytest.mark.parametrize("dim", [64, 256])
def test_linear_exact_matches_oracle(engine, oracle, dim):
    b = W.linear_shared(n=96, dim=dim, seed=21)
    sol = _solve(engine, b)
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    ref = oracle.rk_solve_batch(cfg, b.rhs, b.y0, None, b.t0, b.t_end, shared=b.extra["A"])
    np.testing.assert_array_equal(sol.accepted, ref["accepted"])
    np.testing.assert_array_equal(sol.rejected, ref["rejected"])
    np.testing.assert_array_equal(sol.t, ref["t"])
    np.testing.assert_array_equal(sol.y, ref["y"])


def test_linear_fma_close_to_exact_solution(engine):
    b = W.linear_shared(n=512, dim=256, seed=22)
    ex = b.extra["exact"](5.0)
    for prec in (0, 1):
        sol = _solve(engine, b, precision=prec)
        assert (sol.status == 0).all()
        assert np.abs(sol.y - ex).max() < 1e-7


@pytest.mark.parametrize("dim", [128, 256])
def test_linear_tensor_core_split(engine, dim):
    """tcgen05 stage GEMM with 5 x 8-bit bf16 slices: each product is
    within ~2^-39 relative, so the engine reaches the FP64 engine's accuracy
    against the exact solution.  The embedded error estimate is ~1e9 times
    smaller than |K| here (tol 1e-8, |A y| ~ 10), so it carries a ~1e-3
    relative perturbation, and with the reference's safety factor 1 (a
    rejection lands the next attempt at err ~ tol) that can flip an accept
    decision.  Measured: accepted counts equal the FP64 engine's on 100 %
    (dim 128) and 99.7 % (dim 256) of systems, off by at most one step, and
    final states within 1.5e-9 of it.  Six 6-bit slices (~2^-35) had
    flipped 11 % at dim 256."""
    b = W.linear_shared(n=1024, dim=dim, seed=23)
    ex = b.extra["exact"](5.0)
    fp = _solve(engine, b, precision=0)
    fma = _solve(engine, b, precision=1)
    tc = _solve(engine, b, precision=engine.TC_SPLIT)
    assert (tc.status == 0).all()
    assert np.abs(tc.y - ex).max() < 1e-7
    same_tc = np.mean(tc.accepted == fp.accepted)
    same_fma = np.mean(fma.accepted == fp.accepted)
    assert same_fma >= 0.99, same_fma
    assert same_tc >= 0.97, (same_tc, same_fma)
    assert np.abs(tc.accepted.astype(np.int64) - fp.accepted).max() <= 2
    # different accept decisions on a few systems move their states by ~tol
    assert np.abs(tc.y - fp.y).max() < 2e-8


def _exact_at(b, t_end):
    """Q diag(exp(-lambda t_i)) Q^T y0_i for each system's own end time."""
    q, lam = b.extra["Q"], b.extra["lambda"]
    z = q.T @ b.y0
    return q @ (np.exp(-lam[:, None] * t_end[None, :]) * z)


def test_linear_ragged_batch_end_times_exact(engine, oracle):
    """37 systems (the control kernel serves four per warp, so the last warp
    is partly empty) with per-system end times, so systems stop in different
    rounds: bit-identical to the oracle."""
    b = W.linear_shared(n=37, dim=64, seed=31)
    t_end = np.random.default_rng(5).uniform(1.0, 5.0, 37)
    sol = engine.rk_solve(b.y0, None, b.t0, t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, precision=0, shared=b.extra["A"])
    assert sol.code == 0
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    ref = oracle.rk_solve_batch(cfg, b.rhs, b.y0, None, b.t0, t_end, shared=b.extra["A"])
    np.testing.assert_array_equal(sol.accepted, ref["accepted"])
    np.testing.assert_array_equal(sol.rejected, ref["rejected"])
    np.testing.assert_array_equal(sol.t, ref["t"])
    np.testing.assert_array_equal(sol.y, ref["y"])


def test_linear_tensor_core_ragged_tiles(engine):
    """1,000 systems fill 15 tiles of 64 and leave the 16th with 40; per-system
    end times retire systems from tiles in different rounds, so tiles run
    partly live and, at the end, are skipped by both the producer warp and
    the epilogue warps.  Every system ends at its own t_end within the
    split's accuracy of the exact solution."""
    b = W.linear_shared(n=1000, dim=128, seed=32)
    t_end = np.random.default_rng(6).uniform(1.0, 5.0, 1000)
    tc = engine.rk_solve(b.y0, None, b.t0, t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                         layout=2, precision=engine.TC_SPLIT, shared=b.extra["A"])
    assert tc.code == 0 and (tc.status == 0).all()
    # the last step is clamped to end - t, so t lands on t_end to rounding
    assert (tc.t >= t_end).all() and np.allclose(tc.t, t_end, rtol=1e-12, atol=0.0)
    assert np.abs(tc.y - _exact_at(b, tc.t)).max() < 1e-7


def test_linear_tensor_core_wait_runs_out_and_context_recovers(engine):
    """Failure path of the tensor-core stage GEMM, without a GPU fault: the
    context's fault-injection hook makes the producer withhold the
    accumulator hand-off, so the epilogue's bounded mbarrier wait runs out
    (~10 ms), the kernel sets its error flag and returns, and the solve
    reports BACON_CUDA_ERROR.  With the hook off, the same context then
    solves the batch bit-identically to a solve that never failed."""
    from bacon_gb300 import _capi
    b = W.linear_shared(n=64, dim=128, seed=33)
    ctx = engine.Context(0)
    ref = _solve(engine, b, precision=engine.TC_SPLIT)
    lib = _capi.load()
    assert lib.bacon_ctx_set_fault_injection(ctx.handle, 1) == 0
    with pytest.raises(engine.IVPError) as err:
        engine.rk_solve(b.y0, None, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                        layout=2, precision=engine.TC_SPLIT, shared=b.extra["A"], ctx=ctx)
    assert "bounded mbarrier wait" in str(err.value)
    assert lib.bacon_ctx_set_fault_injection(ctx.handle, 0) == 0
    assert lib.bacon_ctx_set_fault_injection(ctx.handle, 7) != 0
    again = engine.rk_solve(b.y0, None, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                            layout=2, precision=engine.TC_SPLIT, shared=b.extra["A"], ctx=ctx)
    assert again.code == 0
    np.testing.assert_array_equal(again.y, ref.y)
    np.testing.assert_array_equal(again.accepted, ref.accepted)
