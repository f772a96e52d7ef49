"""The allocation-free entry point, bacon_rk_solve_noalloc, called through the
C ABI.

It serves callers that cannot allocate device memory (their memory pool owns
the GPU, or they hold only a stream and device pointers), so it keeps its
scratch in a fixed device array inside the library.  These tests compare it
with the regular entry point, bacon_rk_solve, bit for bit (the tolerance the
other GPU tests use), on two calls in a row: the shared array keeps the
previous call's contents, and each call must reset what has to start at zero.
The file name puts it last in pytest's collection order.
"""
import ctypes

import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.device("cuda"))


def _noalloc(E, L, prob, layout, n, dim, systems_per_warp=0):
    import torch
    out = E.alloc_outputs(dim, n, device=True)
    res = E.make_result(out)
    opts = E.rk_options(layout=layout, memory=E.MEM_DEVICE, systems_per_warp=systems_per_warp)
    torch.cuda.synchronize()
    code = L.bacon_rk_solve_noalloc(ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), None)
    return code, out


def _assert_same(out, ref):
    """Bit-for-bit equality (NaN states of failed systems included)."""
    import torch
    for k, v in (("y", ref.y), ("t", ref.t), ("accepted", ref.accepted), ("rejected", ref.rejected),
                 ("status", ref.status)):
        a, b = out[k], v
        if a.dtype == torch.float64:
            a, b = a.view(torch.int64), b.view(torch.int64)
        assert torch.equal(a, b), k


def test_noalloc_matches_regular_entry_point_twice(engine):
    """Per-system end times (longest-first order in the fixed scratch)."""
    from bacon_gb300 import _capi
    L = _capi.load()
    b = W.lorenz(n=1 << 20).subset(np.arange(0, 1 << 20, 64))  # 16,384 systems, T ~ U[1, 20]
    y0, prm, t0, te = (_device(x) for x in (b.y0, b.params, b.t0, b.t_end))
    ref = engine.rk_solve(y0, prm, t0, te, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2)
    assert ref.code == 0
    prob = engine.make_problem(y0, prm, t0, te, b.tol, b.dt_min, b.dt_max, b.rhs)
    for _ in range(2):
        code, out = _noalloc(engine, L, prob, 2, b.n, 3)
        assert code == 0
        _assert_same(out, ref)


def test_noalloc_failures_and_index_order(engine):
    """Scalar times (index order) and per-system failures: the return code is
    the lowest failing system's status, also on the second call."""
    from bacon_gb300 import _capi
    L = _capi.load()
    b = W.van_der_pol(n=2048, seed=13)
    b.y0 = b.y0.copy()
    b.y0[0, 40] = np.nan
    b.params = b.params.copy()
    b.params[0, 77] = 1e6
    y0, prm = _device(b.y0), _device(b.params)
    ref = engine.rk_solve(y0, prm, 0.0, 10.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2, max_attempts=3000)
    assert ref.code != 0
    prob = engine.make_problem(y0, prm, 0.0, 10.0, b.tol, b.dt_min, b.dt_max, b.rhs)
    opts = engine.rk_options(layout=2, memory=engine.MEM_DEVICE, max_attempts=3000)
    import torch
    for _ in range(2):
        out = engine.alloc_outputs(2, b.n, device=True)
        res = engine.make_result(out)
        torch.cuda.synchronize()
        code = L.bacon_rk_solve_noalloc(ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), None)
        assert code == ref.code
        _assert_same(out, ref)


def test_noalloc_rejects_oversized_batch_and_host_memory(engine):
    from bacon_gb300 import _capi
    L = _capi.load()
    n = (1 << 20) + 1
    y0 = np.zeros((2, n))
    prob = engine.make_problem(y0, np.ones((1, n)), 0.0, 1.0, 1e-6, 1e-6, 0.1, W.RHS_VDP)
    out = engine.alloc_outputs(2, n, device=False)
    res = engine.make_result(out)
    opts = engine.rk_options(layout=2, memory=engine.MEM_DEVICE)
    assert L.bacon_rk_solve_noalloc(ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), None) == 17
    opts = engine.rk_options(layout=2, memory=engine.MEM_HOST)
    assert L.bacon_rk_solve_noalloc(ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), None) == 15


def test_noalloc_zero_size_warm_up_then_no_device_memory_change(engine):
    """A call with n == 0 is the documented warm-up (it places the scratch
    array and the kernel on the device).  After it, a real call leaves the
    device's free memory exactly as it was: the entry point allocates
    nothing."""
    import torch
    from bacon_gb300 import _capi
    L = _capi.load()
    b = W.van_der_pol(n=4096, seed=17)
    y0, prm = _device(b.y0), _device(b.params)
    empty = engine.make_problem(y0[:, :0], prm[:, :0], 0.0, 10.0, b.tol, b.dt_min, b.dt_max, b.rhs)
    opts = engine.rk_options(layout=2, memory=engine.MEM_DEVICE)
    res0 = engine.make_result(engine.alloc_outputs(2, 0, device=True))
    assert L.bacon_rk_solve_noalloc(ctypes.byref(empty), ctypes.byref(opts), ctypes.byref(res0), None) == 0
    ref = engine.rk_solve(y0, prm, 0.0, 10.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, layout=2)
    prob = engine.make_problem(y0, prm, 0.0, 10.0, b.tol, b.dt_min, b.dt_max, b.rhs)
    outs = [engine.alloc_outputs(2, b.n, device=True) for _ in range(2)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for out in outs:
        res = engine.make_result(out)
        assert L.bacon_rk_solve_noalloc(ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    for out in outs:
        _assert_same(out, ref)



def test_noalloc_systems_per_warp(engine):
    """Eight systems per warp through the allocation-free entry point: the
    same results as the regular entry point at 32."""
    from bacon_gb300 import _capi
    L = _capi.load()
    b = W.van_der_pol(n=4096, seed=93)
    y0, prm, t0, te = (_device(x) for x in (b.y0, b.params, b.t0, b.t_end))
    ref = engine.rk_solve(y0, prm, t0, te, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, layout=2)
    prob = engine.make_problem(y0, prm, t0, te, b.tol, b.dt_min, b.dt_max, b.rhs)
    code, out = _noalloc(engine, L, prob, 2, b.n, 2, systems_per_warp=8)
    assert code == 0
    _assert_same(out, ref)
