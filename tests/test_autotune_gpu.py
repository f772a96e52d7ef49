"""Autotuner: picks a launch shape on the caller's batch, caches it, and the
cached shape gives the same (bit-identical) results."""
import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_autotune_caches_and_keeps_results(engine):
    b = W.lorenz(n=1 << 20).subset(np.arange(0, 1 << 20, 32))  # 32768 systems
    kw = dict(rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, layout=2)
    before = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, **kw)
    block, bps = engine.rk_autotune(b.y0, b.params, b.t0, b.t_end, **kw)
    assert block in (64, 128, 256) and 1 <= bps <= 4
    after = engine.rk_solve(b.y0, b.params, b.t0, b.t_end, **kw)
    np.testing.assert_array_equal(after.y, before.y)
    np.testing.assert_array_equal(after.accepted, before.accepted)
