"""FP32-stage mode (BACON_FP32_COMP): float-float stages, FP64 control.

It is not bit-identical to the reference's FP64 arithmetic, so it is judged
by final-state error against an FP64 reference at rtol 1e-12 (scipy DOP853):
it must be as accurate as the exact FP64 engine at the same tolerance.
"""
import numpy as np
import pytest

from bacon_gb300 import accuracy as A
from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _solve(E, b, precision, layout=2, **kw):
    return E.rk_solve(b.y0, b.params, b.t0, b.t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min,
                      dt_max=b.dt_max, layout=layout, precision=precision, **kw)


@pytest.mark.parametrize("make", [lambda: W.van_der_pol(n=256, seed=71),
                                  lambda: W.lotka_volterra(n=256, seed=72)])
def test_fp32comp_accuracy_matches_fp64(engine, make):
    b = make()
    ref = A.reference_final_states(b)
    ex = _solve(engine, b, engine.FP64_EXACT)
    ff = _solve(engine, b, engine.FP32_COMP)
    assert (ff.status == 0).all() and (ex.status == 0).all()
    e_ex = A.final_state_error(ex.y, ref)
    e_ff = A.final_state_error(ff.y, ref)
    assert e_ff["abs_median"] <= 3.0 * e_ex["abs_median"] + 1e-9, (e_ff, e_ex)
    assert e_ff["abs_max"] <= 3.0 * e_ex["abs_max"] + 1e-9, (e_ff, e_ex)
    # same step-count regime as the FP64 engine
    assert abs(np.mean(ff.accepted) / np.mean(ex.accepted) - 1.0) < 0.05


def test_fp32comp_lorenz_short_horizon(engine):
    b = W.lorenz(n=256, seed=73)
    b.t_end = np.minimum(b.t_end, 2.0)
    ref = A.reference_final_states(b)
    ex = _solve(engine, b, engine.FP64_EXACT)
    ff = _solve(engine, b, engine.FP32_COMP)
    assert (ff.status == 0).all()
    e_ex = A.final_state_error(ex.y, ref)
    e_ff = A.final_state_error(ff.y, ref)
    assert e_ff["abs_median"] <= 3.0 * e_ex["abs_median"] + 1e-9, (e_ff, e_ex)


def test_fp32comp_failures_retire_only_their_system(engine):
    b = W.van_der_pol(n=64, seed=74)
    b.y0 = b.y0.copy()
    b.y0[1, 3] = np.nan
    b.t_end = b.t_end.copy()
    b.t_end[9] = -1.0
    sol = _solve(engine, b, engine.FP32_COMP, max_attempts=2000)
    assert sol.status[3] == 13 and sol.status[9] == 5
    ok = np.ones(64, bool)
    ok[[3, 9]] = False
    assert (sol.status[ok] == 0).all()
    assert sol.code == 13  # lowest failing index is system 3


@pytest.mark.parametrize("layout", [0, 1])
def test_fp32comp_other_layouts_run(engine, oracle, layout):
    """The stale-stage (as_compiled) and literal readings run in this mode too
    and end with the same statuses as the exact engine on Van der Pol."""
    b = W.van_der_pol(n=128, seed=75)
    ex = _solve(engine, b, engine.FP64_EXACT, layout=layout, max_attempts=20000)
    ff = _solve(engine, b, engine.FP32_COMP, layout=layout, max_attempts=20000)
    assert np.mean(ex.status == ff.status) >= 0.9
