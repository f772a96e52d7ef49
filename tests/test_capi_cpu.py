"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and the native builder reproduces the reference builder's error
behaviour (src/ivp/rk.rs:168-256).  No GPU work is issued."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bacon_gb300.h")


@pytest.fixture(scope="module")
def capi():
    from bacon_gb300 import _capi, build_ext
    if not os.path.exists(_capi.LIB_PATH):
        build_ext.build()
    return _capi


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bacon_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(capi):
    L = capi.load()
    names = _declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), f"{name} declared in include/bacon_gb300.h but not exported"
    assert set(names) == set(capi.SIGNATURES), "ctypes signature table out of sync with the header"


def _builder(capi, kind=0, dim=1):
    L = capi.load()
    h = ctypes.c_void_p()
    assert L.bacon_builder_new(kind, dim, ctypes.byref(h)) == 0
    return L, h


def test_builder_tolerance_and_dt_validation(capi):
    L, h = _builder(capi)
    assert L.bacon_builder_with_tolerance(h, 0.0) == 3          # ToleranceOOB
    assert L.bacon_builder_with_tolerance(h, -1.0) == 3
    assert L.bacon_builder_with_tolerance(h, 1e-6) == 0
    assert L.bacon_builder_with_maximum_dt(h, 0.0) == 4         # TimeDeltaOOB
    assert L.bacon_builder_with_minimum_dt(h, -1e-3) == 4
    L.bacon_builder_free(h)


def test_builder_dt_cross_clamp(capi):
    """with_maximum_dt lowers a larger minimum; with_minimum_dt raises a
    smaller maximum (rk.rs:179-210)."""
    L, h = _builder(capi)
    y = np.zeros(1)
    assert L.bacon_builder_with_minimum_dt(h, 0.5) == 0
    assert L.bacon_builder_with_maximum_dt(h, 0.1) == 0
    for f, v in ((L.bacon_builder_with_tolerance, 1e-6), (L.bacon_builder_with_initial_time, 0.0),
                 (L.bacon_builder_with_ending_time, 1.0)):
        assert f(h, v) == 0
    assert L.bacon_builder_with_initial_conditions(h, y.ctypes.data_as(capi.DP), 1) == 0
    assert L.bacon_builder_with_derivative(h, 0, None, 0) == 0
    p = capi.Problem()
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 0
    assert p.dt_min == 0.1 and p.dt_max == 0.1
    L.bacon_builder_free(h)

    L, h = _builder(capi)
    assert L.bacon_builder_with_maximum_dt(h, 0.1) == 0
    assert L.bacon_builder_with_minimum_dt(h, 0.5) == 0
    for f, v in ((L.bacon_builder_with_tolerance, 1e-6), (L.bacon_builder_with_initial_time, 0.0),
                 (L.bacon_builder_with_ending_time, 1.0)):
        assert f(h, v) == 0
    assert L.bacon_builder_with_initial_conditions(h, y.ctypes.data_as(capi.DP), 1) == 0
    assert L.bacon_builder_with_derivative(h, 0, None, 0) == 0
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 0
    assert p.dt_min == 0.5 and p.dt_max == 0.5
    L.bacon_builder_free(h)


def test_builder_time_order(capi):
    L, h = _builder(capi)
    assert L.bacon_builder_with_initial_time(h, 1.0) == 0
    assert L.bacon_builder_with_ending_time(h, 1.0) == 5        # TimeEndOOB
    L.bacon_builder_free(h)
    L, h = _builder(capi)
    assert L.bacon_builder_with_ending_time(h, 1.0) == 0
    assert L.bacon_builder_with_initial_time(h, 2.0) == 6       # TimeStartOOB
    L.bacon_builder_free(h)


def test_builder_missing_parameters(capi):
    L, h = _builder(capi)
    p = capi.Problem()
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 1     # MissingParameters
    assert L.bacon_builder_with_tolerance(h, 1e-6) == 0
    assert L.bacon_builder_with_minimum_dt(h, 1e-6) == 0
    assert L.bacon_builder_with_maximum_dt(h, 0.1) == 0
    assert L.bacon_builder_with_initial_time(h, 0.0) == 0
    assert L.bacon_builder_with_ending_time(h, 1.0) == 0
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 1     # no state, no derivative
    y = np.ones(1)
    assert L.bacon_builder_with_initial_conditions(h, y.ctypes.data_as(capi.DP), 1) == 0
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 1     # no derivative
    assert L.bacon_builder_with_derivative(h, 1, None, 0) == 0
    assert L.bacon_builder_problem(h, ctypes.byref(p)) == 0
    assert L.bacon_last_error() is not None
    L.bacon_builder_free(h)


def test_builder_per_system_end_times(capi):
    L, h = _builder(capi)
    assert L.bacon_builder_with_initial_time(h, 0.0) == 0
    ends = np.array([1.0, 2.0, -1.0])
    assert L.bacon_builder_with_ending_times(h, ends.ctypes.data_as(capi.DP), 3) == 5
    L.bacon_builder_free(h)


def test_validate_problem(capi):
    L = capi.load()
    y = np.zeros((2, 4))
    p = capi.Problem()
    p.n, p.dim, p.rhs, p.n_params = 4, 2, 5, 1
    prm = np.ones((1, 4))
    p.y0, p.params = y.ctypes.data, prm.ctypes.data
    p.t0_scalar, p.t_end_scalar, p.tol, p.dt_min, p.dt_max = 0.0, 1.0, 1e-6, 1e-6, 0.1
    assert L.bacon_rk_validate(ctypes.byref(p)) == 0
    p.tol = 0.0
    assert L.bacon_rk_validate(ctypes.byref(p)) == 3
    p.tol, p.dt_min = 1e-6, 0.0
    assert L.bacon_rk_validate(ctypes.byref(p)) == 4
    p.dt_min, p.t_end_scalar = 1e-6, 0.0
    assert L.bacon_rk_validate(ctypes.byref(p)) == 5
    p.t_end_scalar, p.dim = 1.0, 3
    assert L.bacon_rk_validate(ctypes.byref(p)) == 15           # VdP is 2-dimensional
    p.dim, p.n_params = 2, 0
    assert L.bacon_rk_validate(ctypes.byref(p)) == 15           # mu missing


def test_python_builder_errors(capi):
    from bacon_gb300.ivp import IVPError, RungeKutta45
    with pytest.raises(IVPError) as e:
        RungeKutta45.new(1).with_tolerance(-1.0)
    assert e.value.variant == "ToleranceOOB"
    with pytest.raises(IVPError) as e:
        RungeKutta45.new(1).with_initial_time(3.0).with_ending_time(2.0)
    assert e.value.variant == "TimeEndOOB"
    with pytest.raises(IVPError) as e:
        RungeKutta45.new(1).with_dt_min(1e-3).with_dt_max(0.1).with_tolerance(1e-4).solve(())
    assert e.value.variant == "MissingParameters"
    b = RungeKutta45.new(2).with_start(0.0).with_end(1.0).build()
    assert b.dim() == 2


def test_ragged_validation_without_gpu():
    """Ragged batches are checked on the host before any device work."""
    import ctypes

    from bacon_gb300 import _capi
    from bacon_gb300 import workloads as W

    lib = _capi.load()
    r = W.ragged_spring_chains(n=3, seed=1)
    keep = []

    def check(y_off=None, p_off=None, rhs=W.RHS_CHAIN, tol=1e-6, dt_min=1e-12):
        y_off = np.ascontiguousarray(r.y_off if y_off is None else y_off, dtype=np.int64)
        p_off = np.ascontiguousarray(r.p_off if p_off is None else p_off, dtype=np.int64)
        keep.extend([y_off, p_off])
        rp = _capi.RaggedProblem()
        rp.n = len(y_off) - 1
        rp.rhs = rhs
        rp.y_offsets, rp.p_offsets = y_off.ctypes.data, p_off.ctypes.data
        rp.y0, rp.params = r.y0.ctypes.data, r.params.ctypes.data
        rp.tol, rp.dt_min, rp.dt_max = tol, dt_min, 1.0
        return lib.bacon_ragged_validate(ctypes.byref(rp))

    assert check() == 0
    assert check(rhs=W.RHS_VDP) == 16
    assert check(tol=0.0) == 15
    assert check(dt_min=0.0) == 15
    assert check(y_off=[0, 3], p_off=[0, 2]) == 15          # odd dim
    assert check(y_off=[0, 130], p_off=[0, 66]) == 15       # dim above 128
    assert check(y_off=[0, 0], p_off=[0, 1]) == 15          # dim 0
    assert check(y_off=[0, 4], p_off=[0, 2]) == 15          # chain of 2 masses takes 3 params
    assert check(y_off=[1, 5], p_off=[0, 3]) == 15          # offsets must start at 0
    assert check(y_off=[0, 128], p_off=[0, 65]) == 0        # 64 masses
    o = _capi.BdfOptions()
    assert lib.bacon_bdf_solve_mixed(None, None, None, ctypes.byref(o), None, None) == 15
