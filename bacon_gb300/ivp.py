"""Host-side mirror of bacon-sci's IVP builder API, batched.

Mirrors the IVPSolver trait (src/ivp.rs:134-190) as implemented for
RungeKutta45 / RungeKutta23 (src/ivp/rk.rs:118-344, :561, :656): the same
method names, argument meaning, validation order and error variants, with the
checks themselves done by the native builder in the C ABI.  A builder may
describe one system (``with_initial_conditions_slice``) or a batch
(``with_initial_conditions_batch``); ``solve`` runs every system on the GPU.

The README spelling of the API (README.md:23-47: ``with_dt_min``,
``with_dt_max``, ``with_start``, ``with_end``, ``build``, ``solve_ivp``) is
accepted as aliases.

Differences from the reference, all forced by running on a GPU:
  * ``with_derivative`` takes a registry right-hand side (``Rhs``) and
    per-system parameters instead of a Rust closure;
  * ``solve(data)`` ignores ``data`` (parameters travel with the derivative);
  * ``layout`` selects the Butcher-matrix reading: AS_COMPILED (default) is
    what the compiled reference executes, see include/bacon_gb300.h.
"""
from __future__ import annotations

import ctypes
from enum import IntEnum

import numpy as np

from . import _capi
from .engine import (AS_COMPILED, AS_WRITTEN, FEHLBERG, FP32_COMP, FP64_EXACT, FP64_FMA, RK23, RK45,
                     Context, IVPError, Solution, check, rk_solve)

__all__ = ["Rhs", "RungeKutta45", "RungeKutta23", "BDF6", "BDF2", "Adams5", "Adams3", "Euler", "IVPError",
           "IVPIterator", "AS_COMPILED",
           "AS_WRITTEN", "FEHLBERG", "FP64_EXACT", "FP64_FMA", "FP32_COMP"]


class Rhs(IntEnum):
    EXP = 0
    DECAY = 1
    QUADRATIC = 2
    SINE = 3
    HARMONIC = 4
    VDP = 5
    LORENZ = 6
    LOTKA = 7
    ROBERTSON = 8
    CHAIN = 9
    LINEAR = 10


class IVPIterator:
    """Result of ``solve``: iterates over the (t, y) path of a single system
    like the reference's IVPIterator (src/ivp.rs:192-239), and exposes the
    whole batch through ``batch``."""

    def __init__(self, sol: Solution, n: int, dim: int):
        self.batch = sol
        self.n = n
        self.dim = dim

    def path(self, i: int = 0):
        sol = self.batch
        if sol.traj_t is None:
            raise ValueError("solve(record_path=False) keeps no path")
        k = int(sol.accepted[i])
        return [(float(sol.traj_t[i, j]), np.array(sol.traj_y[i, j])) for j in range(k)]

    def __iter__(self):
        if self.n != 1:
            raise ValueError("iterate a batch through .batch or .path(i)")
        yield from self.path(0)
        st = int(self.batch.status[0])
        if st != 0:
            raise IVPError(st)

    def collect_vec(self, i: int = 0):
        """Every accepted (t, y) of system i, or the error it ended with
        (src/ivp.rs:209-211)."""
        st = int(self.batch.status[i])
        if st != 0:
            raise IVPError(st, f"system {i}")
        return self.path(i)


class _RkBuilder:
    KIND = 0
    METHOD = RK45

    def __init__(self, handle: ctypes.c_void_p, dim: int, dyn: bool):
        self._h = handle
        self._dim = dim
        self._dyn = dyn
        self._lib = _capi.load()

    def __del__(self):
        try:
            if self._h:
                self._lib.bacon_builder_free(self._h)
        except Exception:
            pass

    # -- constructors (IVPSolver::new / new_dyn) ----------------------------
    @classmethod
    def new(cls, dim: int = 1):
        lib = _capi.load()
        h = ctypes.c_void_p()
        check(lib.bacon_builder_new(cls.KIND, int(dim), ctypes.byref(h)))
        return cls(h, int(dim), False)

    @classmethod
    def new_dyn(cls, size: int):
        lib = _capi.load()
        h = ctypes.c_void_p()
        check(lib.bacon_builder_new_dyn(cls.KIND, int(size), ctypes.byref(h)))
        return cls(h, int(size), True)

    def dim(self) -> int:
        return self._dim

    # -- builder methods ------------------------------------------------------
    def with_tolerance(self, tol: float):
        check(self._lib.bacon_builder_with_tolerance(self._h, float(tol)))
        return self

    def with_maximum_dt(self, max_dt: float):
        check(self._lib.bacon_builder_with_maximum_dt(self._h, float(max_dt)))
        return self

    def with_minimum_dt(self, min_dt: float):
        check(self._lib.bacon_builder_with_minimum_dt(self._h, float(min_dt)))
        return self

    def with_initial_time(self, initial: float):
        check(self._lib.bacon_builder_with_initial_time(self._h, float(initial)))
        return self

    def with_ending_time(self, ending: float):
        check(self._lib.bacon_builder_with_ending_time(self._h, float(ending)))
        return self

    def with_ending_times(self, ending):
        """Batched extension: one end time per system."""
        a = np.ascontiguousarray(ending, dtype=np.float64).reshape(-1)
        check(self._lib.bacon_builder_with_ending_times(self._h, a.ctypes.data_as(_capi.DP), a.shape[0]))
        return self

    def with_initial_conditions_slice(self, start):
        y = np.ascontiguousarray(start, dtype=np.float64).reshape(-1)
        if y.shape[0] != self._dim:
            raise ValueError(f"initial conditions have {y.shape[0]} entries, the solver dimension is {self._dim}")
        return self._set_y0(y.reshape(self._dim, 1))

    with_initial_conditions = with_initial_conditions_slice

    def with_initial_conditions_batch(self, start):
        """Batched initial conditions, shape (n, dim)."""
        y = np.asarray(start, dtype=np.float64)
        if y.ndim != 2 or y.shape[1] != self._dim:
            raise ValueError("batched initial conditions must have shape (n, dim)")
        return self._set_y0(np.ascontiguousarray(y.T))

    def _set_y0(self, soa):
        self._n = soa.shape[1]
        check(self._lib.bacon_builder_with_initial_conditions(self._h, soa.ctypes.data_as(_capi.DP), self._n))
        return self

    def with_derivative(self, derivative, params=None):
        """``derivative``: an ``Rhs``; ``params``: (n_params,) shared by every
        system or (n, n_params) per system."""
        rhs = int(derivative)
        if params is None:
            check(self._lib.bacon_builder_with_derivative(self._h, rhs, None, 0))
            return self
        pa = np.asarray(params, dtype=np.float64)
        n = getattr(self, "_n", None)
        if n is None:
            raise ValueError("set initial conditions before per-system parameters")
        if pa.ndim == 1:
            pa = np.broadcast_to(pa, (n, pa.shape[0]))
        soa = np.ascontiguousarray(pa.T)
        check(self._lib.bacon_builder_with_derivative(self._h, rhs, soa.ctypes.data_as(_capi.DP), soa.shape[0]))
        return self

    # README.md:23-47 spelling.
    with_dt_min = with_minimum_dt
    with_dt_max = with_maximum_dt
    with_start = with_initial_time
    with_end = with_ending_time

    def build(self):
        return self

    def solve_ivp(self, derivative, data=None, params=None, **kw):
        return self.with_derivative(derivative, params).solve(data, **kw)

    def solve(self, data=None, *, layout: int = AS_COMPILED, precision: int = FP64_EXACT,
              max_attempts: int = 0, record_path: bool | None = None, path_capacity: int = 4096,
              ctx: Context | None = None) -> IVPIterator:
        """Run every system on the GPU (RungeKutta::solve + collect,
        src/ivp/rk.rs:249-343).  Raises IVPError for builder errors
        (MissingParameters, ...); per-system outcomes are in the result."""
        prob = _capi.Problem()
        check(self._lib.bacon_builder_problem(self._h, ctypes.byref(prob)))
        n, dim = int(prob.n), int(prob.dim)
        y0 = np.ctypeslib.as_array(ctypes.cast(prob.y0, _capi.DP), shape=(dim, n)).copy()
        params = None
        if prob.n_params:
            params = np.ctypeslib.as_array(ctypes.cast(prob.params, _capi.DP), shape=(prob.n_params, n)).copy()
        t_end = prob.t_end_scalar
        if prob.t_end:
            t_end = np.ctypeslib.as_array(ctypes.cast(prob.t_end, _capi.DP), shape=(n,)).copy()
        if record_path is None:
            record_path = n <= 64
        cap = path_capacity if record_path else 0
        while True:
            sol = rk_solve(y0, params, prob.t0_scalar, t_end, rhs=prob.rhs, tol=prob.tol,
                           dt_min=prob.dt_min, dt_max=prob.dt_max, method=self.METHOD, layout=layout,
                           precision=precision, max_attempts=max_attempts, traj_cap=cap, ctx=ctx,
                           dyn_dim=bool(prob.dyn_dim))
            if not cap or int(np.max(sol.accepted)) <= cap:
                break
            cap = int(np.max(sol.accepted)) + 1
        return IVPIterator(sol, n, dim)


class _BdfBuilder(_RkBuilder):
    """BDF builder (src/ivp/bdf.rs:124-332): same trait methods as the
    Runge-Kutta builders; ``solve`` runs the batched BDF kernels."""
    KIND = 2
    BDF_METHOD = 0

    def solve(self, data=None, *, mode: int | None = None, max_iter: int = 0, max_steps: int = 0,
              record_path: bool | None = None, path_capacity: int = 4096,
              ctx: Context | None = None, **_ignored) -> IVPIterator:
        """Run every system on the GPU.  ``mode``: BDF_CORRECTED (default) or
        BDF_AS_COMPILED (the reference's 0.16.2 behaviour)."""
        from .engine import BDF_CORRECTED, bdf_solve
        mode = BDF_CORRECTED if mode is None else mode
        prob = _capi.Problem()
        check(self._lib.bacon_builder_problem(self._h, ctypes.byref(prob)))
        n, dim = int(prob.n), int(prob.dim)
        y0 = np.ctypeslib.as_array(ctypes.cast(prob.y0, _capi.DP), shape=(dim, n)).copy()
        params = None
        if prob.n_params:
            params = np.ctypeslib.as_array(ctypes.cast(prob.params, _capi.DP), shape=(prob.n_params, n)).copy()
        t_end = prob.t_end_scalar
        if prob.t_end:
            t_end = np.ctypeslib.as_array(ctypes.cast(prob.t_end, _capi.DP), shape=(n,)).copy()
        if record_path is None:
            record_path = n <= 64
        cap = path_capacity if record_path else 0
        while True:
            sol = bdf_solve(y0, params, prob.t0_scalar, t_end, rhs=prob.rhs, tol=prob.tol,
                            dt_min=prob.dt_min, dt_max=prob.dt_max, method=self.BDF_METHOD, mode=mode,
                            max_iter=max_iter, max_steps=max_steps, traj_cap=cap, ctx=ctx,
                            dyn_dim=bool(prob.dyn_dim))
            if not cap or int(np.max(sol.accepted)) <= cap:
                break
            cap = int(np.max(sol.accepted)) + 1
        return IVPIterator(sol, n, dim)


class BDF6(_BdfBuilder):
    """Sixth-order BDF (src/ivp/bdf.rs:641-706)."""
    KIND = 2
    BDF_METHOD = 0


class BDF2(_BdfBuilder):
    """Second-order BDF (src/ivp/bdf.rs:708-762)."""
    KIND = 3
    BDF_METHOD = 1


class RungeKutta45(_RkBuilder):
    """Runge-Kutta-Fehlberg 4(5) (src/ivp/rk.rs:430-561)."""
    KIND = 0
    METHOD = RK45


class RungeKutta23(_RkBuilder):
    """Bogacki-Shampine 3(2) (src/ivp/rk.rs:563-656)."""
    KIND = 1
    METHOD = RK23


class _AdamsBuilder(_RkBuilder):
    """Adams predictor-corrector builder (src/ivp/adams.rs:134-334): the same
    trait methods and validation as the Runge-Kutta builders; ``solve`` runs
    the batched Adams kernel."""
    ORDER = 5

    def _problem(self):
        prob = _capi.Problem()
        check(self._lib.bacon_builder_problem(self._h, ctypes.byref(prob)))
        n, dim = int(prob.n), int(prob.dim)
        y0 = np.ctypeslib.as_array(ctypes.cast(prob.y0, _capi.DP), shape=(dim, n)).copy()
        params = None
        if prob.n_params:
            params = np.ctypeslib.as_array(ctypes.cast(prob.params, _capi.DP), shape=(prob.n_params, n)).copy()
        t_end = prob.t_end_scalar
        if prob.t_end:
            t_end = np.ctypeslib.as_array(ctypes.cast(prob.t_end, _capi.DP), shape=(n,)).copy()
        return prob, n, dim, y0, params, t_end

    def _run(self, prob, y0, params, t_end, cap, ctx, max_attempts):
        from .engine import adams_solve
        return adams_solve(y0, params, prob.t0_scalar, t_end, rhs=prob.rhs, tol=prob.tol, dt_min=prob.dt_min,
                           dt_max=prob.dt_max, order=self.ORDER, max_attempts=max_attempts, traj_cap=cap, ctx=ctx,
                           dyn_dim=bool(prob.dyn_dim))

    def solve(self, data=None, *, max_attempts: int = 0, record_path: bool | None = None,
              path_capacity: int = 4096, ctx: Context | None = None, **_ignored) -> IVPIterator:
        prob, n, dim, y0, params, t_end = self._problem()
        if record_path is None:
            record_path = n <= 64
        cap = path_capacity if record_path else 0
        while True:
            sol = self._run(prob, y0, params, t_end, cap, ctx, max_attempts)
            if not cap or int(np.max(sol.accepted)) <= cap:
                break
            cap = int(np.max(sol.accepted)) + 1
        return IVPIterator(sol, n, dim)


class Adams5(_AdamsBuilder):
    """5th-order Adams predictor-corrector (src/ivp/adams.rs:605-634)."""
    KIND = 4
    ORDER = 5


class Adams3(_AdamsBuilder):
    """3rd-order Adams predictor-corrector (src/ivp/adams.rs:661-694)."""
    KIND = 5
    ORDER = 3


class Euler(_AdamsBuilder):
    """Euler's method (src/ivp.rs:240-485): with_tolerance is a no-op and the
    step is the first dt given, then the mean with each later one."""
    KIND = 6

    def _run(self, prob, y0, params, t_end, cap, ctx, max_attempts):
        from .engine import euler_solve
        return euler_solve(y0, params, prob.t0_scalar, t_end, rhs=prob.rhs, dt=prob.dt_max,
                           max_steps=max_attempts, traj_cap=cap, ctx=ctx)
