"""CPU oracle — TEST INFRASTRUCTURE ONLY.

ctypes wrapper over ``oracle/_build/liboracle.so``, the C restatement of the
bacon-sci 0.16.2 IVP solvers (src/ivp/rk.rs, src/ivp/bdf.rs).  Only the test
suite, the smoke check and the benchmark's CPU-baseline leg may import this
module; the product package never does.  Parity status of the restatement is
described in oracle/oracle.h ("parity unpinned" at the bit level: the Rust
reference cannot be built here).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

RK45, RK23 = 0, 1
AS_COMPILED, AS_WRITTEN, FEHLBERG = 0, 1, 2
POW_QRT, POW_LIBM = 0, 1
BDF6, BDF2 = 0, 1
BDF_AS_COMPILED, BDF_CORRECTED = 0, 1


class _RkCfg(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("layout", ctypes.c_int32),
        ("pow_mode", ctypes.c_int32),
        ("dyn_dim", ctypes.c_int32),
        ("max_attempts", ctypes.c_int64),
        ("tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


class _AdamsCfg(ctypes.Structure):
    _fields_ = [
        ("order", ctypes.c_int32),
        ("pow_mode", ctypes.c_int32),
        ("dyn_dim", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("max_attempts", ctypes.c_int64),
        ("tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


class _BdfCfg(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("dyn_dim", ctypes.c_int32),
        ("max_iter", ctypes.c_int32),
        ("max_steps", ctypes.c_int64),
        ("tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    srcs = [os.path.join(_HERE, f) for f in os.listdir(_HERE) if f.endswith((".c", ".h"))]
    if not force and os.path.exists(_LIB_PATH):
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(_LIB_PATH) >= newest:
            return _LIB_PATH
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_int64)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.oracle_qrt.restype = ctypes.c_double
        L.oracle_qrt.argtypes = [ctypes.c_double]
        L.oracle_norm.restype = ctypes.c_double
        L.oracle_norm.argtypes = [dp, ctypes.c_int32, ctypes.c_int32]
        L.oracle_rhs.restype = None
        L.oracle_rhs.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, dp, dp, dp, dp]
        L.oracle_rk_solve_one.restype = ctypes.c_int32
        L.oracle_rk_solve_one.argtypes = [
            ctypes.POINTER(_RkCfg), ctypes.c_int32, ctypes.c_int32, dp, dp,
            ctypes.c_double, ctypes.c_double, dp, dp, dp, lp, lp, dp, dp, ctypes.c_int64]
        L.oracle_rk_solve_batch.restype = ctypes.c_double
        L.oracle_rk_solve_batch.argtypes = [
            ctypes.POINTER(_RkCfg), ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
            ctypes.c_int32, dp, dp, dp, dp, dp, dp, dp, lp, lp, ip, ctypes.c_int32]
        if hasattr(L, "oracle_bdf_solve_one"):
            L.oracle_bdf_solve_one.restype = ctypes.c_int32
            L.oracle_bdf_solve_one.argtypes = [
                ctypes.POINTER(_BdfCfg), ctypes.c_int32, ctypes.c_int32, dp, dp,
                ctypes.c_double, ctypes.c_double, dp, dp, dp, lp, lp, dp, dp, ctypes.c_int64]
            L.oracle_corrected_linsolve.restype = ctypes.c_int
            L.oracle_corrected_linsolve.argtypes = [ctypes.c_int32, dp, dp, dp]
            L.oracle_bdf_work.restype = None
            L.oracle_bdf_work.argtypes = [lp, ctypes.c_int]
            L.oracle_bdf_secant_inverse.restype = ctypes.c_int
            L.oracle_bdf_secant_inverse.argtypes = [ctypes.c_int32, dp, dp]
        if hasattr(L, "oracle_adams_solve_one"):
            L.oracle_rootn.restype = ctypes.c_double
            L.oracle_rootn.argtypes = [ctypes.c_double, ctypes.c_int]
            L.oracle_adams_solve_one.restype = ctypes.c_int32
            L.oracle_adams_solve_one.argtypes = [
                ctypes.POINTER(_AdamsCfg), ctypes.c_int32, ctypes.c_int32, dp, dp,
                ctypes.c_double, ctypes.c_double, dp, dp, dp, lp, lp, dp, dp, ctypes.c_int64]
            L.oracle_euler_solve_one.restype = ctypes.c_int32
            L.oracle_euler_solve_one.argtypes = [
                ctypes.c_int32, ctypes.c_int32, dp, dp, ctypes.c_double, ctypes.c_int64,
                ctypes.c_double, ctypes.c_double, dp, dp, dp, lp, dp, dp, ctypes.c_int64]
        if hasattr(L, "oracle_rk_adjoint_one"):
            L.oracle_rk_adjoint_one.restype = ctypes.c_int32
            L.oracle_rk_adjoint_one.argtypes = [
                ctypes.POINTER(_RkCfg), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp,
                ctypes.c_double, ctypes.c_double, dp, dp, dp, dp, dp, ctypes.c_int32]
            L.oracle_rk_fwdsens_one.restype = ctypes.c_int32
            L.oracle_rk_fwdsens_one.argtypes = [
                ctypes.POINTER(_RkCfg), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp,
                ctypes.c_double, ctypes.c_double, dp, dp, dp, dp]
            L.oracle_rk_frozen_fd_one.restype = ctypes.c_int32
            L.oracle_rk_frozen_fd_one.argtypes = [
                ctypes.POINTER(_RkCfg), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp,
                ctypes.c_double, ctypes.c_double, dp, dp, ctypes.c_double, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def rk_cfg(method=RK45, layout=AS_WRITTEN, pow_mode=POW_QRT, dyn_dim=False,
           max_attempts=0, tol=1e-6, dt_min=1e-6, dt_max=0.1):
    return _RkCfg(method, layout, pow_mode, int(dyn_dim), int(max_attempts), tol, dt_min, dt_max)


@dataclass
class Path:
    status: int
    t: float
    y: np.ndarray
    accepted: int
    rejected: int
    traj_t: np.ndarray | None = None
    traj_y: np.ndarray | None = None


def rk_solve_one(cfg, rhs, y0, t0, t_end, params=None, shared=None, traj_cap=0) -> Path:
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    dim = y0.shape[0]
    p = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    y = np.zeros(dim)
    t = ctypes.c_double()
    a = ctypes.c_int64()
    r = ctypes.c_int64()
    tt = ty = None
    if traj_cap:
        tt = np.zeros(traj_cap)
        ty = np.zeros((traj_cap, dim))
    st = L.oracle_rk_solve_one(ctypes.byref(cfg), rhs, dim, _dp(p), _dp(sh), t0, t_end,
                               _dp(y0), _dp(y), ctypes.byref(t), ctypes.byref(a),
                               ctypes.byref(r), _dp(tt), _dp(ty), traj_cap)
    if traj_cap:
        n = min(a.value, traj_cap)
        tt, ty = tt[:n], ty[:n]
    return Path(st, t.value, y, a.value, r.value, tt, ty)


def rk_solve_batch(cfg, rhs, y0_soa, params_soa, t0, t_end, shared=None, threads=None):
    """y0_soa: (dim, n); params_soa: (P, n); t0, t_end: (n,).  Returns dict."""
    L = lib()
    y0_soa = np.ascontiguousarray(y0_soa, dtype=np.float64)
    dim, n = y0_soa.shape
    if params_soa is None or params_soa.size == 0:
        params_soa = np.zeros((0, n))
    params_soa = np.ascontiguousarray(params_soa, dtype=np.float64)
    n_params = params_soa.shape[0]
    t0 = np.ascontiguousarray(np.broadcast_to(t0, (n,)), dtype=np.float64)
    t_end = np.ascontiguousarray(np.broadcast_to(t_end, (n,)), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    y = np.zeros((dim, n))
    t = np.zeros(n)
    acc = np.zeros(n, dtype=np.int64)
    rej = np.zeros(n, dtype=np.int64)
    st = np.zeros(n, dtype=np.int32)
    threads = threads or os.cpu_count() or 1
    secs = L.oracle_rk_solve_batch(
        ctypes.byref(cfg), rhs, dim, n, n_params, _dp(y0_soa),
        _dp(params_soa) if n_params else None, _dp(sh), _dp(t0), _dp(t_end), _dp(y), _dp(t),
        acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        rej.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), threads)
    return {"y": y, "t": t, "accepted": acc, "rejected": rej, "status": st,
            "seconds": secs, "threads": threads}


def qrt(x: float) -> float:
    return lib().oracle_qrt(float(x))


def corrected_linsolve(A, b):
    """The corrected BDF's linear solve alone (pivoted LU, row-scaled U,
    inverted 32x32 diagonal blocks): x with A x = b, or None on a zero pivot."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    ok = lib().oracle_corrected_linsolve(A.shape[0], _dp(A), _dp(b), _dp(x))
    return x if ok else None


def norm(x, dyn_dim=False) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().oracle_norm(_dp(x), x.shape[0], int(dyn_dim))


def rhs_eval(rhs, t, y, params=None, shared=None):
    y = np.ascontiguousarray(y, dtype=np.float64)
    p = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    f = np.zeros_like(y)
    lib().oracle_rhs(rhs, y.shape[0], t, _dp(y), _dp(p), _dp(sh), _dp(f))
    return f


def rk_adjoint_one(cfg, rhs, y0, params, t0, t_end, target, checkpoint_every=32):
    """Discrete adjoint (oracle), segments of checkpoint_every accepted steps
    replayed with fused multiply-adds as the GPU's reverse kernel does:
    returns (status, loss, dL/dy0, dL/dp)."""
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    gy = np.zeros(y0.shape[0])
    gp = np.zeros(p.shape[0])
    loss = ctypes.c_double()
    st = L.oracle_rk_adjoint_one(ctypes.byref(cfg), rhs, y0.shape[0], p.shape[0], _dp(p), t0, t_end,
                                 _dp(y0), _dp(tg), ctypes.byref(loss), _dp(gy), _dp(gp), int(checkpoint_every))
    return st, loss.value, gy, gp


def rk_frozen_fd_one(cfg, rhs, y0, params, t0, t_end, target, h=1e-6):
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    gy = np.zeros(y0.shape[0])
    gp = np.zeros(p.shape[0])
    st = L.oracle_rk_frozen_fd_one(ctypes.byref(cfg), rhs, y0.shape[0], p.shape[0], _dp(p), t0, t_end,
                                   _dp(y0), _dp(tg), h, _dp(gy), _dp(gp))
    return st, gy, gp


def rk_fwdsens_one(cfg, rhs, y0, params, t0, t_end, target):
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    gy = np.zeros(y0.shape[0])
    gp = np.zeros(p.shape[0])
    st = L.oracle_rk_fwdsens_one(ctypes.byref(cfg), rhs, y0.shape[0], p.shape[0], _dp(p), t0, t_end,
                                 _dp(y0), _dp(tg), _dp(gy), _dp(gp))
    return st, gy, gp


def bdf_cfg(method=BDF6, mode=BDF_CORRECTED, dyn_dim=False, max_iter=0, max_steps=0, tol=1e-6,
            dt_min=1e-10, dt_max=1.0):
    return _BdfCfg(method, mode, int(dyn_dim), int(max_iter), int(max_steps), tol, dt_min, dt_max)


def bdf_solve_one(cfg, rhs, y0, t0, t_end, params=None, shared=None, traj_cap=0) -> Path:
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    dim = y0.shape[0]
    p = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    y = np.zeros(dim)
    t = ctypes.c_double()
    a = ctypes.c_int64()
    r = ctypes.c_int64()
    tt = ty = None
    if traj_cap:
        tt = np.zeros(traj_cap)
        ty = np.zeros((traj_cap, dim))
    st = L.oracle_bdf_solve_one(ctypes.byref(cfg), rhs, dim, _dp(p), _dp(sh), t0, t_end,
                                _dp(y0), _dp(y), ctypes.byref(t), ctypes.byref(a),
                                ctypes.byref(r), _dp(tt), _dp(ty), traj_cap)
    if traj_cap:
        n = min(a.value, traj_cap)
        tt, ty = tt[:n], ty[:n]
    return Path(st, t.value, y, a.value, r.value, tt, ty)


def bdf_secant_inverse(A):
    """(which, inverse) of the as-compiled BDF's secant: 1 partial-pivot LU,
    2 full-pivot LU, 3 QR, 0 SingularMatrix (inverse None)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    inv = np.zeros_like(A)
    which = lib().oracle_bdf_secant_inverse(A.shape[0], _dp(A), _dp(inv))
    return which, (inv if which > 0 else None)


def bdf_work(reset: bool = True) -> dict:
    """Corrected-BDF work on the calling thread since the last reset:
    Newton solves, Newton iterations, the factorisations needed at the least,
    and the elimination FMAs executed and of the dense LU (see
    oracle_bdf_work in oracle.h)."""
    out = np.zeros(5, dtype=np.int64)
    lib().oracle_bdf_work(out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(reset))
    return {"newton_solves": int(out[0]), "newton_iters": int(out[1]), "factorisations": int(out[2]),
            "elim_fmas": int(out[3]), "elim_fmas_dense": int(out[4])}


# ---- Adams predictor-corrector and Euler (src/ivp/adams.rs, src/ivp.rs) ----
def adams_cfg(order=5, pow_mode=POW_QRT, dyn_dim=False, max_attempts=0, tol=1e-6, dt_min=1e-6, dt_max=0.1):
    return _AdamsCfg(int(order), int(pow_mode), int(dyn_dim), 0, int(max_attempts), tol, dt_min, dt_max)


def rootn(x: float, n: int) -> float:
    return lib().oracle_rootn(float(x), int(n))


def adams_solve_one(cfg, rhs, y0, t0, t_end, params=None, shared=None, traj_cap=0) -> Path:
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    dim = y0.shape[0]
    p = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    y = np.zeros(dim)
    t = ctypes.c_double()
    a = ctypes.c_int64()
    r = ctypes.c_int64()
    tt = ty = None
    if traj_cap:
        tt = np.zeros(traj_cap)
        ty = np.zeros((traj_cap, dim))
    st = L.oracle_adams_solve_one(ctypes.byref(cfg), rhs, dim, _dp(p), _dp(sh), t0, t_end, _dp(y0), _dp(y),
                                  ctypes.byref(t), ctypes.byref(a), ctypes.byref(r), _dp(tt), _dp(ty), traj_cap)
    if traj_cap:
        n = min(a.value, traj_cap)
        tt, ty = tt[:n], ty[:n]
    return Path(st, t.value, y, a.value, r.value, tt, ty)


def euler_solve_one(rhs, y0, t0, t_end, dt, params=None, shared=None, max_steps=0, traj_cap=0) -> Path:
    L = lib()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    dim = y0.shape[0]
    p = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float64)
    sh = None if shared is None else np.ascontiguousarray(shared, dtype=np.float64)
    y = np.zeros(dim)
    t = ctypes.c_double()
    a = ctypes.c_int64()
    tt = ty = None
    if traj_cap:
        tt = np.zeros(traj_cap)
        ty = np.zeros((traj_cap, dim))
    st = L.oracle_euler_solve_one(rhs, dim, _dp(p), _dp(sh), dt, int(max_steps), t0, t_end, _dp(y0), _dp(y),
                                  ctypes.byref(t), ctypes.byref(a), _dp(tt), _dp(ty), traj_cap)
    if traj_cap:
        n = min(a.value, traj_cap)
        tt, ty = tt[:n], ty[:n]
    return Path(st, t.value, y, a.value, 0, tt, ty)
