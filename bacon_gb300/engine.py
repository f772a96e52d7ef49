"""Low-level batched solves over the C ABI.

``rk_solve`` accepts either host numpy arrays (the library stages them
through device memory: BACON_MEM_HOST) or CUDA tensors that are already
resident on the GPU (BACON_MEM_DEVICE).  Arrays are SoA: ``y0`` is
(dim, n), ``params`` is (n_params, n).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _capi

RK45, RK23 = 0, 1
AS_COMPILED, AS_WRITTEN, FEHLBERG = 0, 1, 2
FP64_EXACT, FP64_FMA, FP32_COMP, TC_SPLIT = 0, 1, 2, 3
MEM_DEVICE, MEM_HOST = 0, 1


class IVPError(Exception):
    """An IVPError variant (src/ivp.rs:50-76) or an engine extension code."""

    def __init__(self, code: int, message: str = ""):
        self.code = int(code)
        self.variant = _capi.STATUS_NAMES.get(self.code, f"Status{self.code}")
        super().__init__(f"{self.variant}: {message}" if message else self.variant)


def check(code: int) -> None:
    if code != 0:
        raise IVPError(code, _capi.last_error())


class Context:
    """Owns a bacon_ctx (stream, scratch, graph and tuning caches) on one device."""

    def __init__(self, device: int = 0):
        self._lib = _capi.load()
        h = ctypes.c_void_p()
        check(self._lib.bacon_ctx_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self._lib.bacon_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.bacon_ctx_kernel_launches(self.handle))

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        s = ctypes.c_void_p()
        check(self._lib.bacon_ctx_stream(self.handle, ctypes.byref(s)))
        return int(s.value or 0)

    def last_kernel_ms(self) -> float:
        """Device time of the last solve's main kernel (CUDA events on the
        context's stream)."""
        ms = ctypes.c_double()
        check(self._lib.bacon_ctx_last_kernel_ms(self.handle, ctypes.byref(ms)))
        return ms.value

    def last_reverse_ms(self) -> float:
        """Device time of the last adjoint's reverse kernel."""
        ms = ctypes.c_double()
        check(self._lib.bacon_ctx_last_reverse_ms(self.handle, ctypes.byref(ms)))
        return ms.value

    def fp64_peak_gflops(self) -> float:
        g = ctypes.c_double()
        check(self._lib.bacon_measure_fp64_peak(self.handle, ctypes.byref(g)))
        return g.value


_default: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


@dataclass
class Solution:
    """Per-system outcome of a batched solve (host arrays or CUDA tensors)."""
    y: Any            # (dim, n)
    t: Any            # (n,)
    accepted: Any     # (n,)
    rejected: Any     # (n,)
    status: Any       # (n,)
    code: int         # BACON_OK or the lowest failing system's status
    traj_t: Any = None
    traj_y: Any = None
    traj_off: Any = None   # dense output: system i's items are [traj_off[i], traj_off[i+1])


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _is_device(a) -> bool:
    return not isinstance(a, np.ndarray) and getattr(a, "is_cuda", False)


def make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs, dyn_dim=False, shared=None):
    """Build a bacon_problem; t0 / t_end may be scalars or per-system arrays."""
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    p = _capi.Problem()
    p.n = n
    p.dim = dim
    p.rhs = int(rhs)
    p.n_params = 0 if params is None else int(params.shape[0])
    p.dyn_dim = int(bool(dyn_dim))
    p.y0 = _ptr(y0)
    p.params = _ptr(params) if p.n_params else None
    if np.isscalar(t0):
        p.t0 = None
        p.t0_scalar = float(t0)
    else:
        p.t0 = _ptr(t0)
    if np.isscalar(t_end):
        p.t_end = None
        p.t_end_scalar = float(t_end)
    else:
        p.t_end = _ptr(t_end)
    p.shared = _ptr(shared)
    p.tol, p.dt_min, p.dt_max = float(tol), float(dt_min), float(dt_max)
    return p


def rk_options(method=RK45, layout=FEHLBERG, precision=FP64_EXACT, memory=MEM_HOST, max_attempts=0,
               block=0, blocks_per_sm=0, use_graph=True, schedule=0, systems_per_warp=0):
    o = _capi.RkOptions()
    o.method, o.layout, o.precision, o.memory = method, layout, precision, memory
    o.max_attempts = int(max_attempts)
    o.block, o.blocks_per_sm = int(block), int(blocks_per_sm)
    o.use_graph = int(bool(use_graph))
    o.schedule = int(schedule)
    o.systems_per_warp = int(systems_per_warp)
    return o


def alloc_outputs(dim: int, n: int, device: bool, traj_cap: int = 0, pin: bool = False):
    if device:
        import torch
        dev = torch.device("cuda")
        out = dict(y=torch.empty((dim, n), dtype=torch.float64, device=dev),
                   t=torch.empty(n, dtype=torch.float64, device=dev),
                   accepted=torch.empty(n, dtype=torch.int32, device=dev),
                   rejected=torch.empty(n, dtype=torch.int32, device=dev),
                   status=torch.empty(n, dtype=torch.int32, device=dev))
        if traj_cap:
            out["traj_t"] = torch.empty((n, traj_cap), dtype=torch.float64, device=dev)
            out["traj_y"] = torch.empty((n, traj_cap, dim), dtype=torch.float64, device=dev)
        return out
    if pin:
        import torch
        def mk(shape, dt):
            return torch.empty(shape, dtype=dt, pin_memory=True).numpy()
        f64, i32 = torch.float64, torch.int32
    else:
        def mk(shape, dt):
            return np.empty(shape, dtype=dt)
        f64, i32 = np.float64, np.int32
    out = dict(y=mk((dim, n), f64), t=mk(n, f64), accepted=mk(n, i32), rejected=mk(n, i32),
               status=mk(n, i32))
    if traj_cap:
        out["traj_t"] = mk((n, traj_cap), f64)
        out["traj_y"] = mk((n, traj_cap, dim), f64)
    return out


def make_result(out, traj_cap=0):
    r = _capi.RkResult()
    r.y_final, r.t_final = _ptr(out["y"]), _ptr(out["t"])
    r.accepted, r.rejected, r.status = _ptr(out["accepted"]), _ptr(out["rejected"]), _ptr(out["status"])
    r.traj_t = _ptr(out.get("traj_t"))
    r.traj_y = _ptr(out.get("traj_y"))
    r.traj_cap = int(traj_cap)
    return r


def _dense_call(fn, handle, prob, opts, out, device, dim, n, capacity):
    """Calls a *_solve_dense entry point.  With capacity None it first asks
    for the item count (capacity 0), then allocates exactly that.  Returns
    (code, t, y, offsets)."""
    if device:
        import torch
        dev = torch.device("cuda")
        mk = lambda shape, dt: torch.empty(shape, dtype=dt, device=dev)  # noqa: E731
        f64, i64 = torch.float64, torch.int64
    else:
        mk = lambda shape, dt: np.empty(shape, dtype=dt)  # noqa: E731
        f64, i64 = np.float64, np.int64
    off = mk(n + 1, i64)
    res = make_result(out)
    if capacity is None:
        dz = _capi.DenseOutput()
        dz.capacity, dz.t, dz.y, dz.offsets = 0, None, None, _ptr(off)
        code = fn(handle, ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), ctypes.byref(dz))
        if code in (14, 15, 16):
            raise IVPError(code, _capi.last_error())
        capacity = int(dz.total)
    t = mk(max(capacity, 1), f64)
    y = mk((max(capacity, 1), dim), f64)
    dz = _capi.DenseOutput()
    dz.capacity, dz.t, dz.y, dz.offsets = int(capacity), _ptr(t), _ptr(y), _ptr(off)
    code = fn(handle, ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res), ctypes.byref(dz))
    total = int(dz.total)
    return code, t[:total], y[:total], off


def rk_solve(y0, params, t0, t_end, *, rhs, tol, dt_min, dt_max, method=RK45, layout=FEHLBERG,
             precision=FP64_EXACT, max_attempts=0, traj_cap=0, ctx: Context | None = None,
             plain=False, block=0, blocks_per_sm=0, use_graph=True, dyn_dim=False, out=None,
             raise_on_error=False, schedule=0, shared=None, dense=False, dense_capacity=None,
             systems_per_warp=0) -> Solution:
    """Batched RK45/RK23 solve.  Inputs are all numpy (host) or all CUDA tensors.
    ``shared``: the dim x dim matrix of BACON_RHS_LINEAR (row-major).
    ``dense``: every yielded item of every system, packed (bacon_rk_solve_dense):
    the Solution's traj_t (total,), traj_y (total, dim) and traj_off (n+1,)."""
    ctx = ctx or default_context()
    device = _is_device(y0)
    if not device:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        if params is not None:
            params = np.ascontiguousarray(params, dtype=np.float64)
        if not np.isscalar(t0):
            t0 = np.ascontiguousarray(t0, dtype=np.float64)
        if not np.isscalar(t_end):
            t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    if shared is not None and not device:
        shared = np.ascontiguousarray(shared, dtype=np.float64)
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    prob = make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs, dyn_dim, shared)
    opts = rk_options(method, layout, precision, MEM_DEVICE if device else MEM_HOST, max_attempts,
                      block, blocks_per_sm, use_graph, schedule, systems_per_warp)
    if out is None:
        out = alloc_outputs(dim, n, device, traj_cap)
    lib = _capi.load()
    if dense:
        code, tt, ty, off = _dense_call(lib.bacon_rk_solve_dense, ctx.handle, prob, opts, out, device, dim, n,
                                        dense_capacity)
        if code in (14, 15, 16) or (raise_on_error and code != 0):
            raise IVPError(code, _capi.last_error())
        return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code), tt, ty, off)
    res = make_result(out, traj_cap)
    fn = lib.bacon_rk_solve_plain if plain else lib.bacon_rk_solve
    code = fn(ctx.handle, ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(res))
    if code in (14, 15, 16) or (raise_on_error and code != 0):
        raise IVPError(code, _capi.last_error())
    return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code),
                    out.get("traj_t"), out.get("traj_y"))


@dataclass
class AdjointSolution:
    """Forward outcome plus the loss and its gradients per system."""
    forward: Solution
    loss: Any      # (n,)
    dl_dy0: Any    # (dim, n)
    dl_dp: Any     # (n_params, n) or None
    code: int


def rk_solve_adjoint(y0, params, t0, t_end, target, *, rhs, tol, dt_min, dt_max, method=RK45,
                     layout=FEHLBERG, max_attempts=0, checkpoint_every=32, max_steps=1024,
                     ctx: Context | None = None, block=0, blocks_per_sm=0, out=None, grads=None,
                     schedule=0, raise_on_error=False) -> AdjointSolution:
    """Batched solve_ivp_adjoint: loss_i = ||y_i(T) - target_i||^2 and its
    gradient with respect to y0_i and params_i (discrete adjoint, checkpoints
    every ``checkpoint_every`` accepted steps)."""
    ctx = ctx or default_context()
    device = _is_device(y0)
    if not device:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        target = np.ascontiguousarray(target, dtype=np.float64)
        if params is not None:
            params = np.ascontiguousarray(params, dtype=np.float64)
        if not np.isscalar(t0):
            t0 = np.ascontiguousarray(t0, dtype=np.float64)
        if not np.isscalar(t_end):
            t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    n_params = 0 if params is None else int(params.shape[0])
    prob = make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs)
    opts = rk_options(method, layout, FP64_EXACT, MEM_DEVICE if device else MEM_HOST, max_attempts,
                      block, blocks_per_sm, False, schedule)
    if out is None:
        out = alloc_outputs(dim, n, device)
    if grads is None:
        if device:
            import torch
            mk = lambda *s: torch.empty(s, dtype=torch.float64, device=y0.device)  # noqa: E731
        else:
            mk = lambda *s: np.empty(s, dtype=np.float64)  # noqa: E731
        grads = dict(loss=mk(n), dl_dy0=mk(dim, n), dl_dp=mk(max(n_params, 1), n))
    res = make_result(out)
    adj = _capi.Adjoint()
    adj.target = _ptr(target)
    adj.loss, adj.dl_dy0 = _ptr(grads["loss"]), _ptr(grads["dl_dy0"])
    adj.dl_dp = _ptr(grads["dl_dp"]) if n_params else None
    adj.checkpoint_every, adj.max_steps = int(checkpoint_every), int(max_steps)
    code = _capi.load().bacon_rk_solve_adjoint(ctx.handle, ctypes.byref(prob), ctypes.byref(opts),
                                               ctypes.byref(res), ctypes.byref(adj))
    if code in (14, 15, 16) or (raise_on_error and code != 0):
        raise IVPError(code, _capi.last_error())
    fwd = Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code))
    return AdjointSolution(fwd, grads["loss"], grads["dl_dy0"], grads["dl_dp"] if n_params else None,
                           int(code))


def rk_autotune(y0, params, t0, t_end, *, rhs, tol, dt_min, dt_max, method=RK45, layout=FEHLBERG,
                precision=FP64_EXACT, max_attempts=0, ctx: Context | None = None, out=None,
                schedule=0, details=False):
    """Time the candidate kernel variants (register budgets) and launch shapes
    on this batch and cache the fastest in the context (used by later solves
    of the same kernel and batch size).  Returns (threads per block,
    persistent CTAs per SM), or with details=True a dict of the whole
    bacon_tune_result."""
    ctx = ctx or default_context()
    device = _is_device(y0)
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    prob = make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs)
    opts = rk_options(method, layout, precision, MEM_DEVICE if device else MEM_HOST, max_attempts,
                      0, 0, False, schedule)
    if out is None:
        out = alloc_outputs(dim, n, device)
    res = make_result(out)
    t = _capi.TuneResult()
    check(_capi.load().bacon_rk_autotune_ex(ctx.handle, ctypes.byref(prob), ctypes.byref(opts),
                                            ctypes.byref(res), ctypes.byref(t)))
    if details:
        return {f: getattr(t, f) for f, _ in _capi.TuneResult._fields_}
    return t.block, t.blocks_per_sm


def rk_set_tuned(y0, *, rhs, variant, block, blocks_per_sm, method=RK45, layout=FEHLBERG, precision=FP64_EXACT,
                 ctx: Context | None = None, systems_per_warp=32):
    """Pin the kernel variant, launch shape and systems per warp the
    context uses for this kernel and batch size (bacon_rk_set_tuned)."""
    ctx = ctx or default_context()
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    prob = _capi.Problem()
    prob.n, prob.dim, prob.rhs = n, dim, int(rhs)
    opts = rk_options(method, layout, precision)
    t = _capi.TuneResult()
    t.variant, t.block, t.blocks_per_sm = int(variant), int(block), int(blocks_per_sm)
    t.systems_per_warp = int(systems_per_warp)
    check(_capi.load().bacon_rk_set_tuned(ctx.handle, ctypes.byref(prob), ctypes.byref(opts), ctypes.byref(t)))


BDF6, BDF2 = 0, 1
BDF_AS_COMPILED, BDF_CORRECTED = 0, 1


def bdf_solve(y0, params, t0, t_end, *, rhs, tol, dt_min, dt_max, method=BDF6, mode=BDF_CORRECTED,
              max_iter=0, max_steps=0, traj_cap=0, ctx: Context | None = None, block=0, blocks_per_sm=0,
              dyn_dim=False, out=None, raise_on_error=False, dense=False, dense_capacity=None) -> Solution:
    """Batched BDF6 / BDF2 solve (systems of dimension <= 8); ``dense`` as
    rk_solve (bacon_bdf_solve_dense)."""
    ctx = ctx or default_context()
    device = _is_device(y0)
    if not device:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        if params is not None:
            params = np.ascontiguousarray(params, dtype=np.float64)
        if not np.isscalar(t0):
            t0 = np.ascontiguousarray(t0, dtype=np.float64)
        if not np.isscalar(t_end):
            t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    prob = make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs, dyn_dim)
    o = _capi.BdfOptions()
    o.method, o.mode, o.memory = method, mode, MEM_DEVICE if device else MEM_HOST
    o.max_iter, o.max_steps, o.block, o.blocks_per_sm = int(max_iter), int(max_steps), int(block), int(blocks_per_sm)
    if out is None:
        out = alloc_outputs(dim, n, device, traj_cap)
    if dense:
        code, tt, ty, off = _dense_call(_capi.load().bacon_bdf_solve_dense, ctx.handle, prob, o, out, device, dim, n,
                                        dense_capacity)
        if code in (14, 15, 16) or (raise_on_error and code != 0):
            raise IVPError(code, _capi.last_error())
        return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code), tt, ty, off)
    res = make_result(out, traj_cap)
    code = _capi.load().bacon_bdf_solve(ctx.handle, ctypes.byref(prob), ctypes.byref(o), ctypes.byref(res))
    if code in (14, 15, 16) or (raise_on_error and code != 0):
        raise IVPError(code, _capi.last_error())
    return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code),
                    out.get("traj_t"), out.get("traj_y"))


@dataclass
class RaggedSolution:
    """Per-system outcome of a ragged solve: y is flat, system i's final state
    is y[y_off[i]:y_off[i+1]]."""
    y: Any
    t: Any
    accepted: Any
    rejected: Any
    status: Any
    code: int
    traj_t: Any = None     # dense output: system i's items are [traj_off[i], traj_off[i+1])
    traj_y: Any = None     # flat: its states from traj_voff[i], dim_i values each
    traj_off: Any = None
    traj_voff: Any = None


def _alloc_ragged(total: int, n: int, device: bool):
    if device:
        import torch
        dev = torch.device("cuda")
        return dict(y=torch.empty(total, dtype=torch.float64, device=dev),
                    t=torch.empty(n, dtype=torch.float64, device=dev),
                    accepted=torch.empty(n, dtype=torch.int32, device=dev),
                    rejected=torch.empty(n, dtype=torch.int32, device=dev),
                    status=torch.empty(n, dtype=torch.int32, device=dev))
    return dict(y=np.empty(total), t=np.empty(n), accepted=np.empty(n, np.int32),
                rejected=np.empty(n, np.int32), status=np.empty(n, np.int32))


def bdf_solve_mixed(uniform=None, ragged=None, *, method=BDF6, max_iter=0, max_steps=0,
                    ctx: Context | None = None, blocks_per_sm=0, uniform_out=None, ragged_out=None,
                    raise_on_error=False, dense=False):
    """One launch of the corrected BDF over a stiff batch of a uniform part
    (attributes y0 (dim, n), params, t0, t_end, rhs, tol, dt_min, dt_max, as
    workloads.Batch) and a ragged part (y_off, p_off, flat y0 and params, t0,
    t_end, rhs, tol, dt_min, dt_max, as workloads.RaggedBatch).  Arrays are
    all numpy (host) or all CUDA tensors.  Returns (Solution | None,
    RaggedSolution | None).  ``dense``: every yielded item of both parts,
    packed (bacon_bdf_solve_mixed_dense), in the solutions' traj_* fields."""
    ctx = ctx or default_context()
    first = uniform.y0 if uniform is not None else ragged.y0
    device = _is_device(first)
    prob = None
    uout = None
    if uniform is not None:
        prob = make_problem(uniform.y0, uniform.params, uniform.t0, uniform.t_end, uniform.tol,
                            uniform.dt_min, uniform.dt_max, uniform.rhs)
        dim, n = int(uniform.y0.shape[0]), int(uniform.y0.shape[1])
        uout = uniform_out if uniform_out is not None else alloc_outputs(dim, n, device)
    rp = None
    rout = None
    if ragged is not None:
        rp = _capi.RaggedProblem()
        rp.n = int(ragged.y_off.shape[0]) - 1
        rp.rhs = int(ragged.rhs)
        rp.y_offsets, rp.p_offsets = _ptr(ragged.y_off), _ptr(ragged.p_off)
        rp.y0, rp.params = _ptr(ragged.y0), _ptr(ragged.params)
        for name in ("t0", "t_end"):
            v = getattr(ragged, name)
            if np.isscalar(v):
                setattr(rp, name, None)
                setattr(rp, name + "_scalar", float(v))
            else:
                setattr(rp, name, _ptr(v))
        rp.tol, rp.dt_min, rp.dt_max = float(ragged.tol), float(ragged.dt_min), float(ragged.dt_max)
        rout = ragged_out if ragged_out is not None else _alloc_ragged(int(ragged.y0.shape[0]), rp.n, device)
    o = _capi.BdfOptions()
    o.method, o.mode, o.memory = method, BDF_CORRECTED, MEM_DEVICE if device else MEM_HOST
    o.max_iter, o.max_steps, o.block, o.blocks_per_sm = int(max_iter), int(max_steps), 0, int(blocks_per_sm)
    ures = make_result(uout, 0) if uout is not None else None
    rres = None
    if rout is not None:
        rres = _capi.RaggedResult()
        rres.y_final, rres.t_final = _ptr(rout["y"]), _ptr(rout["t"])
        rres.accepted, rres.rejected, rres.status = _ptr(rout["accepted"]), _ptr(rout["rejected"]), _ptr(rout["status"])
    args = (ctx.handle, ctypes.byref(prob) if prob is not None else None,
            ctypes.byref(rp) if rp is not None else None, ctypes.byref(o),
            ctypes.byref(ures) if ures is not None else None, ctypes.byref(rres) if rres is not None else None)
    udz = gdz = None
    if dense:
        code, udz, gdz = _mixed_dense_call(args, uniform, ragged, device)
    else:
        code = _capi.load().bacon_bdf_solve_mixed(*args)
    if code in (14, 15, 16) or (raise_on_error and code != 0):
        raise IVPError(code, _capi.last_error())
    us = None
    if uout is not None:
        us = Solution(uout["y"], uout["t"], uout["accepted"], uout["rejected"], uout["status"], int(code))
        if udz is not None:
            us.traj_t, us.traj_y, us.traj_off = udz
    rs = None
    if rout is not None:
        rs = RaggedSolution(rout["y"], rout["t"], rout["accepted"], rout["rejected"], rout["status"], int(code))
        if gdz is not None:
            rs.traj_t, rs.traj_y, rs.traj_off, rs.traj_voff = gdz
    return us, rs


def _mixed_dense_call(args, uniform, ragged, device):
    """bacon_bdf_solve_mixed_dense: the item counts first (capacity 0), then
    the solve into arrays of exactly that size.  Returns (code, uniform
    (t, y, offsets) or None, ragged (t, y, offsets, value offsets) or None)."""
    if device:
        import torch
        dev = torch.device("cuda")
        mk = lambda shape, dt: torch.empty(shape, dtype=dt, device=dev)  # noqa: E731
        f64, i64 = torch.float64, torch.int64
    else:
        mk = lambda shape, dt: np.empty(shape, dtype=dt)  # noqa: E731
        f64, i64 = np.float64, np.int64
    udz = gdz = None
    uoff = goff = gvoff = None
    if uniform is not None:
        dim, n = int(uniform.y0.shape[0]), int(uniform.y0.shape[1])
        uoff = mk(n + 1, i64)
        udz = _capi.DenseOutput()
        udz.capacity, udz.t, udz.y, udz.offsets = 0, None, None, _ptr(uoff)
    if ragged is not None:
        gn = int(ragged.y_off.shape[0]) - 1
        goff, gvoff = mk(gn + 1, i64), mk(gn + 1, i64)
        gdz = _capi.RaggedDenseOutput()
        gdz.capacity, gdz.value_capacity, gdz.t, gdz.y = 0, 0, None, None
        gdz.offsets, gdz.value_offsets = _ptr(goff), _ptr(gvoff)
    fn = _capi.load().bacon_bdf_solve_mixed_dense
    by = lambda x: ctypes.byref(x) if x is not None else None  # noqa: E731
    code = fn(*args, by(udz), by(gdz))
    if code in (14, 15, 16):
        raise IVPError(code, _capi.last_error())
    ut = uy = gt = gy = None
    if udz is not None:
        cap = int(udz.total)
        ut, uy = mk(max(cap, 1), f64), mk((max(cap, 1), dim), f64)
        udz.capacity, udz.t, udz.y = cap, _ptr(ut), _ptr(uy)
    if gdz is not None:
        cap, vcap = int(gdz.total), int(gdz.total_values)
        gt, gy = mk(max(cap, 1), f64), mk(max(vcap, 1), f64)
        gdz.capacity, gdz.value_capacity, gdz.t, gdz.y = cap, vcap, _ptr(gt), _ptr(gy)
    code = fn(*args, by(udz), by(gdz))
    u = (ut[:int(udz.total)], uy[:int(udz.total)], uoff) if udz is not None else None
    g = (gt[:int(gdz.total)], gy[:int(gdz.total_values)], goff, gvoff) if gdz is not None else None
    return code, u, g


def adams_solve(y0, params, t0, t_end, *, rhs, tol, dt_min, dt_max, order=5, max_attempts=0, traj_cap=0,
                ctx: Context | None = None, block=0, blocks_per_sm=0, dyn_dim=False, out=None,
                raise_on_error=False, dense=False, dense_capacity=None, systems_per_warp=0) -> Solution:
    """Batched Adams5 / Adams3 predictor-corrector (src/ivp/adams.rs); ``dense``
    as rk_solve (bacon_adams_solve_dense)."""
    return _adams_like(y0, params, t0, t_end, rhs=rhs, tol=tol, dt_min=dt_min, dt_max=dt_max, order=order,
                       euler_dt=None, max_attempts=max_attempts, traj_cap=traj_cap, ctx=ctx, block=block,
                       blocks_per_sm=blocks_per_sm, dyn_dim=dyn_dim, out=out, raise_on_error=raise_on_error,
                       dense=dense, dense_capacity=dense_capacity, systems_per_warp=systems_per_warp)


def euler_solve(y0, params, t0, t_end, *, rhs, dt, max_steps=0, traj_cap=0, ctx: Context | None = None,
                block=0, blocks_per_sm=0, out=None, raise_on_error=False, dense=False,
                dense_capacity=None) -> Solution:
    """Batched Euler with a fixed step dt (src/ivp.rs:240-485); ``dense`` as
    rk_solve (bacon_euler_solve_dense)."""
    return _adams_like(y0, params, t0, t_end, rhs=rhs, tol=1.0, dt_min=dt, dt_max=dt, order=1, euler_dt=dt,
                       max_attempts=max_steps, traj_cap=traj_cap, ctx=ctx, block=block,
                       blocks_per_sm=blocks_per_sm, dyn_dim=False, out=out, raise_on_error=raise_on_error,
                       dense=dense, dense_capacity=dense_capacity, systems_per_warp=0)


def _adams_like(y0, params, t0, t_end, *, rhs, tol, dt_min, dt_max, order, euler_dt, max_attempts, traj_cap, ctx,
                block, blocks_per_sm, dyn_dim, out, raise_on_error, dense, dense_capacity, systems_per_warp) -> Solution:
    ctx = ctx or default_context()
    device = _is_device(y0)
    if not device:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        if params is not None:
            params = np.ascontiguousarray(params, dtype=np.float64)
        if not np.isscalar(t0):
            t0 = np.ascontiguousarray(t0, dtype=np.float64)
        if not np.isscalar(t_end):
            t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    dim, n = int(y0.shape[0]), int(y0.shape[1])
    prob = make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, rhs, dyn_dim)
    o = _capi.AdamsOptions()
    o.order = 5 if order == 1 else int(order)
    o.memory = MEM_DEVICE if device else MEM_HOST
    o.max_attempts, o.block, o.blocks_per_sm = int(max_attempts), int(block), int(blocks_per_sm)
    o.systems_per_warp = int(systems_per_warp)
    if out is None:
        out = alloc_outputs(dim, n, device, traj_cap)
    L = _capi.load()
    if dense:
        if euler_dt is None:
            fn = L.bacon_adams_solve_dense
        else:
            def fn(h, pr, op, rs, dz):
                return L.bacon_euler_solve_dense(h, pr, float(euler_dt), op, rs, dz)
        code, tt, ty, off = _dense_call(fn, ctx.handle, prob, o, out, device, dim, n, dense_capacity)
        if code in (14, 15, 16) or (raise_on_error and code != 0):
            raise IVPError(code, _capi.last_error())
        return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code), tt, ty, off)
    res = make_result(out, traj_cap)
    if euler_dt is None:
        code = L.bacon_adams_solve(ctx.handle, ctypes.byref(prob), ctypes.byref(o), ctypes.byref(res))
    else:
        code = L.bacon_euler_solve(ctx.handle, ctypes.byref(prob), float(euler_dt), ctypes.byref(o),
                                   ctypes.byref(res))
    if code in (14, 15, 16) or (raise_on_error and code != 0):
        raise IVPError(code, _capi.last_error())
    return Solution(out["y"], out["t"], out["accepted"], out["rejected"], out["status"], int(code),
                    out.get("traj_t"), out.get("traj_y"))
