"""High-accuracy FP64 references for final-state error reports.

Integrates many systems at once as one block-diagonal system with scipy's
DOP853 at rtol = atol = 1e-12, the accuracy reference against which every
result of the engine (any precision mode) reports its final-state error.
CPU only; scipy is imported lazily.
"""
from __future__ import annotations

import numpy as np

from . import workloads as W


def _rhs(rhs: int, prm: np.ndarray):
    if rhs == W.RHS_VDP:
        mu = prm[0]

        def f(t, Y):
            y0, y1 = Y[0::2], Y[1::2]
            out = np.empty_like(Y)
            out[0::2] = y1
            out[1::2] = mu * (1.0 - y0 * y0) * y1 - y0
            return out
    elif rhs == W.RHS_LORENZ:
        s, r, b = prm

        def f(t, Y):
            x, y, z = Y[0::3], Y[1::3], Y[2::3]
            out = np.empty_like(Y)
            out[0::3] = s * (y - x)
            out[1::3] = x * (r - z) - y
            out[2::3] = x * y - b * z
            return out
    elif rhs == W.RHS_LOTKA:
        a, b, c, d = prm

        def f(t, Y):
            x, y = Y[0::2], Y[1::2]
            out = np.empty_like(Y)
            out[0::2] = a * x - b * x * y
            out[1::2] = c * x * y - d * y
            return out
    else:
        raise ValueError(f"no reference right-hand side for rhs {rhs}")
    return f


def reference_final_states(batch: W.Batch, rtol: float = 1e-12, atol: float = 1e-12) -> np.ndarray:
    """y(t_end) for every system of the batch, shape (dim, n).  Systems with
    different end times are integrated together to the largest end time with
    dense output and sampled at their own end times."""
    from scipy.integrate import solve_ivp

    dim, n = batch.dim, batch.n
    f = _rhs(batch.rhs, batch.params)
    y0 = np.ascontiguousarray(batch.y0.T).reshape(-1)
    t0 = float(batch.t0[0])
    if not np.all(batch.t0 == t0):
        raise ValueError("reference assumes a common start time")
    tmax = float(np.max(batch.t_end))
    uniform = bool(np.all(batch.t_end == tmax))
    sol = solve_ivp(f, (t0, tmax), y0, method="DOP853", rtol=rtol, atol=atol, dense_output=not uniform)
    if not sol.success:
        raise RuntimeError(sol.message)
    if uniform:
        return sol.y[:, -1].reshape(n, dim).T.copy()
    out = np.empty((dim, n))
    for i in range(n):
        out[:, i] = sol.sol(batch.t_end[i])[i * dim:(i + 1) * dim]
    return out


def final_state_error(y: np.ndarray, ref: np.ndarray) -> dict:
    """Absolute and relative max-norm errors per system, summarised."""
    err = np.abs(np.asarray(y) - ref).max(axis=0)
    rel = err / np.maximum(np.abs(ref).max(axis=0), 1e-300)
    return {"abs_median": float(np.median(err)), "abs_max": float(err.max()),
            "rel_median": float(np.median(rel)), "rel_max": float(rel.max()), "systems": int(err.size)}
