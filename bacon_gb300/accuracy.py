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


def chain_matrix(k: np.ndarray, c: float) -> np.ndarray:
    """The constant Jacobian of a damped spring-mass chain with m = len(k)
    unit masses (BACON_RHS_CHAIN): state (x_1..x_m, v_1..v_m), x' = v,
    v_i' = k_i (x_{i-1} - x_i) + k_{i+1} (x_{i+1} - x_i) - c v_i with
    x_0 = x_{m+1} = 0 and k_{m+1} = 0."""
    m = len(k)
    J = np.zeros((2 * m, 2 * m))
    J[:m, m:] = np.eye(m)
    for i in range(m):
        kr = k[i + 1] if i + 1 < m else 0.0
        J[m + i, i] = -(k[i] + kr)
        if i > 0:
            J[m + i, i - 1] = k[i]
        if i + 1 < m:
            J[m + i, i + 1] = kr
        J[m + i, m + i] = -c
    return J


def chain_exact_final(y0: np.ndarray, params: np.ndarray, t: float) -> np.ndarray:
    """Exact y(t) = expm(J t) y0 of one chain (params = k_1..k_m, c)."""
    from scipy.linalg import expm
    m = len(y0) // 2
    return expm(chain_matrix(params[:m], float(params[m])) * t) @ y0


def robertson_reference(y0: np.ndarray, params: np.ndarray, t_end: float, rtol: float = 1e-12,
                        atol: float = 1e-14) -> np.ndarray:
    """y(t_end) of one Robertson system (k1, k2, k3) with scipy's Radau and
    the analytic Jacobian, at rtol 1e-12."""
    from scipy.integrate import solve_ivp
    k1, k2, k3 = (float(v) for v in params)

    def f(t, y):
        return [-k1 * y[0] + k3 * y[1] * y[2], k1 * y[0] - k2 * y[1] * y[1] - k3 * y[1] * y[2],
                k2 * y[1] * y[1]]

    def jac(t, y):
        return [[-k1, k3 * y[2], k3 * y[1]], [k1, -2.0 * k2 * y[1] - k3 * y[2], -k3 * y[1]],
                [0.0, 2.0 * k2 * y[1], 0.0]]

    sol = solve_ivp(f, (0.0, t_end), np.asarray(y0, float), method="Radau", rtol=rtol, atol=atol, jac=jac)
    if not sol.success:
        raise RuntimeError(sol.message)
    return sol.y[:, -1].copy()
