"""Algorithmic floating-point work of the Runge-Kutta attempt.

The roofline of the integrators counts the operations the algorithm of
src/ivp/rk.rs:361-423 needs per attempt, with the zero tableau entries
skipped: every product and every sum is one flop, and a division, a square
root and the fourth root of the controller count as one flop each.  The
counts follow the compile-time tableaux of bacon_gb300/csrc/tableau.cuh.
"""
from __future__ import annotations

# flops of one right-hand-side evaluation (bacon_gb300/csrc/rhs.cuh)
RHS_FLOPS = {0: 0, 1: 0, 2: 1, 3: 1, 4: 0, 5: 5, 6: 8, 7: 8, 8: 8}
RHS_USES_T = {2, 3}

_RKF45_A = {(1, 0): 1, (2, 0): 1, (2, 1): 1, (3, 0): 1, (3, 1): 1, (3, 2): 1, (4, 0): 1, (4, 1): 1,
            (4, 2): 1, (4, 3): 1, (5, 0): 1, (5, 1): 1, (5, 2): 1, (5, 3): 1, (5, 4): 1}
_BS23_A = {(1, 0): 1, (2, 1): 1, (3, 0): 1, (3, 1): 1, (3, 2): 1}
TABLEAUX = {
    0: dict(S=6, nnz_a=len(_RKF45_A), nnz_b=4, nnz_e=5, e0=True),   # RKF45
    1: dict(S=4, nnz_a=len(_BS23_A), nnz_b=3, nnz_e=4, e0=True),    # Bogacki-Shampine
}


def flops_per_attempt(method: int, rhs: int, dim: int) -> tuple[int, int]:
    """(flops of every attempt, extra flops of an accepted attempt)."""
    t = TABLEAUX[method]
    D = dim
    stage = 2 * D * t["nnz_a"] + t["S"] * (RHS_FLOPS[rhs] + D + (2 if rhs in RHS_USES_T else 0))
    err = D + 2 * D * (t["nnz_e"] - 1) + 2 * D + 1      # e-vector, norm (with sqrt), / dt
    ctrl = 1 + 3                                         # end clamp; tol/err, fourth root, dt scale
    accept = 1 + 2 * D * t["nnz_b"]
    return stage + err + ctrl, accept


def rk_flops(method: int, rhs: int, dim: int, attempts: int, accepted: int) -> int:
    per, acc = flops_per_attempt(method, rhs, dim)
    return per * int(attempts) + acc * int(accepted)

