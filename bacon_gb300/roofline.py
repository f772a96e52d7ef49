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



# flops of one vector-Jacobian product of the adjoint (Vjp<> in rhs.cuh)
VJP_FLOPS = {5: 12, 6: 17, 7: 17}


def adjoint_flops(method: int, rhs: int, dim: int, n_params: int, attempts: int, accepted: int) -> int:
    """Forward recording pass plus the reverse kernel: per accepted step a
    replay of the stages and the step update, then the reverse sweep (the
    stage weights lam*b_s, one VJP per stage with dt scaling, the parameter
    and state accumulations, and the transposed tableau products)."""
    t = TABLEAUX[method]
    D, S = dim, t["S"]
    fwd = rk_flops(method, rhs, dim, attempts, accepted)
    replay = 2 * D * t["nnz_a"] + S * (RHS_FLOPS[rhs] + D) + 2 * D * t["nnz_b"] + 1
    sweep = S * D + S * (D + VJP_FLOPS[rhs] + n_params + D) + 2 * D * t["nnz_a"]
    return fwd + int(accepted) * (replay + sweep)


# flops of the chain right-hand side per state component and of the
# analytic Jacobians of the stiff right-hand sides
CHAIN_FLOPS_PER_COMPONENT = 3.5
JAC_FLOPS = {8: 10, 9: 0}


def bdf_flops(dim: int, rhs_flops: float, steps: float, newton_solves: float, newton_iters: float,
              factorisations: float, jac_flops: float = 0.0, q: int = 6, lu_fraction: float = 1.0) -> float:
    """Corrected BDF: per step the predictor and the error norm; per Newton
    solve the Jacobian, the matrix I - h b_q J and the history constant; per
    Newton iteration the right-hand side, the residual, the two triangular
    substitutions (2 dim^2) and the update with its norm; per
    factorisation the LU (2/3 dim^3 dense, times lu_fraction: the share of
    its updates the elimination executes, since it skips updates by exactly
    zero entries), the pivot reciprocals, and the inversion of the diagonal
    32-row blocks of L and U (each column the solve of a unit vector over the
    whole triangle: 2 nb^2 (nb - 1) flops per block of nb rows)."""
    n = float(dim)
    per_step = 2 * n * (q + 1) + 3 * n + 1
    per_solve = jac_flops + 2 * n * n + 2 * n * q
    per_iter = rhs_flops + 3 * n + 2 * n * n + 3 * n + 1
    blocks = [min(32, dim - s) for s in range(0, dim, 32)]
    per_fact = lu_fraction * 2.0 * n ** 3 / 3.0 + n + sum(2.0 * nb * nb * (nb - 1) for nb in blocks)
    return steps * per_step + newton_solves * per_solve + newton_iters * per_iter + factorisations * per_fact


def linear_tc_flops(dim: int, attempts: int, stages: int = 6, slice_pairs: int = 15,
                    last_pairs: int | None = None) -> tuple[float, float]:
    """(bf16 tensor-core flops, FP64-equivalent flops) of the GEMMs of the
    shared-matrix linear solve: every attempt of every system multiplies a
    vector by A `stages` times, as slice_pairs bf16 slice products on the
    tensor cores (last_pairs for the last product, which feeds only the error
    estimate), or one FP64 matrix-vector product of 2 dim^2."""
    per = float(attempts) * 2.0 * dim * dim
    lp = slice_pairs if last_pairs is None else last_pairs
    return per * ((stages - 1) * slice_pairs + lp), per * stages
