"""The corrected BDF's linear solve, checked on its own (CPU, oracle).

The GPU kernels are bit-identical to the oracle's corrected BDF, whose linear
solve is this engine's own: a partial-pivot LU with fused updates, the rows
of U scaled by the pivot reciprocals, the 32x32 diagonal blocks of both
factors replaced by their inverses, and block solves as products with those
inverses.  These tests check that it solves linear systems to working
accuracy: for random matrices of every block layout (one partial block, full
blocks, a partial last block), for the matrices the stiff chains meet
(M = I - h b J with stiffnesses up to 1e6), and with pivoting forced.
"""
import numpy as np
import pytest

DIMS = [1, 2, 5, 31, 32, 33, 63, 64, 65, 96, 97, 100, 127, 128]


def _residual(A, x, b):
    return np.linalg.norm(A @ x - b) / (np.linalg.norm(A, 2) * np.linalg.norm(x) + np.linalg.norm(b))


@pytest.mark.parametrize("n", DIMS)
def test_random_systems(oracle, n):
    rng = np.random.default_rng(100 + n)
    for _ in range(3):
        A = rng.standard_normal((n, n))
        b = rng.standard_normal(n)
        x = oracle.corrected_linsolve(A, b)
        assert x is not None
        assert _residual(A, x, b) < 1e-13 * n
        x_ref = np.linalg.solve(A, b)
        cond = np.linalg.cond(A)
        assert np.linalg.norm(x - x_ref) <= 1e-13 * cond * np.linalg.norm(x_ref) * n


def _chain_jacobian(k, damping):
    """The spring chain's Jacobian (unit masses): x' = v, v_i' = k_i (x_{i-1}
    - x_i) + k_{i+1} (x_{i+1} - x_i) - c v_i, fixed ends."""
    N = len(k)
    J = np.zeros((2 * N, 2 * N))
    J[:N, N:] = np.eye(N)
    for i in range(N):
        kr = k[i + 1] if i + 1 < N else 0.0
        J[N + i, i] = -(k[i] + kr)
        if i > 0:
            J[N + i, i - 1] = k[i]
        if i + 1 < N:
            J[N + i, i + 1] = k[i + 1]
        J[N + i, N + i] = -damping
    return J


@pytest.mark.parametrize("masses", [2, 16, 17, 33, 48, 49, 64])
@pytest.mark.parametrize("hb", [1e-6, 1e-3, 0.3])
def test_stiff_chain_matrices(oracle, masses, hb):
    rng = np.random.default_rng(masses)
    k = 10.0 ** (6.0 * rng.random(masses))
    J = _chain_jacobian(k, 2.0 * np.sqrt(k.max()))
    M = np.eye(2 * masses) - hb * J
    b = rng.standard_normal(2 * masses)
    x = oracle.corrected_linsolve(M, b)
    assert x is not None
    assert _residual(M, x, b) < 1e-13 * 2 * masses


@pytest.mark.parametrize("n", [40, 97, 128])
def test_pivoting_forced(oracle, n):
    """A tiny leading diagonal forces row swaps at every pivot; the solve is
    still accurate."""
    rng = np.random.default_rng(7 * n)
    A = rng.standard_normal((n, n))
    A[np.arange(n), np.arange(n)] *= 1e-12
    b = rng.standard_normal(n)
    x = oracle.corrected_linsolve(A, b)
    assert x is not None
    assert _residual(A, x, b) < 1e-12 * n


def test_zero_pivot_reported(oracle):
    A = np.zeros((5, 5))
    A[0, 0] = 1.0
    assert oracle.corrected_linsolve(A, np.ones(5)) is None


def test_secant_fallbacks_full_pivot_lu_and_qr(oracle):
    """secant inverts its finite-difference Jacobian with nalgebra's LU, then
    full-pivot LU, then QR, then fails with SingularMatrix
    (src/ivp/bdf.rs:429-443).  The "+" finite difference makes the columns
    nearly equal, so the fallbacks are reached on multi-dimensional systems.
    Matrices with one row a multiple of another (exactly singular before
    rounding) take each path: the rounding of the elimination decides which
    factorisation ends with an exactly zero pivot."""
    rng = np.random.default_rng(3)
    A = rng.normal(size=(4, 4))
    which, inv = oracle.bdf_secant_inverse(A)
    assert which == 1
    np.testing.assert_allclose(A @ inv, np.eye(4), atol=1e-12)
    r0 = np.array([3 / 7, 0.2, 1 / 3])
    full = np.stack([r0, np.array([1.5, -0.6, -1.0]), r0 * 0.3])
    which, inv = oracle.bdf_secant_inverse(full)
    assert which == 2 and np.all(np.isfinite(inv))
    q0 = np.array([5.0, 3 / 7])
    which, inv = oracle.bdf_secant_inverse(np.stack([q0, q0 * 0.5]))
    assert which == 3 and np.all(np.isfinite(inv))
    which, inv = oracle.bdf_secant_inverse(np.array([[0.0, 1.0], [0.0, 1.0]]))
    assert which == 0 and inv is None
