"""Seeded synthetic batches for the five benchmark workloads.

The reference (aftix/bacon) publishes no benchmark inputs, so every batch is
generated here from a fixed numpy seed with the shapes and value
distributions of the workload description.  Arrays are SoA: ``y0`` is
(dim, n), ``params`` is (n_params, n).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

RHS_EXP, RHS_DECAY, RHS_QUADRATIC, RHS_SINE, RHS_HARMONIC = 0, 1, 2, 3, 4
RHS_VDP, RHS_LORENZ, RHS_LOTKA, RHS_ROBERTSON, RHS_CHAIN, RHS_LINEAR = 5, 6, 7, 8, 9, 10


@dataclass
class Batch:
    name: str
    rhs: int
    y0: np.ndarray          # (dim, n)
    params: np.ndarray      # (n_params, n)
    t0: np.ndarray          # (n,)
    t_end: np.ndarray       # (n,)
    tol: float
    dt_min: float
    dt_max: float
    seed: int
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.y0.shape[1]

    @property
    def dim(self) -> int:
        return self.y0.shape[0]

    def subset(self, idx) -> "Batch":
        idx = np.asarray(idx)
        return Batch(self.name, self.rhs, np.ascontiguousarray(self.y0[:, idx]),
                     np.ascontiguousarray(self.params[:, idx]), self.t0[idx].copy(),
                     self.t_end[idx].copy(), self.tol, self.dt_min, self.dt_max, self.seed,
                     dict(self.extra))


def van_der_pol(n: int = 4096, seed: int = 1) -> Batch:
    """4096 Van der Pol oscillators y'' = mu (1 - y^2) y' - y as 2-dim systems:
    mu ~ U[0.1, 2], y0 ~ U[-2, 2]^2, t in [0, 10], tol 1e-6, dt in [1e-6, 0.1]."""
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.1, 2.0, n)
    y0 = rng.uniform(-2.0, 2.0, (2, n))
    return Batch("van_der_pol", RHS_VDP, y0, mu[None, :].copy(), np.zeros(n), np.full(n, 10.0),
                 1e-6, 1e-6, 0.1, seed)


def lorenz(n: int = 1 << 20, seed: int = 2) -> Batch:
    """Lorenz-63 batch: sigma ~ U[9, 11], rho ~ U[20, 30], beta ~ U[2.4, 2.9],
    y0 ~ N(0, 5^2 I), end time T ~ U[1, 20] (uneven work), tol 1e-6.
    dt bounds are not given by the workload; dt_min 1e-8, dt_max 0.1 chosen."""
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(9.0, 11.0, n)
    rho = rng.uniform(20.0, 30.0, n)
    beta = rng.uniform(2.4, 2.9, n)
    y0 = rng.normal(0.0, 5.0, (3, n))
    t_end = rng.uniform(1.0, 20.0, n)
    return Batch("lorenz", RHS_LORENZ, y0, np.stack([sigma, rho, beta]), np.zeros(n), t_end,
                 1e-6, 1e-8, 0.1, seed)


def lotka_volterra(n: int = 1 << 18, seed: int = 3) -> Batch:
    """Lotka-Volterra dx = a x - b x y, dy = c x y - d y: a,b,c,d ~ U[0.5, 1.5],
    y0 ~ U[0.5, 2]^2, t in [0, 15], tol 1e-7, target ~ U[0.5, 2]^2.
    dt bounds chosen: dt_min 1e-8, dt_max 0.1."""
    rng = np.random.default_rng(seed)
    prm = rng.uniform(0.5, 1.5, (4, n))
    y0 = rng.uniform(0.5, 2.0, (2, n))
    target = rng.uniform(0.5, 2.0, (2, n))
    return Batch("lotka_volterra", RHS_LOTKA, y0, prm, np.zeros(n), np.full(n, 15.0),
                 1e-7, 1e-8, 0.1, seed, {"target": target, "checkpoint_every": 32})


def robertson(n: int = 1 << 16, seed: int = 5) -> Batch:
    """Robertson kinetics: k1 ~ 1e-2 U[2,6], k2 ~ 1e7 U[1,5], k3 ~ 1e4 U[0.5,2],
    y0 = (1, 0, 0), t in [0, 1e4], tol 1e-6; dt bounds chosen 1e-10 .. 1e3."""
    rng = np.random.default_rng(seed)
    k1 = 1e-2 * rng.uniform(2.0, 6.0, n)
    k2 = 1e7 * rng.uniform(1.0, 5.0, n)
    k3 = 1e4 * rng.uniform(0.5, 2.0, n)
    y0 = np.zeros((3, n))
    y0[0] = 1.0
    return Batch("robertson", RHS_ROBERTSON, y0, np.stack([k1, k2, k3]), np.zeros(n),
                 np.full(n, 1e4), 1e-6, 1e-10, 1e3, seed)


def spring_chains(n: int = 1 << 15, masses: int = 4, seed: int = 6) -> Batch:
    """Damped spring-mass chains with `masses` unit masses (dim 2*masses):
    stiffness k_i = 10^U[0, 6] (ratio up to 1e6), damping c = 2 sqrt(max k)
    on every mass (critical for the stiffest spring, so the stiff modes are
    real and decaying), x0 ~ U[-1, 1], v0 = 0, t in [0, 10], tol 1e-6.
    Damping, end time and dt bounds (1e-12 .. 1) are not given by the
    workload description and are chosen here."""
    rng = np.random.default_rng(seed)
    k = 10.0 ** rng.uniform(0.0, 6.0, (masses, n))
    c = 2.0 * np.sqrt(k.max(axis=0))
    y0 = np.zeros((2 * masses, n))
    y0[:masses] = rng.uniform(-1.0, 1.0, (masses, n))
    return Batch(f"spring_chain_{masses}", RHS_CHAIN, y0, np.concatenate([k, c[None, :]]), np.zeros(n),
                 np.full(n, 10.0), 1e-6, 1e-12, 1.0, seed)


def linear_shared(n: int = 1 << 16, dim: int = 256, seed: int = 4) -> Batch:
    """y' = A y with one shared A = Q diag(-lambda) Q^T (Q orthogonal from the
    QR factorisation of a Gaussian matrix, lambda log-uniform in [1e-2, 1e1]),
    y0 ~ N(0, I), t in [0, 5], tol 1e-8.  dt bounds chosen: 1e-10 .. 0.1.
    The exact solution is Q diag(exp(-lambda t)) Q^T y0 (extra["exact"])."""
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(dim, dim)))
    q = q * np.sign(np.diag(r))
    lam = 10.0 ** rng.uniform(-2.0, 1.0, dim)
    A = (q * -lam) @ q.T
    y0 = rng.normal(size=(dim, n))

    def exact(t: float, cols=slice(None)):
        return q @ (np.exp(-lam * t)[:, None] * (q.T @ y0[:, cols]))

    return Batch("linear_shared", RHS_LINEAR, y0, np.zeros((0, n)), np.zeros(n), np.full(n, 5.0),
                 1e-8, 1e-10, 0.1, seed, {"A": np.ascontiguousarray(A), "Q": q, "lambda": lam,
                                          "exact": exact})


@dataclass
class RaggedBatch:
    """Systems of one right-hand side with uneven sizes, packed flat: system
    i's state is y0[y_off[i]:y_off[i+1]], its parameters
    params[p_off[i]:p_off[i+1]]."""
    name: str
    rhs: int
    y_off: np.ndarray       # (n+1,) int64
    p_off: np.ndarray       # (n+1,) int64
    y0: np.ndarray          # (y_off[n],)
    params: np.ndarray      # (p_off[n],)
    t0: np.ndarray          # (n,)
    t_end: np.ndarray       # (n,)
    tol: float
    dt_min: float
    dt_max: float
    seed: int

    @property
    def n(self) -> int:
        return self.y_off.shape[0] - 1

    @property
    def dims(self) -> np.ndarray:
        return np.diff(self.y_off)

    def system(self, i: int):
        """(y0_i, params_i) of system i."""
        return (self.y0[self.y_off[i]:self.y_off[i + 1]], self.params[self.p_off[i]:self.p_off[i + 1]])

    def subset(self, idx) -> "RaggedBatch":
        idx = np.asarray(idx)
        ys = [self.y0[self.y_off[i]:self.y_off[i + 1]] for i in idx]
        ps = [self.params[self.p_off[i]:self.p_off[i + 1]] for i in idx]
        y_off = np.concatenate([[0], np.cumsum([len(y) for y in ys])]).astype(np.int64)
        p_off = np.concatenate([[0], np.cumsum([len(p) for p in ps])]).astype(np.int64)
        return RaggedBatch(self.name, self.rhs, y_off, p_off,
                           np.concatenate(ys) if ys else np.zeros(0),
                           np.concatenate(ps) if ps else np.zeros(0), self.t0[idx].copy(),
                           self.t_end[idx].copy(), self.tol, self.dt_min, self.dt_max, self.seed)


def ragged_spring_chains(n: int = 1 << 16, min_masses: int = 2, max_masses: int = 64,
                         seed: int = 7) -> RaggedBatch:
    """Damped spring-mass chains of uneven length: m_i ~ U{min..max} unit
    masses (dim 2 m_i), with spring_chains' value distributions per system:
    k = 10^U[0, 6] (stiffness ratio up to 1e6), c = 2 sqrt(max k), x0 ~
    U[-1, 1], v0 = 0, t in [0, 10], tol 1e-6, dt in [1e-12, 1]."""
    rng = np.random.default_rng(seed)
    m = rng.integers(min_masses, max_masses + 1, n)
    y_off = np.concatenate([[0], np.cumsum(2 * m)]).astype(np.int64)
    p_off = np.concatenate([[0], np.cumsum(m + 1)]).astype(np.int64)
    y0 = np.zeros(int(y_off[-1]))
    params = np.empty(int(p_off[-1]))
    for i in range(n):
        mi = int(m[i])
        k = 10.0 ** rng.uniform(0.0, 6.0, mi)
        params[p_off[i]:p_off[i] + mi] = k
        params[p_off[i] + mi] = 2.0 * np.sqrt(k.max())
        y0[y_off[i]:y_off[i] + mi] = rng.uniform(-1.0, 1.0, mi)
    return RaggedBatch("ragged_spring_chains", RHS_CHAIN, y_off, p_off, y0, params, np.zeros(n),
                       np.full(n, 10.0), 1e-6, 1e-12, 1.0, seed)


def stiff_batch(n: int = 131072, seed: int = 8):
    """The stiff BDF6 batch: n/2 Robertson systems (robertson()) and n/2
    spring-mass chains with m ~ U{2..64} masses (ragged_spring_chains()).
    Returns (Batch, RaggedBatch)."""
    half = n // 2
    return robertson(n=half, seed=seed), ragged_spring_chains(n=n - half, seed=seed + 1)
