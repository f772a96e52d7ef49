"""External accuracy pins of the corrected BDF on the stiff workload, on CPU.

The corrected BDF is this engine's own stiff method, so bit parity with its
CPU restatement says nothing about whether it is accurate.  These checks
compare the restatement with answers from outside it: the exact solution
expm(J t) y0 of the (linear) spring-mass chains, and scipy's Radau at
rtol 1e-12 for Robertson kinetics (frozen in tests/golden/stiff_reference.npz
by tests/golden/make_stiff_reference.py).  The GPU engine is bit-identical to
the restatement; tests/test_stiff_accuracy_gpu.py checks it against the same
answers on the full 64-chain and 64-Robertson samples.
"""
import os

import numpy as np
import pytest

from bacon_gb300 import accuracy as A
from bacon_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stiff_reference.npz")
ABS_BOUND = 1e-5  # max-norm absolute error at tol 1e-6


def test_chain_matrix_matches_rhs(oracle):
    """The Jacobian used for expm is the chain right-hand side itself."""
    _, ch = W.stiff_batch(256)
    for i in range(4):
        y0, p = ch.system(i)
        m = len(y0) // 2
        J = A.chain_matrix(p[:m], p[m])
        y = np.random.default_rng(i).normal(size=2 * m)
        np.testing.assert_allclose(J @ y, oracle.rhs_eval(W.RHS_CHAIN, 0.0, y, params=p), rtol=1e-13, atol=1e-9)


@pytest.mark.parametrize("m", [2, 3, 4, 5])
def test_corrected_bdf_chain_vs_expm(oracle, m):
    _, ch = W.stiff_batch(131072)
    i = int(np.flatnonzero(ch.dims == 2 * m)[0])
    y0, p = ch.system(i)
    cfg = oracle.bdf_cfg(mode=oracle.BDF_CORRECTED, dyn_dim=True, tol=ch.tol, dt_min=ch.dt_min, dt_max=ch.dt_max)
    r = oracle.bdf_solve_one(cfg, ch.rhs, y0, 0.0, 10.0, params=p)
    assert r.status == 0
    assert np.abs(r.y - A.chain_exact_final(y0, p, 10.0)).max() <= ABS_BOUND


def test_fixture_is_radau_rtol_1e12():
    g = np.load(GOLDEN)
    assert g["robertson_y"].shape == (3, 64)
    for j in (0, 37):
        ref = A.robertson_reference(g["robertson_y0"][:, j], g["robertson_params"][:, j],
                                    float(g["robertson_t_end"]))
        np.testing.assert_allclose(ref, g["robertson_y"][:, j], rtol=1e-10, atol=1e-16)


def test_corrected_bdf_robertson_vs_radau(oracle):
    g = np.load(GOLDEN)
    rob, _ = W.stiff_batch(131072)
    cfg = oracle.bdf_cfg(mode=oracle.BDF_CORRECTED, tol=rob.tol, dt_min=rob.dt_min, dt_max=rob.dt_max)
    for j in range(0, 64, 8):
        i = int(g["robertson_index"][j])
        np.testing.assert_array_equal(rob.params[:, i], g["robertson_params"][:, j])
        r = oracle.bdf_solve_one(cfg, rob.rhs, rob.y0[:, i], 0.0, 1e4, params=rob.params[:, i])
        assert r.status == 0
        assert np.abs(r.y - g["robertson_y"][:, j]).max() <= ABS_BOUND
