"""External accuracy of the GPU's corrected BDF6 on the stiff workload.

The mixed launch is bit-identical to the CPU restatement of the corrected BDF
(tests/test_bdf_ragged_gpu.py), which only shows that the two agree.  Here
the GPU's final states are compared with answers from outside the engine:
- 64 damped spring-mass chains of the workload's generator, one for each
  m = 2..64 masses plus a second m = 64 (dims 4..128), against the exact
  solution expm(J t) y0 (the chains are linear);
- 64 Robertson systems of the workload, evenly spaced through its Robertson
  half, against scipy's Radau at rtol 1e-12 (tests/golden/stiff_reference.npz).
The bound is an absolute max-norm error of 1e-5 at the workload's tol 1e-6
(the engine's error control is absolute, as the reference's).
"""
import os

import numpy as np
import pytest

from bacon_gb300 import accuracy as A
from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stiff_reference.npz")
ABS_BOUND = 1e-5


def test_chains_dims_4_to_128_vs_expm(engine):
    _, ch = W.stiff_batch(131072)
    idx = [int(np.flatnonzero(ch.dims == 2 * m)[0]) for m in range(2, 65)]
    idx.append(int(np.flatnonzero(ch.dims == 128)[1]))
    sub = ch.subset(idx)
    _, rs = engine.bdf_solve_mixed(None, sub)
    assert rs.code == 0 and (rs.status == 0).all()
    worst = 0.0
    for j in range(sub.n):
        y0, p = sub.system(j)
        exact = A.chain_exact_final(y0, p, float(sub.t_end[j]))
        err = np.abs(rs.y[sub.y_off[j]:sub.y_off[j + 1]] - exact).max()
        worst = max(worst, err)
    assert worst <= ABS_BOUND, worst


def test_robertson_vs_radau_rtol_1e12(engine):
    g = np.load(GOLDEN)
    rob, _ = W.stiff_batch(131072)
    sub = rob.subset(g["robertson_index"])
    np.testing.assert_array_equal(sub.params, g["robertson_params"])
    us, _ = engine.bdf_solve_mixed(sub, None)
    assert us.code == 0 and (us.status == 0).all()
    err = np.abs(us.y - g["robertson_y"]).max()
    assert err <= ABS_BOUND, err
