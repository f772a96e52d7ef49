"""Right-hand sides compiled by the caller (bacon_rk_solve_user).

The reference's derivative is any Rust closure (src/ivp.rs:34-48); the
engine's counterpart for systems outside its registry is a functor the
caller compiles into the persistent kernel with include/bacon_gb300_rhs.cuh.
The test compiles tests/user_rhs/user_rhs.cu with nvcc into a shared
library, as a user would, and solves through the C ABI:
- a copy of the registry's Van der Pol must give the registry's bits;
- a forced Duffing oscillator, which the registry lacks, must match scipy's
  DOP853 at rtol 1e-12 to the accuracy its tolerance allows.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from bacon_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "user_rhs", "user_rhs.cu")


@pytest.fixture(scope="module")
def user_lib():
    """The caller's library, built in-tree (tests/user_rhs/_build, not
    tracked) as a user's build would place it."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    bdir = os.path.join(ROOT, "tests", "user_rhs", "_build")
    os.makedirs(bdir, exist_ok=True)
    out = os.path.join(bdir, "libuser_rhs.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3",
                    "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "bacon_gb300", "csrc"), SRC, "-o", out], check=True)
    return ctypes.CDLL(out)


def _solve_user(engine, lib, launcher, y0, params, t0, t_end, tol, dt_min, dt_max, precision=0, layout=2,
                systems_per_warp=0):
    from bacon_gb300 import _capi
    prob = engine.make_problem(y0, params, t0, t_end, tol, dt_min, dt_max, 11)  # BACON_RHS_USER
    opts = engine.rk_options(layout=layout, precision=precision, systems_per_warp=systems_per_warp)
    out = engine.alloc_outputs(y0.shape[0], y0.shape[1], device=False)
    res = engine.make_result(out)
    fn = ctypes.cast(getattr(lib, launcher), ctypes.c_void_p)
    code = _capi.load().bacon_rk_solve_user(engine.default_context().handle, ctypes.byref(prob), ctypes.byref(opts),
                                            ctypes.byref(res), fn, None)
    return code, out


def test_user_van_der_pol_is_the_registry_bit_for_bit(engine, user_lib):
    b = W.van_der_pol(n=2048, seed=51)
    ref = engine.rk_solve(b.y0, b.params, 0.0, 10.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=2)
    for precision in (0, 1):
        if precision == 1:
            ref = engine.rk_solve(b.y0, b.params, 0.0, 10.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min,
                                  dt_max=b.dt_max, layout=2, precision=1)
        for spw in (0, 8):
            code, out = _solve_user(engine, user_lib, "user_vdp_launch", b.y0, b.params, 0.0, 10.0, b.tol,
                                    b.dt_min, b.dt_max, precision=precision, systems_per_warp=spw)
            assert code == ref.code == 0
            np.testing.assert_array_equal(out["y"], ref.y)
            np.testing.assert_array_equal(out["accepted"], ref.accepted)
            np.testing.assert_array_equal(out["rejected"], ref.rejected)


def test_user_duffing_vs_dop853(engine, user_lib):
    from scipy.integrate import solve_ivp
    rng = np.random.default_rng(52)
    n = 64
    prm = np.stack([rng.uniform(0.1, 0.3, n), rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n),
                    rng.uniform(0.2, 0.5, n), rng.uniform(0.8, 1.4, n)])
    y0 = rng.uniform(-1.0, 1.0, (2, n))
    code, out = _solve_user(engine, user_lib, "user_duffing_launch", y0, prm, 0.0, 20.0, 1e-8, 1e-10, 0.05)
    assert code == 0 and (out["status"] == 0).all()
    worst = 0.0
    for i in range(n):
        d, a, bb, g, w = prm[:, i]
        f = lambda t, y: [y[1], g * np.cos(w * t) - d * y[1] - a * y[0] - bb * y[0] ** 3]  # noqa: E731
        s = solve_ivp(f, (0.0, 20.0), y0[:, i], method="DOP853", rtol=1e-12, atol=1e-12)
        worst = max(worst, float(np.abs(out["y"][:, i] - s.y[:, -1]).max()))
    assert worst <= 1e-5, worst


def test_unsupported_combination_reported(engine, user_lib):
    """The FP32-stage mode is not compiled by the launcher: UNSUPPORTED."""
    b = W.van_der_pol(n=32, seed=53)
    code, _ = _solve_user(engine, user_lib, "user_vdp_launch", b.y0, b.params, 0.0, 1.0, b.tol, b.dt_min, b.dt_max,
                          precision=2)
    assert code == 16
