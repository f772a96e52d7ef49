"""The C ABI from a plain C program (tests/c_caller/solve_vdp.c), built with
the system C compiler against include/bacon_gb300.h and the engine's shared
library, as a foreign caller (the Rust crate's FFI, cgo, ...) would bind it:
its results equal the Python harness's solve of the same batch bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 2048


def _inputs():
    i = np.arange(N)
    y0 = np.empty((2, N))
    y0[0] = -2.0 + 4.0 * ((i * 37) % 101) / 100.0
    y0[1] = -2.0 + 4.0 * ((i * 53) % 103) / 102.0
    mu = 0.1 + 1.9 * ((i * 29) % 97) / 96.0
    return y0, mu[None, :]


def test_c_program_matches_python_harness(engine, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib_dir = os.path.join(ROOT, "bacon_gb300", "_lib")
    bdir = os.path.join(ROOT, "tests", "c_caller", "_build")
    os.makedirs(bdir, exist_ok=True)
    exe = os.path.join(bdir, "solve_vdp")
    subprocess.run([cc, "-std=c11", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_caller", "solve_vdp.c"), "-L", lib_dir, "-lbacon_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    out = tmp_path / "vdp.bin"
    subprocess.run([exe, str(out)], check=True)
    raw = out.read_bytes()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    assert n == N
    off = 8
    y = np.frombuffer(raw[off:off + 16 * n], np.float64).reshape(2, n)
    off += 16 * n
    t = np.frombuffer(raw[off:off + 8 * n], np.float64)
    off += 8 * n
    acc, rej, st = (np.frombuffer(raw[off + 4 * n * k:off + 4 * n * (k + 1)], np.int32) for k in range(3))
    code = int(np.frombuffer(raw[off + 12 * n:off + 12 * n + 4], np.int32)[0])

    y0, mu = _inputs()
    ref = engine.rk_solve(y0, mu, 0.0, 10.0, rhs=5, tol=1e-6, dt_min=1e-6, dt_max=0.1, layout=2)
    assert code == ref.code == 0
    np.testing.assert_array_equal(y, ref.y)
    np.testing.assert_array_equal(t, ref.t)
    np.testing.assert_array_equal(acc, ref.accepted)
    np.testing.assert_array_equal(rej, ref.rejected)
    np.testing.assert_array_equal(st, ref.status)
