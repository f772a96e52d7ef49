"""Regenerates tests/golden/rk_golden.npz from the CPU oracle.

The Rust reference cannot be built in this environment, so these fixtures are
oracle outputs (parity unpinned against the compiled reference); they freeze
the restatement so that later changes to it, and the GPU engine on a machine
without a compiler for the oracle, are checked against fixed bits.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bacon_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = [
    # name, batch, method, layout, cap
    ("vdp_compiled", W.van_der_pol(n=16, seed=101), 0, 0, 20000),
    ("vdp_written", W.van_der_pol(n=16, seed=102), 0, 1, 20000),
    ("vdp_fehlberg", W.van_der_pol(n=16, seed=103), 0, 2, 0),
    ("vdp_rk23", W.van_der_pol(n=16, seed=104), 1, 1, 0),
    ("lorenz_fehlberg", W.lorenz(n=16, seed=105), 0, 2, 0),
    ("lotka_fehlberg", W.lotka_volterra(n=16, seed=106), 0, 2, 0),
]


def main():
    out = {}
    for name, b, method, layout, cap in CASES:
        t_end = float(np.min(b.t_end)) if b.rhs == W.RHS_LORENZ else float(b.t_end[0])
        cfg = O.rk_cfg(method=method, layout=layout, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, max_attempts=cap)
        r = O.rk_solve_batch(cfg, b.rhs, b.y0, b.params, 0.0, t_end, threads=2)
        out[f"{name}:cfg"] = np.array([b.rhs, method, layout, b.tol, b.dt_min, b.dt_max, t_end])
        out[f"{name}:cap"] = np.array(cap)
        out[f"{name}:y0"] = b.y0
        out[f"{name}:params"] = b.params
        for k in ("y", "t", "accepted", "rejected", "status"):
            out[f"{name}:{k}"] = r[k]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rk_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
