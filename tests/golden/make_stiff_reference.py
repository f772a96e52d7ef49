"""Regenerates tests/golden/stiff_reference.npz: rtol-1e-12 final states of
64 Robertson systems of the stiff workload, for the external accuracy check of
the corrected BDF.

The systems are evenly spaced through the Robertson half of the 131,072-system
stiff batch (workloads.stiff_batch(131072), seed 8).  Each is integrated to
t = 1e4 with scipy's Radau at rtol 1e-12, atol 1e-14 and the analytic
Jacobian.  Radau takes ~0.6 s per system here, which is why the states are
frozen in a fixture instead of recomputed in every test run.
Run from the repository root:  python tests/golden/make_stiff_reference.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bacon_gb300 import accuracy as A  # noqa: E402
from bacon_gb300 import workloads as W  # noqa: E402

N_SYSTEMS = 64
T_END = 1e4


def main():
    rob, _ = W.stiff_batch(131072)
    idx = np.linspace(0, rob.n - 1, N_SYSTEMS).astype(np.int64)
    ref = np.empty((3, N_SYSTEMS))
    for j, i in enumerate(idx):
        ref[:, j] = A.robertson_reference(rob.y0[:, i], rob.params[:, i], T_END)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "stiff_reference.npz")
    np.savez_compressed(path, robertson_index=idx, robertson_params=rob.params[:, idx],
                        robertson_y0=rob.y0[:, idx], robertson_t_end=np.array(T_END), robertson_y=ref,
                        rtol=np.array(1e-12), atol=np.array(1e-14))
    print("wrote", path)


if __name__ == "__main__":
    main()
