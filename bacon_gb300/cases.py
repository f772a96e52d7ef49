"""Run one benchmark workload once, device-resident, and print a JSON summary.

    python -m bacon_gb300.cases lorenz --n 131072 [--precision fp32_comp] [--tuned 1,256,4]
    python -m bacon_gb300.cases stiff --n 8192
    python -m bacon_gb300.cases chains --n 4096
    python -m bacon_gb300.cases linear --n 8192 [--precision tc_split]
    python -m bacon_gb300.cases adjoint --n 16384
    python -m bacon_gb300.cases vdp --n 4096
    python -m bacon_gb300.cases adams --n 4096 [--t-end 1]

Each case generates the workload's seeded batch at the given size (the
workload generators in workloads.py), solves it `--repeat` times through the
engine's public calls and prints the last solve's kernel time and status
counts.  It is the small, self-contained command the profiles cite.
``--tuned VARIANT,BLOCK,CTAS_PER_SM`` pins the RK kernel variant and launch
shape (bacon_rk_set_tuned), e.g. the ones the benchmark's autotuner chose.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import engine as E
from . import workloads as W

PRECISION = {"fp64_exact": E.FP64_EXACT, "fp64_fma": E.FP64_FMA, "fp32_comp": E.FP32_COMP,
             "tc_split": E.TC_SPLIT}


def _dev(torch, *xs):
    return [torch.from_numpy(np.ascontiguousarray(x)).to("cuda") for x in xs]


def _ragged_dev(torch, r):
    return W.RaggedBatch(r.name, r.rhs, *_dev(torch, r.y_off, r.p_off, r.y0, r.params, r.t0, r.t_end),
                         r.tol, r.dt_min, r.dt_max, r.seed)


def _uniform_dev(torch, b):
    return W.Batch(b.name, b.rhs, *_dev(torch, b.y0, b.params, b.t0, b.t_end), b.tol, b.dt_min, b.dt_max, b.seed)


def _counts(status):
    s = status.cpu().numpy() if hasattr(status, "cpu") else np.asarray(status)
    return {int(k): int((s == k).sum()) for k in np.unique(s)}


def run(case: str, n: int, precision: str, repeat: int, tuned: tuple | None = None, t_end: float = 10.0) -> dict:
    import torch
    ctx = E.Context(0)
    prec = PRECISION[precision]
    out: dict = {"case": case, "n": n, "precision": precision}
    for _ in range(repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if case in ("lorenz", "vdp"):
            b = W.lorenz(n=n) if case == "lorenz" else W.van_der_pol(n=n)
            y0, p, ts, te = _dev(torch, b.y0, b.params, b.t0, b.t_end)
            if tuned is not None:
                E.rk_set_tuned(y0, rhs=b.rhs, variant=tuned[0], block=tuned[1], blocks_per_sm=tuned[2],
                               layout=E.FEHLBERG, precision=prec, ctx=ctx)
            s = E.rk_solve(y0, p, ts, te, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                           layout=E.FEHLBERG, precision=prec, ctx=ctx)
            out["status"] = _counts(s.status)
        elif case == "linear":
            b = W.linear_shared(n=n)
            y0, A = _dev(torch, b.y0, b.extra["A"])
            s = E.rk_solve(y0, None, 0.0, 5.0, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                           layout=E.FEHLBERG, precision=prec, ctx=ctx, shared=A)
            out["status"] = _counts(s.status)
        elif case == "adams":
            b = W.van_der_pol(n=n)
            y0, p = _dev(torch, b.y0, b.params)
            s = E.adams_solve(y0, p, 0.0, t_end, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max, order=5,
                              ctx=ctx)
            out["status"] = _counts(s.status)
        elif case == "adjoint":
            b = W.lotka_volterra(n=n)
            y0, p, tgt = _dev(torch, b.y0, b.params, b.extra["target"])
            a = E.rk_solve_adjoint(y0, p, 0.0, 15.0, tgt, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min,
                                   dt_max=b.dt_max, ctx=ctx)
            out["status"] = _counts(a.forward.status)
            out["reverse_ms"] = ctx.last_reverse_ms()
            out["record_ms"] = ctx.last_kernel_ms()
        elif case in ("stiff", "chains"):
            if case == "stiff":
                rob, ch = W.stiff_batch(n)
                u = _uniform_dev(torch, rob)
            else:
                u, ch = None, W.ragged_spring_chains(n=n)
            us, rs = E.bdf_solve_mixed(u, _ragged_dev(torch, ch), ctx=ctx)
            out["chain_status"] = _counts(rs.status)
            out["chain_accepted_mean"] = float(rs.accepted.double().mean().item())
            if us is not None:
                out["uniform_status"] = _counts(us.status)
        else:
            raise SystemExit(f"unknown case {case}")
        torch.cuda.synchronize()
        out["wall_s"] = time.perf_counter() - t0
        out["kernel_ms"] = ctx.last_kernel_ms()
    return out


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case", choices=["lorenz", "vdp", "adams", "linear", "adjoint", "stiff", "chains"])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--precision", default="fp64_exact", choices=sorted(PRECISION))
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--tuned", default=None, help="VARIANT,BLOCK,CTAS_PER_SM for lorenz / vdp")
    ap.add_argument("--t-end", type=float, default=10.0, help="end time of the adams case (the workload's is 10)")
    a = ap.parse_args()
    tuned = tuple(int(x) for x in a.tuned.split(",")) if a.tuned else None
    if tuned is not None and len(tuned) != 3:
        raise SystemExit("--tuned wants VARIANT,BLOCK,CTAS_PER_SM")
    print(json.dumps(run(a.case, a.n, a.precision, a.repeat, tuned, a.t_end)))


if __name__ == "__main__":
    main()
