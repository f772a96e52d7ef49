#!/usr/bin/env python3
"""Benchmark: batched RK45 solves/s of the GB300 engine.

One step = one batched solve of 1,048,576 independent Lorenz-63 systems
(sigma ~ U[9,11], rho ~ U[20,30], beta ~ U[2.4,2.9], y0 ~ N(0, 5^2 I),
end times T ~ U[1,20], tol 1e-6) with the RKF45 engine in FP64 arithmetic that
is bit-identical to the CPU restatement of the reference (tableau variant
"fehlberg": the reference's as-compiled matrix does not integrate these
systems).  Inputs are generated from fixed seeds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl bacon|reference]

Under torchrun every rank solves its own batch of the same size (weak
scaling, no collective on the data path); the reported value is the total
over ranks divided by the slowest rank's time.  ``--impl reference`` times
the CPU restatement of the reference solver on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched RK45 solves/s & adjoint grads/s @rtol 1e-6 vs plain GPU RK45 & CPU"
UNIT = "solves/s"
L2_FLUSH_BYTES = 256 << 20   # larger than the 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="bacon", choices=["bacon", "reference"])
    ap.add_argument("--n", type=int, default=1 << 20, help="systems per GPU")
    ap.add_argument("--cpu-sample", type=int, default=16384, help="systems in the CPU sample")
    ap.add_argument("--skip-extras", action="store_true", help="skip plain/FMA/CPU side measurements")
    ap.add_argument("--stiff-n", type=int, default=32768,
                    help="systems of the stiff-batch side measurement (half Robertson, half chains); the "
                         "workload's full size is 131072")
    ap.add_argument("--precision", default="fp64_exact", choices=["fp64_exact", "fp64_fma", "fp32_comp"],
                    help="arithmetic of the timed solve (the headline is fp64_exact)")
    return ap.parse_args()


def workload(n, rank):
    from bacon_gb300 import workloads as W
    return W.lorenz(n=n, seed=2 + rank)


def config(args, b):
    return {"workload": "lorenz63", "n_systems_per_gpu": b.n, "dim": 3, "tol": b.tol,
            "dt_min": b.dt_min, "dt_max": b.dt_max, "t0": 0.0, "t_end": "U[1,20] per system",
            "method": "RKF45", "tableau": "fehlberg", "precision": args.precision,
            "parity": "bit-identical to the CPU restatement (tests/test_rk_gpu.py)",
            "l2": "256 MiB device write before every timed step (inputs ~100 MB fit in L2)",
            "parallelism": f"replicas x{args.gpus} (independent batches, no collective)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return {"unavailable": "nvidia-smi produced no samples"}
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"unavailable": "unparsable nvidia-smi output"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def run_reference(args, rank, world):
    """CPU restatement of the reference solver on the host cores."""
    if rank != 0:
        return
    from oracle import oracle as O
    b = workload(args.n, 0)
    rng = np.random.default_rng(123)
    idx = np.sort(rng.choice(b.n, size=min(args.cpu_sample, b.n), replace=False))
    s = b.subset(idx)
    cfg = O.rk_cfg(layout=O.FEHLBERG, pow_mode=O.POW_LIBM, tol=s.tol, dt_min=s.dt_min, dt_max=s.dt_max)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.rk_solve_batch(cfg, s.rhs, s.y0[:, :256], s.params[:, :256], s.t0[:256], s.t_end[:256], threads=threads)
    secs = []
    for _ in range(args.steps):
        r = O.rk_solve_batch(cfg, s.rhs, s.y0, s.params, s.t0, s.t_end, threads=threads)
        secs.append(r["seconds"])
    value = s.n * len(secs) / sum(secs)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy)", "config": config(args, b),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{s.n} of the {b.n} Lorenz systems per step (seeded subset); "
                                       "C restatement of src/ivp/rk.rs with the platform pow()"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_pool(fn, items, threads):
    """Runs fn over items on `threads` host threads (the oracle's C calls drop
    the GIL); returns (results, seconds)."""
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(fn, items))
    return res, time.perf_counter() - t0


def other_cpu_baselines(W):
    """The CPU restatement timed on bounded samples of the other workloads, on
    all host threads (reported baselines: the GPU numbers are measured on the
    full workloads)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    out = {}
    vb = W.van_der_pol()
    cfg = O.rk_cfg(layout=O.FEHLBERG, pow_mode=O.POW_QRT, tol=vb.tol, dt_min=vb.dt_min, dt_max=vb.dt_max)
    r = O.rk_solve_batch(cfg, vb.rhs, vb.y0, vb.params, vb.t0, vb.t_end, threads=threads)
    out["van_der_pol_4096"] = {"value": vb.n / r["seconds"], "unit": "solves/s", "cores": threads,
                               "sample": "all 4096 systems"}
    lb = W.linear_shared(n=2 * threads)
    cfg = O.rk_cfg(layout=O.FEHLBERG, pow_mode=O.POW_QRT, tol=lb.tol, dt_min=lb.dt_min, dt_max=lb.dt_max)
    r = O.rk_solve_batch(cfg, lb.rhs, lb.y0, np.zeros((0, lb.n)), lb.t0, lb.t_end, shared=lb.extra["A"],
                         threads=threads)
    out["linear_shared_A_256"] = {"value": lb.n / r["seconds"], "unit": "solves/s", "cores": threads,
                                  "sample": f"{lb.n} of the 65536 states (same A)"}
    lv = W.lotka_volterra(n=1 << 18)
    idx = np.arange(0, lv.n, lv.n // (64 * threads))
    cfg = O.rk_cfg(layout=O.FEHLBERG, pow_mode=O.POW_QRT, tol=lv.tol, dt_min=lv.dt_min, dt_max=lv.dt_max)
    _, sec = cpu_pool(lambda i: O.rk_adjoint_one(cfg, lv.rhs, lv.y0[:, i], lv.params[:, i], 0.0, 15.0,
                                                 lv.extra["target"][:, i]), idx, threads)
    out["adjoint"] = {"value": len(idx) / sec, "unit": "grads/s", "cores": threads,
                      "sample": f"{len(idx)} of the 262144 Lotka-Volterra systems"}
    sub = vb.subset(np.arange(0, vb.n, vb.n // (8 * threads)))
    acfg = O.adams_cfg(order=5, tol=sub.tol, dt_min=sub.dt_min, dt_max=sub.dt_max)
    _, sec = cpu_pool(lambda i: O.adams_solve_one(acfg, sub.rhs, sub.y0[:, i], 0.0, 10.0, params=sub.params[:, i]),
                      range(sub.n), threads)
    out["adams5_van_der_pol_4096"] = {"value": sub.n / sec, "unit": "solves/s", "cores": threads,
                                      "sample": f"{sub.n} of the 4096 Van der Pol systems"}
    rob, ch = W.stiff_batch(131072)
    k = 4 * threads
    ri = np.linspace(0, rob.n - 1, k).astype(int)
    ci = np.linspace(0, ch.n - 1, k).astype(int)
    rcfg = O.bdf_cfg(mode=O.BDF_CORRECTED, tol=rob.tol, dt_min=rob.dt_min, dt_max=rob.dt_max)
    ccfg = O.bdf_cfg(mode=O.BDF_CORRECTED, dyn_dim=True, tol=ch.tol, dt_min=ch.dt_min, dt_max=ch.dt_max)

    def one(job):
        kind, i = job
        if kind == 0:
            return O.bdf_solve_one(rcfg, rob.rhs, rob.y0[:, i], 0.0, 1e4, params=rob.params[:, i]).status
        y0, p = ch.system(i)
        return O.bdf_solve_one(ccfg, ch.rhs, y0, 0.0, 10.0, params=p).status

    _, sec = cpu_pool(one, [(0, i) for i in ri] + [(1, i) for i in ci], threads)
    out["bdf6_stiff"] = {"value": 2 * k / sec, "unit": "solves/s", "cores": threads,
                         "sample": f"{k} Robertson + {k} chains (evenly spaced) of the 131072-system batch"}
    return out


def other_workloads(E, W, ctx, dev, torch, stiff_n=131072):
    """The other benchmark workloads, one timed solve each (device-resident)."""
    out = {}

    def to_dev(*xs):
        return [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in xs]

    # Van der Pol, 4096 systems, t in [0, 10] (the CPU-runnable workload).
    vb = W.van_der_pol()
    vy, vp = to_dev(vb.y0, vb.params)
    kw = dict(rhs=vb.rhs, tol=vb.tol, dt_min=vb.dt_min, dt_max=vb.dt_max, layout=E.FEHLBERG, ctx=ctx)
    E.rk_solve(vy, vp, 0.0, 10.0, **kw)
    s = E.rk_solve(vy, vp, 0.0, 10.0, **kw)
    ms = ctx.last_kernel_ms()
    out["van_der_pol_4096"] = {"value": vb.n / (ms * 1e-3), "unit": "solves/s", "kernel_ms": ms,
                               "statuses_ok": bool((s.status == 0).all().item())}

    # The same Van der Pol batch with Adams5 (the reference's predictor-
    # corrector, src/ivp/adams.rs): it restarts from an RK4 bootstrap after
    # every dt change, so it takes ~10^5 step calls per system.
    E.adams_solve(vy, vp, 0.0, 10.0, rhs=vb.rhs, tol=vb.tol, dt_min=vb.dt_min, dt_max=vb.dt_max, order=5, ctx=ctx)
    a5 = E.adams_solve(vy, vp, 0.0, 10.0, rhs=vb.rhs, tol=vb.tol, dt_min=vb.dt_min, dt_max=vb.dt_max, order=5,
                       ctx=ctx)
    ams = ctx.last_kernel_ms()
    st = a5.status.cpu().numpy()
    out["adams5_van_der_pol_4096"] = {
        "value": vb.n / (ams * 1e-3), "unit": "solves/s", "kernel_ms": ams,
        "status_counts": {int(k): int((st == k).sum()) for k in np.unique(st)},
        "step_calls_mean": float((a5.accepted.double() + a5.rejected.double()).mean().item()),
        "step_calls_max": float((a5.accepted.double() + a5.rejected.double()).max().item()),
        "note": "the reference's Adams5 restarts from an RK4 bootstrap after every dt change (~7e5 step calls "
                "per system on average here, step_calls_max for the slowest) and one thread runs each system's "
                "steps serially, each dependent FP64 operation ~64 cycles: the launch lasts as long as the slowest "
                "system, and 4096 systems fill 32 of 152 SMs, so a larger batch, not this one, is where the GPU "
                "pays off"}

    # Linear y' = A y, shared A (n = 256), 65,536 states, tol 1e-8.
    lb = W.linear_shared()
    ly, lA = to_dev(lb.y0, lb.extra["A"])
    lk = dict(rhs=lb.rhs, tol=lb.tol, dt_min=lb.dt_min, dt_max=lb.dt_max, layout=E.FEHLBERG, ctx=ctx, shared=lA)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tc = E.rk_solve(ly, None, 0.0, 5.0, precision=E.TC_SPLIT, **lk)
    torch.cuda.synchronize()
    tc_s = time.perf_counter() - t0
    sub = 8192
    sy_, = to_dev(lb.y0[:, :sub])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fp = E.rk_solve(sy_, None, 0.0, 5.0, precision=E.FP64_FMA, **lk)
    torch.cuda.synchronize()
    fp_s = time.perf_counter() - t0
    exact = lb.extra["exact"](5.0, slice(0, sub))
    out["linear_shared_A_256"] = {
        "tensor_split": {"value": lb.n / tc_s, "unit": "solves/s", "n": lb.n,
                         "max_abs_err_vs_exact_first_8192": float(np.abs(tc.y[:, :sub].cpu().numpy() - exact).max()),
                         "statuses_ok": bool((tc.status == 0).all().item())},
        "fp64_fma": {"value": sub / fp_s, "unit": "solves/s", "n": sub,
                     "max_abs_err_vs_exact": float(np.abs(fp.y.cpu().numpy() - exact).max())},
        "what": "lock-step RKF45 rounds; stage GEMM 256x256 x 256xN on tcgen05 (bf16 5x8-bit slices, FP32 "
                "accumulation exact on the leading diagonals, ~2^-39 product error) vs FP64 DFMA SIMT GEMM; "
                "wall time of the whole solve"}

    # Stiff batch, corrected BDF6, one launch: 65,536 Robertson systems (a
    # thread each) and 65,536 damped spring-mass chains of m ~ U{2..64} masses
    # (dim 4..128, a warp each, factors in shared memory).
    rob, ch = W.stiff_batch(stiff_n)
    u = W.Batch(rob.name, rob.rhs, *to_dev(rob.y0, rob.params, rob.t0, rob.t_end), rob.tol, rob.dt_min, rob.dt_max,
                rob.seed)
    r = W.RaggedBatch(ch.name, ch.rhs, *to_dev(ch.y_off, ch.p_off, ch.y0, ch.params, ch.t0, ch.t_end), ch.tol,
                      ch.dt_min, ch.dt_max, ch.seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    us, rs = E.bdf_solve_mixed(u, r, ctx=ctx)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = ctx.last_kernel_ms()
    out["bdf6_stiff"] = {
        "value": stiff_n / (ms * 1e-3), "unit": "solves/s", "n": stiff_n, "kernel_ms": ms, "wall_s": wall,
        "sample": "full workload" if stiff_n == 131072 else
                  f"{stiff_n} of the workload's 131072 systems, same generator and mix (--stiff-n 131072 for all)",
        "robertson": {"n": rob.n, "t_end": 1e4, "statuses_ok": bool((us.status == 0).all().item()),
                      "accepted_mean": float(us.accepted.double().mean().item())},
        "spring_chains": {"n": ch.n, "dims": "4..128 (m ~ U{2..64} masses)", "t_end": 10.0,
                          "statuses_ok": bool((rs.status == 0).all().item()),
                          "accepted_mean": float(rs.accepted.double().mean().item())},
        "what": "corrected BDF6 (Newton, analytic Jacobian, partial-pivot LU) in one launch: Robertson one "
                "system per thread, chains one per warp with LU factors in shared memory and a 16-entry "
                "factor cache per warp; bit-identical to the CPU restatement (tests/test_bdf_ragged_gpu.py)"}
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    from bacon_gb300 import engine as E
    from bacon_gb300 import roofline as R

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    ctx = E.Context(local)
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)
    b = workload(args.n, rank)
    fp64_peak = ctx.fp64_peak_gflops()

    y0 = torch.from_numpy(b.y0).to(dev)
    prm = torch.from_numpy(b.params).to(dev)
    t0 = torch.from_numpy(b.t0).to(dev)
    te = torch.from_numpy(b.t_end).to(dev)
    out = E.alloc_outputs(3, b.n, device=True)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    prec = {"fp64_exact": E.FP64_EXACT, "fp64_fma": E.FP64_FMA, "fp32_comp": E.FP32_COMP}[args.precision]

    def solve(precision=prec, dst=None):
        return E.rk_solve(y0, prm, t0, te, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                          layout=E.FEHLBERG, precision=precision, out=dst or out, ctx=ctx,
                          raise_on_error=True)

    for _ in range(max(args.warmup, 0)):
        solve()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    step_ms, kern_ms = [], []
    launches0 = ctx.kernel_launches
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            solve()
            e1.record(ext)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            kern_ms.append(ctx.last_kernel_ms())
        barrier()
    wall = time.perf_counter() - wall0
    launches = ctx.kernel_launches - launches0

    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = b.n * world * args.steps / (total_ms * 1e-3)

    acc = out["accepted"].cpu().numpy().astype(np.int64)
    rej = out["rejected"].cpu().numpy().astype(np.int64)
    status = out["status"].cpu().numpy()
    attempts = int(acc.sum() + rej.sum())
    flops = R.rk_flops(0, b.rhs, 3, attempts, int(acc.sum()))
    kavg = sum(kern_ms) / len(kern_ms)
    achieved = flops / (kavg * 1e-3) / 1e12
    peak = fp64_peak / 1e3
    traffic = None
    prof = os.path.join(ROOT, "profiles", "rk_persistent_lorenz_1m.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")

    # ---- end to end: host (pinned) buffers through the C ABI ----
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    hy0, hprm, ht0, hte = pin(b.y0), pin(b.params), pin(b.t0), pin(b.t_end)
    hout = E.alloc_outputs(3, b.n, device=False, pin=True)
    h2d = hy0.nbytes + hprm.nbytes + ht0.nbytes + hte.nbytes
    d2h = sum(hout[k].nbytes for k in ("y", "t", "accepted", "rejected", "status"))
    E.rk_solve(hy0, hprm, ht0, hte, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
               layout=E.FEHLBERG, precision=prec, out=hout, ctx=ctx, raise_on_error=True)
    barrier()
    e2e_s = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        E.rk_solve(hy0, hprm, ht0, hte, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                   layout=E.FEHLBERG, precision=prec, out=hout, ctx=ctx, raise_on_error=True)
        e2e_s.append(time.perf_counter() - s0)
    e2e_total = sum(e2e_s)
    if world > 1:
        t = torch.tensor([e2e_total], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = b.n * world * args.steps / e2e_total
    assert np.array_equal(hout["y"], out["y"].cpu().numpy()), "host and device paths disagree"

    extras = {}
    if not args.skip_extras:
        flush.fill_(1.0)
        torch.cuda.synchronize()
        fout = E.alloc_outputs(3, b.n, device=True)
        s0 = time.perf_counter()
        solve(E.FP64_FMA, fout)
        torch.cuda.synchronize()
        extras["fp64_fma_mode"] = {"value": b.n / (time.perf_counter() - s0), "unit": UNIT,
                                   "note": "same workload, products and sums contracted (not bit-exact)"}
        pout = E.alloc_outputs(3, b.n, device=True)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        E.rk_solve(y0, prm, t0, te, rhs=b.rhs, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max,
                   layout=E.FEHLBERG, out=pout, ctx=ctx, plain=True, raise_on_error=True)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - s0
        same = bool(torch.equal(pout["y"], out["y"]))
        extras["plain_gpu_baseline"] = {
            "value": b.n / plain_s, "unit": UNIT, "identical_results": same,
            "what": "one launch per attempt, state in HBM, dense tableau, host loop until done"}
        extras["speedup_vs_plain"] = value / world / (b.n / plain_s)

        # FP32-stage mode (float-float stages, FP64 control), same workload.
        cout = E.alloc_outputs(3, b.n, device=True)
        solve(E.FP32_COMP, cout)
        comp_ms = []
        for _ in range(2):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            solve(E.FP32_COMP, cout)
            comp_ms.append(ctx.last_kernel_ms())
        comp_value = b.n / (min(comp_ms) * 1e-3)
        extras["fp32_comp_mode"] = {"value": comp_value, "unit": UNIT,
                                    "speedup_vs_fp64_exact": comp_value / (value / world),
                                    "speedup_vs_plain": comp_value / (b.n / plain_s),
                                    "what": "float-float stages on the FP32 pipe, FP64 accept test and dt"}

        # Final-state error against FP64 DOP853 at rtol 1e-12 (sample: T <= 5).
        from bacon_gb300 import accuracy as A
        short = np.flatnonzero(b.t_end <= 5.0)[:32]
        sb = b.subset(short)
        ref = A.reference_final_states(sb)
        extras["final_state_error_vs_rtol1e-12"] = {
            "fp64_exact": A.final_state_error(out["y"].cpu().numpy()[:, short], ref),
            "fp32_comp": A.final_state_error(cout["y"].cpu().numpy()[:, short], ref),
            "sample": f"{short.size} Lorenz systems with T <= 5 (chaotic: error grows with T)"}

        # Discrete adjoint (batched solve_ivp_adjoint) on the Lotka-Volterra workload.
        from bacon_gb300 import workloads as W
        lv = W.lotka_volterra()
        ly0, lprm, ltg = (torch.from_numpy(np.ascontiguousarray(x)).to(dev)
                          for x in (lv.y0, lv.params, lv.extra["target"]))
        lout = E.alloc_outputs(2, lv.n, device=True)
        kw = dict(rhs=lv.rhs, tol=lv.tol, dt_min=lv.dt_min, dt_max=lv.dt_max, ctx=ctx, out=lout)
        E.rk_solve(ly0, lprm, 0.0, 15.0, layout=E.FEHLBERG, **kw)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        E.rk_solve(ly0, lprm, 0.0, 15.0, layout=E.FEHLBERG, **kw)
        fwd_ms = ctx.last_kernel_ms()
        adj = E.rk_solve_adjoint(ly0, lprm, 0.0, 15.0, ltg, layout=E.FEHLBERG, **kw)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        adj = E.rk_solve_adjoint(ly0, lprm, 0.0, 15.0, ltg, layout=E.FEHLBERG, **kw)
        adj_wall = time.perf_counter() - s0
        rec_ms, rev_ms = ctx.last_kernel_ms(), ctx.last_reverse_ms()
        adj_ms = rec_ms + rev_ms
        grad = torch.cat([adj.dl_dy0, adj.dl_dp]).cpu().numpy()
        fd_rel = None
        if rank == 0:
            from oracle import oracle as O
            cfg = O.rk_cfg(layout=O.FEHLBERG, tol=lv.tol, dt_min=lv.dt_min, dt_max=lv.dt_max)
            worst = 0.0
            for i in range(0, lv.n, lv.n // 16):
                _, fy, fp = O.rk_frozen_fd_one(cfg, lv.rhs, lv.y0[:, i], lv.params[:, i], 0.0, 15.0,
                                               lv.extra["target"][:, i], 1e-6)
                g = grad[:, i]
                worst = max(worst, float(np.abs(g - np.concatenate([fy, fp])).max() / np.abs(g).max()))
            fd_rel = worst
        extras["adjoint"] = {
            "value": lv.n / (adj_ms * 1e-3), "unit": "grads/s", "workload": "Lotka-Volterra, 262144 systems, "
            "t in [0,15], tol 1e-7, loss = sum ||y(T)-target||^2, checkpoint every 32 accepted steps",
            "e2e_value": lv.n / adj_wall, "forward_ms": fwd_ms, "adjoint_ms": adj_ms,
            "record_forward_ms": rec_ms, "reverse_ms": rev_ms, "cost_vs_forward": adj_ms / fwd_ms,
            "max_rel_diff_vs_frozen_central_fd_h1e-6": fd_rel, "fd_sample": 16}
        extras.update(other_workloads(E, W, ctx, dev, torch, stiff_n=args.stiff_n))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy, Lorenz-63 batch)", "config": config(args, b),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "measured live (FP64 FMA probe kernel); MEASURED_PEAKS.json has no FP64 entry",
                         "flops_per_launch": flops, "kernel_ms": kavg,
                         "work": "194 flops per attempt + 25 per accepted attempt (bacon_gb300/roofline.py)"},
            "clocks": clocks.summary(), "wall_s_timed_region": wall,
            "statuses_ok": bool((status == 0).all()), "attempts_per_solve": attempts / b.n}
    line.update(extras)

    if rank == 0 and world == 1 and not args.skip_extras:
        from oracle import oracle as O
        rng = np.random.default_rng(123)
        idx = np.sort(rng.choice(b.n, size=min(args.cpu_sample, b.n), replace=False))
        s = b.subset(idx)
        threads = os.cpu_count() or 1
        cfg = O.rk_cfg(layout=O.FEHLBERG, pow_mode=O.POW_QRT, tol=s.tol, dt_min=s.dt_min, dt_max=s.dt_max)
        r = O.rk_solve_batch(cfg, s.rhs, s.y0, s.params, s.t0, s.t_end, threads=threads)
        line["cpu_baseline"] = {
            "value": s.n / r["seconds"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{s.n} of the {b.n} Lorenz systems (seeded subset), all host threads",
            "sample_bit_identical": bool(np.array_equal(r["y"], out["y"].cpu().numpy()[:, idx])
                                         and np.array_equal(r["accepted"], acc[idx]))}
        for name, base in other_cpu_baselines(W).items():
            if isinstance(line.get(name), dict):
                line[name]["cpu_baseline"] = base
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
