"""World-size-2 gloo test of the sharded (replicas / weak-scaling) path on
CPU: each rank solves its contiguous shard with the CPU oracle, the shards
gather back to the single-process result bit for bit, and the max-over-ranks
reduction returns the slowest rank's time."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from bacon_gb300 import distributed as D
from bacon_gb300 import workloads as W


def test_shard_ranges_cover_batch():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            spans = [D.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    b = W.van_der_pol(n=512, seed=17)
    sb = D.shard(b, rank, world)
    cfg = O.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    r = O.rk_solve_batch(cfg, sb.rhs, sb.y0, sb.params, sb.t0, sb.t_end, threads=1)
    y = D.gather_columns(r["y"], b.n, dist)
    acc = D.gather_columns(r["accepted"][None, :], b.n, dist)[0]
    slowest = D.max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        np.savez(os.path.join(out_dir, "gathered.npz"), y=y, acc=acc, slowest=slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shards_match_single_process(tmp_path, oracle):
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    g = np.load(tmp_path / "gathered.npz")
    b = W.van_der_pol(n=512, seed=17)
    cfg = oracle.rk_cfg(layout=2, tol=b.tol, dt_min=b.dt_min, dt_max=b.dt_max)
    r = oracle.rk_solve_batch(cfg, b.rhs, b.y0, b.params, b.t0, b.t_end, threads=2)
    np.testing.assert_array_equal(g["y"], r["y"])
    np.testing.assert_array_equal(g["acc"], r["accepted"])
    assert float(g["slowest"]) == 2.0
