"""Replicas-only multi-GPU path, exercised as world_size-2 gloo ranks on CPU.

bench.py --gpus N runs N independent scenes (seed + rank) with no collective
on the data path; only the timing is reduced (max over ranks) and the value is
all ranks' steps over that time.  Here each rank steps the CPU oracle on its
own scene and the same reduction is checked.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [os.path.join(repo, "fluid-simulation_gb300"), os.path.join(repo, "oracle"), repo]
    import bench
    import oracle
    from fluidgb import scenes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = bench.dist_env()
    assert (r, w) == (rank, world)
    p = scenes.params_for(16, iters=10, tol=0.0)
    parts = scenes.seed_particles(16, scenes.box(0.5, 0.5), seed=scenes.DEFAULT_SEED + rank)
    o = oracle.OracleFluid(p, parts.shape[0])
    o.set_particles(parts)
    steps = 3
    import time
    t0 = time.perf_counter()
    o.step(steps)
    ms = (time.perf_counter() - t0) * 1000.0
    x, _ = o.get_particles()
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    chk = torch.tensor([float(np.float64(x[:, :3].sum()))], dtype=torch.float64)
    allchk = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(allchk, chk)
    value = bench.replica_value(world, steps, float(t.item()))
    out[rank] = (ms, float(t.item()), value, [float(c.item()) for c in allchk])
    dist.destroy_process_group()


def test_two_replicas_reduce_time_and_stay_independent():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(300)
        assert pr.exitcode == 0
    (ms0, max0, v0, c0), (ms1, max1, v1, c1) = out[0], out[1]
    assert max0 == max1 == max(ms0, ms1)
    assert v0 == v1 == pytest.approx(2 * 3 / (max0 / 1000.0))
    assert c0 == c1 and c0[0] != c0[1]  # different seeds -> independent scenes
