"""The N > 1 bench path on CPU: two gloo ranks (127.0.0.1) take disjoint systems
and agree on the maximum of their timings; the whole-job rate counts every
rank's systems over the slowest rank. The reference arm does nothing on rank 1."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = bench.dist_env()
    seeds = [sh["seed"] for sh in bench.rank_shapes(8, 2024, r)]
    ms = bench.max_over_ranks([100.0 + 50.0 * r, 10.0 * (r + 1)], w, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, seeds, ms))


def test_two_gloo_ranks_shard_and_take_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict((r, (seeds, ms)) for r, seeds, ms in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert not set(out[0][0]) & set(out[1][0])          # no system on both ranks
    assert out[0][1] == out[1][1] == [150.0, 20.0]      # element-wise max over ranks
    import bench
    assert bench.whole_job_rate(2, 8, 150.0) == pytest.approx(2 * 8 / 0.150)


def test_reference_arm_is_silent_on_other_ranks(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    import argparse
    ns = argparse.Namespace(gpus=2, steps=1, warmup=3, nsys=64, seed=2024, ngrid=8)
    assert bench.run_reference(ns) is None
    assert capsys.readouterr().out == ""
