"""bench.py's multi-GPU mode on CPU ranks.  The assembly path has no data exchange between GPUs:
`--gpus N` under torchrun runs N independent replicas (weak scaling), and the only cross-rank step is
the maximum of the replicas' times.  Two `gloo` ranks check that step; the reference arm does its
work on rank 0 only and the other ranks leave without printing."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, values, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        out.put((rank, bench.max_over_ranks(values[rank])))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("values", [(1.25, 7.5), (9.0, 2.0)])
def test_max_over_two_gloo_ranks(values):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: max(values), 1: max(values)}


def test_max_over_ranks_without_a_process_group():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    args = argparse.Namespace(workload="plate", warmup=3, steps=1, gpus=2)
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
