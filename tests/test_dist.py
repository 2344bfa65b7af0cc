"""Multi-rank plumbing of bench.py on CPU: two gloo ranks (127.0.0.1), each an independent
replica; the job time is the slowest rank's and the rate counts every rank's changes.  The
reference arm does its work on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "DSSSP_BENCH_BACKEND": "gloo"})
    import bench

    d = bench.Dist()
    assert d.world == world and d.rank == rank
    d.barrier()
    rate, t_max = bench.whole_job_rate(d, batch=1000, steps=10, local_seconds=0.5 + rank)
    ref_rc = bench.run_reference(type("A", (), {"workload": "er10k", "steps": 1, "warmup": 0, "gpus": world})(), d) \
        if rank != 0 else 0
    d.close()
    out[rank] = (rate, t_max, ref_rc)


def test_two_rank_replicas_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    for rank in range(world):
        rate, t_max, ref_rc = res[rank]
        assert t_max == pytest.approx(1.5)               # slowest rank
        assert rate == pytest.approx(2 * 1000 * 10 / 1.5)  # all ranks' work / slowest time
        assert ref_rc == 0                                 # non-zero ranks exit without work
