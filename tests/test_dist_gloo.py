"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The analysis has no cross-GPU exchange: under torchrun every rank analyses
its own instance and the job's time is the slowest rank's.  These tests run
the same reduction and aggregation code with the gloo backend.
"""
import os
import socket

import pytest
import torch
import torch.distributed as tdist
import torch.multiprocessing as mp

from conftest import REPO


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, times, out):
    import importlib.util
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench", os.path.join(REPO, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    ms = bench._max_over_ranks(torch, tdist, "cpu", times[rank])
    value = bench.whole_job_columns_per_s(world, 64800, ms)
    tdist.barrier()
    out[rank] = (ms, value)
    tdist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    times = [210.0, 250.0]
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), times, out), nprocs=world, join=True)
    for rank in range(world):
        ms, value = out[rank]
        assert ms == 250.0
        assert value == pytest.approx(2 * 64800 / 0.250)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", os.path.join(REPO, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class Args:
        config, steps, warmup, gpus = 1, 1, 0, 2
    called = []
    monkeypatch.setattr(bench, "pkg", lambda name: called.append(name))
    assert bench.run_reference(Args(), 1, 2) is None
    assert called == []              # rank 1 does no work
