"""Multi-process host logic of replica runs on CPU (gloo, world size 2):
day shards cover every day once; max over ranks; the cross-shard linear
stack equals one rank stacking all windows (FP64 oracle, relative 1e-12);
the aggregate weak-scaling rate."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from fastxc_gb300 import replicas
    from oracle import xc_oracle as xo

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(0)  # same data on every rank; each stacks its own days
        ndays, nstep, nchan, nspec = 5, 4, 6, 33
        spec = rng.standard_normal((ndays * nstep, nchan, nspec)) + 1j * rng.standard_normal((ndays * nstep, nchan, nspec))
        src, rec = np.array([0, 1, 2, 0]), np.array([3, 4, 5, 5])
        days = replicas.day_shard(ndays, rank, world)
        w = slice(days.start * nstep, days.stop * nstep)
        local = xo.xc_stack(spec[w], src, rec, 1.0 / ((days.stop - days.start) * nstep))
        mean, total = replicas.linear_stack_over_shards(local, (days.stop - days.start) * nstep)
        slowest = replicas.reduce_max(1.0 + rank)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), mean=mean, total=total, slowest=slowest,
                 days=np.array(list(days)))
    finally:
        dist.destroy_process_group()


def test_day_shards_cover_every_day_once():
    from fastxc_gb300 import replicas

    for ndays in (1, 5, 30, 31):
        for world in (1, 2, 3, 8):
            got = [d for r in range(world) for d in replicas.day_shard(ndays, r, world)]
            assert got == list(range(ndays))


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from fastxc_gb300 import replicas
    from oracle import xc_oracle as xo

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = np.load(tmp_path / "r0.npz"), np.load(tmp_path / "r1.npz")
    assert sorted(list(r0["days"]) + list(r1["days"])) == list(range(5))
    rng = np.random.default_rng(0)
    spec = rng.standard_normal((20, 6, 33)) + 1j * rng.standard_normal((20, 6, 33))
    ref = xo.xc_stack(spec, np.array([0, 1, 2, 0]), np.array([3, 4, 5, 5]), 1.0 / 20)
    for r in (r0, r1):
        assert int(r["total"]) == 20 and float(r["slowest"]) == 2.0
        assert np.abs(r["mean"] - ref).max() <= 1e-12 * np.abs(ref).max()
    assert replicas.whole_job_rate(100.0, 2, 0.5) == 400.0
