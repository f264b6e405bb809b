"""Multi-process host logic of bench.py on CPU (gloo, world size 2): replicas
report all ranks' frames over the slowest rank's time; the reference arm runs
on rank 0 only."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # rank 1 is the slow one
    value, tmax = bench.aggregate(frames_per_rank=100, seconds_per_rank=1.0 + rank, world=world)
    bench.barrier(world)
    q.put((rank, value, tmax))
    dist.destroy_process_group()


def test_replica_aggregation_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, tmax in res:
        assert tmax == pytest.approx(2.0)
        assert value == pytest.approx(200 / 2.0)


def test_dist_env_defaults(monkeypatch):
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_env() == (0, 1, 0)
    assert bench.aggregate(10, 2.0, 1) == (5.0, 2.0)


def test_reference_arm_other_ranks_exit_without_work(capsys):
    import bench

    args = bench.parse_args(["--impl", "reference", "--steps", "1", "--warmup", "0"])
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
