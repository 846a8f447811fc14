"""Multi-rank host logic of the shot-parallel path, on CPU with gloo (world size 2).

Each rank takes a disjoint round-robin slice of the shot list (readmodel.py:121-126)
and the job rate uses all ranks' work over the slowest rank's time.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import a3d_dist


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        shots = [(x, y, 2) for x in range(0, 40, 8) for y in range(0, 24, 8)]
        mine = a3d_dist.shots_for_rank(shots, rank, world)
        seconds = 1.0 + rank  # rank 1 is the slow one
        rate = a3d_dist.job_rate(len(mine) * 100, seconds, dist)
        slowest = a3d_dist.max_over_ranks(seconds, dist)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        out.put((rank, rate, slowest, gathered))
    finally:
        dist.destroy_process_group()


def test_two_rank_shot_split_and_rate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shots = [(x, y, 2) for x in range(0, 40, 8) for y in range(0, 24, 8)]
    for rank, rate, slowest, gathered in res:
        assert slowest == 2.0
        assert rate == pytest.approx(len(shots) * 100 / 2.0)
        flat = [s for part in gathered for s in part]
        assert sorted(flat) == sorted(shots) and len(flat) == len(set(flat))
        assert gathered[0] == shots[0::2] and gathered[1] == shots[1::2]


def test_single_process_defaults():
    assert a3d_dist.shots_for_rank([1, 2, 3], 0, 1) == [1, 2, 3]
    assert a3d_dist.job_rate(10, 2.0) == 5.0
    with pytest.raises(ValueError):
        a3d_dist.shots_for_rank([1], 2, 2)
