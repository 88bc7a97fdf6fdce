"""Replica parallelism (one process per GPU, no data-path collective) on CPU: two gloo ranks
check the max-over-ranks timing, the whole-job rate and the dealing of ensemble members."""
import os
import socket

import pytest

from impec2d_gb300 import replicas as R


def test_shard_deals_every_member_once():
    for n in (0, 1, 7, 256):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in R.shard(n, r, world))
            assert got == list(range(n))
            sizes = [len(R.shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    # members listed size by size (64 per size): every rank gets the same mix
    sizes = [s for s in (128, 256, 384, 512) for _ in range(64)]
    for r in range(4):
        mine = [sizes[i] for i in R.shard(len(sizes), r, 4)]
        assert all(mine.count(s) == 16 for s in (128, 256, 384, 512))
    with pytest.raises(ValueError):
        R.shard(4, 2, 2)


def test_single_process_needs_no_group():
    assert R.max_over_ranks(3.5) == 3.5
    assert R.whole_job_rate(100.0, 2.0, 1) == 50.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = R.dist_info()
        assert (r, w, lr) == (rank, world, rank)
        # each rank "times" a different amount of work; the job takes the slowest
        t = R.max_over_ranks(1.0 + rank)
        rate = R.whole_job_rate(1000.0, t, w)
        out.put((rank, t, rate, R.shard(10, r, w)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _, _ in res] == [2.0, 2.0]
    assert all(rate == 1000.0 for _, _, rate, _ in res)  # 2 ranks x 1000 units / 2 s
    assert res[0][3] == [0, 2, 4, 6, 8] and res[1][3] == [1, 3, 5, 7, 9]
