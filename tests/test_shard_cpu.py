"""The multi-GPU bookkeeping of the engine (cuphoto.shard) on the CPU: two
gloo ranks in their own processes share a barrier, the slowest rank's time,
the total work and one split of a scene set, as the benchmark's ranks do on
their GPUs.  No data path is exchanged: each rank's volumes are its own."""
import os
import socket

import pytest

from cuphoto import shard


def test_partition_by_cost_is_complete_disjoint_and_balanced():
    costs = [n ** 3 * f for n, f in [(64, 10), (384, 120), (128, 30), (256, 90), (96, 50), (320, 15), (200, 70),
                                      (72, 110), (160, 40), (352, 20), (88, 100), (240, 60), (112, 80), (296, 35),
                                      (136, 25), (184, 95)]]
    for world in (1, 2, 3, 4, 8):
        parts = shard.partition_by_cost(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        # the largest item alone bounds how even the split can be
        bound = max(1.0, max(costs) / (sum(costs) / world))
        assert shard.balance(costs, parts) <= max(bound, 1.35)
    assert shard.partition_by_cost([], 2) == [[], []]
    assert shard.partition_by_cost([5.0], 3) == [[0], [], []]


def test_single_process_is_the_identity():
    assert shard.max_over_ranks(3.5) == 3.5
    assert shard.sum_over_ranks(2.0) == 2.0
    assert shard.whole_job_rate(100.0, 4.0) == 25.0
    shard.barrier()
    assert shard.scene_seed(0, 1, 3) == 103


def _rank_main(rank, world, port, errors):
    try:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
        try:
            shard.barrier()
            # rank r took (r + 1) * 10 ms and processed (r + 1) * 1000 units
            assert shard.max_over_ranks((rank + 1) * 0.010) == pytest.approx(world * 0.010)
            assert shard.sum_over_ranks((rank + 1) * 1000) == sum((r + 1) * 1000 for r in range(world))
            rate = shard.whole_job_rate((rank + 1) * 1000, (rank + 1) * 0.010)
            assert rate == pytest.approx(sum((r + 1) * 1000 for r in range(world)) / (world * 0.010))
            # every rank computes the same split and takes its own part
            costs = [7, 3, 9, 1, 4, 4, 8, 2]
            mine = shard.partition_by_cost(costs, world)[rank]
            got = [None] * world
            dist.all_gather_object(got, mine)
            assert sorted(i for p in got for i in p) == list(range(len(costs)))
            # scenes made per rank do not collide
            seeds = [None] * world
            dist.all_gather_object(seeds, [shard.scene_seed(0, rank, i) for i in range(16)])
            assert len({s for p in seeds for s in p}) == 16 * world
        finally:
            dist.destroy_process_group()
    except BaseException as e:  # reported to the parent, which fails the test
        errors.put("rank %d: %r" % (rank, e))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.timeout(120)
def test_two_gloo_ranks_share_time_work_and_split():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    errors = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, errors)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    msgs = []
    while not errors.empty():
        msgs.append(errors.get())
    assert not alive, "a rank did not finish"
    assert not msgs, msgs
    assert all(p.exitcode == 0 for p in procs)
