"""The multi-GPU form is replicas only: each rank renders its own frames and
the whole-job figure is (sum of segments) / (slowest rank's time).  The
cross-rank combination bench.py uses is checked here on CPU with two gloo
ranks (no GPU, no collective on any data path)."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    elapsed, total = bench.combine_replicas(dist, 1.5 + rank, 1000 * (rank + 1), "cpu")
    q.put((rank, elapsed, total))
    dist.destroy_process_group()


def test_two_replicas_combine_max_time_and_sum_of_segments():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.5, 2.5]
    assert [o[2] for o in out] == [3000.0, 3000.0]


def test_one_rank_passes_through():
    import bench
    assert bench.combine_replicas(None, 2.0, 7, "cpu") == (2.0, 7.0)
