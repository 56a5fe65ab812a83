"""bench.py at N > 1 runs independent replicas (the path does not shard on one box): the job
time is the slowest rank's, found with a MAX all-reduce. Checked with two gloo ranks on CPU."""
import os
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out[rank] = bench.slowest_rank_ms(10.0 + 5.0 * rank, world, "cpu")
    dist.destroy_process_group()


def test_slowest_rank_time_two_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29500 + os.getpid() % 1000
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == 15.0 and out[1] == 15.0


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank_ms(7.5, 1, "cpu") == 7.5
