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


def test_reference_arm_line():
    """bench.py --impl reference: the CPU restatement of the reference step on the benchmark
    workload, one JSON line whose step counts are the ones timed."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "MLUPS" and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 0 and line["value"] > 0
    assert line["config"]["workload"].startswith("periodic hill 256x128x192")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["steps"] == 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
