"""The multi-rank (replicas) path of bench.py on CPU: two gloo ranks.

bench.py --gpus N runs one independent box per rank (seed + rank), times
each rank, takes the slowest rank's time (max over ranks) and reports the
particle-steps of all ranks over it; the reference arm runs on rank 0 only.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took (r + 1) seconds: the job time is the slowest rank's
    t = bench.reduce_max(float(rank + 1), dist)
    v = bench.job_value(world, 1000, 10, t)
    seed = bench.rank_seed(bench.CONFIGS["ndgp_512_1024"], rank)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, "rank%d.txt" % rank), "w") as f:
        f.write("%r %r %d\n" % (t, v, seed))


def test_two_gloo_ranks_reduce_to_the_slowest(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = [open(os.path.join(tmp_path, "rank%d.txt" % r)).read().split() for r in range(world)]
    for r, (t, v, seed) in enumerate(got):
        assert float(t) == 2.0                      # max over ranks
        assert float(v) == pytest.approx(2 * 1000 * 10 / 2.0 / 1e6)
        assert int(seed) == 5003 + r                # independent boxes


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                        "lcdm_64_128", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
