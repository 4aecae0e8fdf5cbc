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


def _batch_rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = bench.CONFIGS["fofr_batch_64x64_128"]
    mine = bench.shard(bench.batch_boxes(cfg), rank, world)
    # the batch's graph time on this rank; the job's time is the slowest
    t = bench.reduce_max(0.1 * (rank + 1), dist)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, "batch%d.txt" % rank), "w") as f:
        f.write(repr((t, [(b["Seed"], b["inverted"], b["fofr0"]) for b in mine])))


def test_batch_boxes_split_across_gloo_ranks(tmp_path):
    """The 64-box sweep is the workload that shards: rank r runs boxes
    r, r + N, ... as its own batch, with no collective on the data path; the
    job time is the slowest rank's."""
    pytest.importorskip("torch")
    import ast
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    import bench

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_batch_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = [ast.literal_eval(open(os.path.join(tmp_path, "batch%d.txt" % r)).read()) for r in range(world)]
    everything = [(b["Seed"], b["inverted"], b["fofr0"]) for b in bench.batch_boxes(bench.CONFIGS["fofr_batch_64x64_128"])]
    assert len(got[0][1]) == len(got[1][1]) == 32
    assert sorted(got[0][1] + got[1][1]) == sorted(everything)   # every box exactly once
    assert got[0][1] == everything[0::2] and got[1][1] == everything[1::2]
    assert got[0][0] == got[1][0] == pytest.approx(0.2)


def test_gpus_flag_starts_its_own_ranks():
    """bench.py --gpus 2 without a launcher starts two ranks itself (torch's
    launcher on this node); the reference arm then prints one line, from
    rank 0."""
    pytest.importorskip("torch")
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env["MGP_BENCH_PORT"] = str(_free_port())
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--config", "lcdm_64_128", "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
