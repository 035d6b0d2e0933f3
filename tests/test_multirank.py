"""The bench's multi-rank path on the CPU: two gloo ranks on 127.0.0.1.

Instances are independent SCFT solves, so `bench.py --gpus N` runs the same
batch on every rank with no collective on the data path; the ranks meet only
at the barrier around the timed region and in the maximum of their timings,
and the whole-job rate is the units all ranks processed over the slowest
rank's time.  These tests run that logic (bench.Ranks, bench.job_rate) as two
spawned processes, and check that the reference arm does its work on rank 0
only.
"""
import json
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


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    r = bench.Ranks(world, "gloo", "cpu")
    r.barrier()
    local_ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    ms = r.allmax(local_ms)
    units = 15 * 100  # 15 instances x 100 iterations on every rank
    rate = bench.job_rate(units, world, ms / 1e3)
    r.barrier()
    r.close()
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "rate": rate}, f)


def test_two_gloo_ranks_agree_on_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(world)]
    for r in res:
        assert r["ms"] == 20.0  # both ranks see the slowest rank's time
        assert r["rate"] == pytest.approx(15 * 100 * world / 0.020)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    r = bench.Ranks(1, "gloo", "cpu")
    assert r.dist is None
    r.barrier()
    assert r.allmax(3.5) == 3.5
    r.close()
    assert bench.job_rate(1500, 1, 0.5) == 3000.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_maps_no_repository_library():
    """The reference arm times the compiled reference only: its process must
    not load libscft.so (or any other shared object built in the repository)."""
    from ref_case import REF_BIN

    if not os.path.exists(REF_BIN):
        pytest.skip("oracle binary not built")
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "plate64_N100", "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0, line
    assert line["repo_libraries_mapped"] == [], line["repo_libraries_mapped"]
