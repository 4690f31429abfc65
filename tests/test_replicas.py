"""The N > 1 path of bench.py on the CPU: independent replicas (one process
per GPU, disjoint Philox keys) joined only by a gloo group for the barriers,
the max-over-ranks time and the summed move counts.  Two gloo ranks on
127.0.0.1 run the same exchange the GPU ranks run; the reference arm under
torchrun runs on rank 0 only.
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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    group = bench.Replicas(world)
    group.barrier()
    moves = 1000.0 * (rank + 1)          # ranks advance different walker counts
    seconds = 0.5 + rank                 # rank 1 is the slower one
    rate = bench.whole_job_rate(moves, seconds, group)
    top = group.max(float(rank))
    count = group.sum(1.0)
    group.barrier()
    group.close()
    with open(os.path.join(out, "rank%d.json" % rank), "w") as f:
        json.dump(dict(rate=rate, top=top, count=count, seed=bench.replica_seed(100, rank)), f)


def test_two_gloo_replicas_exchange_only_timing_and_counts(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    mp.start_processes(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [json.load(open(tmp_path / ("rank%d.json" % k))) for k in range(2)]
    for g in got:
        # whole-job value: all ranks' moves over the slowest rank's time
        assert g["rate"] == pytest.approx((1000.0 + 2000.0) / 1.5)
        assert g["top"] == 1.0 and g["count"] == 2.0
    assert got[0]["seed"] != got[1]["seed"]
    assert abs(got[0]["seed"] - got[1]["seed"]) >= 1000


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    group = bench.Replicas(1)
    group.barrier()
    assert group.max(2.5) == 2.5 and group.sum(3.0) == 3.0
    assert bench.whole_job_rate(600.0, 2.0, group) == 300.0
    group.close()


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
