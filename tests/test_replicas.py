"""The multi-GPU path of bench.py on CPU: replicas over gloo ranks.

The transport does not shard (each GPU runs its own photons with its own
seeds: replicas), so the only cross-rank work is the timing protocol -- a
barrier around the timed region, the maximum of the ranks' times and the sum
of their photons -- and the reference arm, which rank 0 alone runs and
prints.  Both are exercised here with world size 2 on the gloo backend.
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


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.dist_init(world)
    bench.barrier(w)
    res = {"rank": r, "max": bench.allmax(10.0 * (r + 1), w), "sum": bench.allsum(r + 1, w)}
    bench.barrier(w)
    with open(os.path.join(out, "rank%d.json" % r), "w") as f:
        json.dump(res, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_timing_reductions_over_two_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        res = json.load(open(tmp_path / ("rank%d.json" % r)))
        assert res == {"rank": r, "max": 20.0, "sum": 3.0}


@pytest.mark.timeout(600)
def test_reference_arm_prints_one_line_under_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--photons", "1e6"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
