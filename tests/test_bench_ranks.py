"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): the
slowest rank's time sets the job's time, the whole-job value counts every
rank's particles, and the reference arm under torchrun prints one line from
rank 0 while the other rank exits without work."""
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


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks([1.0 + rank, 5.0 - rank, 0.25 * (rank + 1)], dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fh:
        json.dump(got, fh)


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    for r in range(world):
        with open(tmp_path / ("rank%d.json" % r)) as fh:
            assert json.load(fh) == [2.0, 5.0, 0.5]


def test_job_value_and_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([0.5, 0.25]) == [0.5, 0.25]
    # 2 replicas of 2,097,152 particles x 4 outputs in 1 ms
    assert bench.job_value(2, 2097152, 4, 1e-3) == pytest.approx(16.777216)


def test_reference_arm_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--nside", "12", "--cpu-sample", "256"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
