"""The multi-process path of bench.py on CPU: the path shards into
independent replicas with no data-path collective, so the only exchange is
the max-over-ranks of the timed region (gloo, world size 2), and under
torchrun the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(1.5 + rank, dist, "cpu")  # rank 1 is the slow replica
    q.put((rank, slowest, bench.job_rate(100.0, 4, world, slowest)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both replicas see the slowest time; the job rate counts both replicas' work over it
    assert out == [(0, 2.5, 100.0 * 4 * 2 / 2.5), (1, 2.5, 100.0 * 4 * 2 / 2.5)]


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
    assert bench.job_rate(10.0, 3, 1, 2.0) == 15.0


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "1", "--workload", "cornell"]
    proc = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [json.loads(line) for line in proc.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    # the arm runs the oracle only: the scene comes from a child process as upload bytes
    assert line["maps_gpu_library"] is False
    # the same workload dict as the GPU arm's line at this replica count (which implementation ran is
    # the top-level "kernel", not part of the config)
    assert line["kernel"] == "cpu" and "kernel" not in line["config"]
    assert line["config"]["precision"] == "fp32" and line["config"]["parallelism"] == "replicas x2"
    assert line["config"]["image"] == [256, 256] and line["config"]["spp"] == 16


def test_both_arms_print_one_workload_config():
    # the GPU arm describes its world object, the reference arm the counts of the world it received as
    # upload bytes: the same workload gives the same config dict, whichever implementation ran
    sys.path.insert(0, str(ROOT))
    import bench

    class World:
        def triangle_count(self):
            return 2096640

        def node_count(self):
            return 2358439

    ours = bench.workload_config(World(), "fp32", 1)
    ref = bench.workload_config(bench._Counts({"triangles": 2096640, "bvh_nodes": 2358439}), "fp32", 1)
    assert ours == ref and "kernel" not in ours
    assert ours["precision"] == "fp32" and ours["parallelism"] == "replicas x1"
