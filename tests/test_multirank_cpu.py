"""The N > 1 host logic of bench.py on CPU (world size 2, gloo).

The path is one lattice per GPU, so N ranks run N independent replicas: the
only exchange is the barrier around the timed region and the maximum of the
ranks' times (bench.Dist).  Here two gloo ranks check both, and the reference
arm under torchrun prints exactly one line (rank 0) while rank 1 exits 0
without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist("gloo")
    assert (d.rank, d.world) == (rank, world)
    d.barrier()
    m = d.max(10.0 * (rank + 1))
    d.barrier()
    d.close()
    with open(os.path.join(out, f"r{rank}.txt"), "w") as f:
        f.write(repr(m))


def test_dist_barrier_and_max_two_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / f"r{r}.txt").read_text()) == 20.0


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "su2_fp64_32",
           "--gpus", "2", "--steps", "2", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
