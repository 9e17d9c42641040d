"""The N > 1 (replicas) path of bench.py on CPU with the gloo backend.

A Markov chain does not shard, so N GPUs run N independent replicas; the
only cross-rank steps are the barriers around the timed region and the
max-over-ranks of the elapsed time.  These tests run two ranks on the host:
the max reduction and barrier helpers directly, and the reference arm under
torch.distributed.run, where rank 0 alone prints the JSON line and the other
rank exits 0 without work.
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


def _allreduce_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    bench.barrier(w)
    m = bench.allreduce_max(1.5 + rank, w)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": m}, f)
    dist.destroy_process_group()


def test_allreduce_max_and_barrier_two_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_allreduce_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert json.loads((tmp_path / f"rank{r}.json").read_text())["max"] == 2.5


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--config", "L4", "--gpus", "2", "--steps", "1", "--warmup", "0", "--ref-calls", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["cpu_baseline"]["kind"] == "port"
