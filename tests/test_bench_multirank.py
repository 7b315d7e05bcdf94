"""The multi-rank side of bench.py on CPU: two gloo ranks on 127.0.0.1.
bench.py runs one independent replica per GPU (no data-path collective);
its barrier and max-over-ranks reduction are checked here, and the reference
arm is run under torchrun with two ranks: rank 0 alone prints its line."""
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


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(2)
    d.barrier()
    m = d.max(1.5 + rank)          # the slowest rank's time
    d.barrier()
    d.close()
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(m))


def test_dist_barrier_and_max_over_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        assert float(open(tmp_path / f"r{r}.txt").read()) == 2.5


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    import oracle
    oracle.build()
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--nx", "64", "--ny", "32", "--bubbles", "2",
           "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    # the reference's own sources where they were built here, else the port
    assert line["cpu_baseline"]["kind"] == ("reference" if oracle.ref_available() else "port")
    assert line["config"]["curvature"] == "plain"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
