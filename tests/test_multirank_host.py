"""The replica path of the benchmark with two ranks on the CPU (gloo): the
whole-job reduction (slowest rank's time, every rank's k-mers) and the
reference arm, which rank 0 alone runs and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dt, kmers = bench.over_ranks(1.0 + 0.5 * rank, 1000 * (rank + 1), torch.device("cpu"),
                                     world)
        q.put((rank, dt, kmers))
    finally:
        dist.destroy_process_group()


def test_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    assert got == [(0, 1.5, 3000.0), (1, 1.5, 3000.0)]


def test_over_ranks_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.over_ranks(0.25, 7, None, 1) == (0.25, 7.0)


def test_reference_arm_prints_once_on_rank_zero():
    """Under torchrun with two ranks, rank 0 times the host restatement and
    prints one JSON line; rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--steps", "1", "--warmup", "3", "--reads-per-step", "3000"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "k-mers/s" and d["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "k-mers/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert 2800 <= d["config"]["reads_per_step"] < 3000    # N-reads dropped
    # the reference arm runs the oracle's restatement and never the GPU library
    assert not any("libgoetia_gb300" in p for p in d["repo_libraries_loaded"])
    assert any("liboracle" in p for p in d["repo_libraries_loaded"])
