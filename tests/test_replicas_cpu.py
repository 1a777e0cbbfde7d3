"""Multi-rank (replica) bookkeeping on CPU with the gloo backend, world size 2.

The path shards as independent replicas: ranks exchange no data, only the
timing is combined (barrier, maximum over ranks).  The first test drives the
helper directly from two spawned ranks; the second launches the benchmark's
reference arm under torchrun with two ranks, where rank 0 alone runs and
prints one JSON line and rank 1 exits cleanly without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "lammps-mlip-package_gb300"))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from mlipg import replicas
    info = replicas.init("gloo")
    replicas.barrier(info)
    slowest = replicas.max_over_ranks(1.5 + rank, info)
    rate = replicas.aggregate_rate(100.0, 1.0 + rank, info)
    replicas.barrier(info)
    replicas.finish(info)
    q.put((rank, info, slowest, rate))


def test_max_over_ranks_and_rate_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, info, slowest, rate in out:
        assert info == {"rank": rank, "world": 2}
        assert slowest == 2.5                 # the slower rank's time
        assert rate == pytest.approx(100.0)   # 2 ranks x 100 units / 2.0 s


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload", "fcc-al-256",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                    # rank 0 only
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
