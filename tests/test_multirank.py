"""The N > 1 bench path on CPU: world-size-2 gloo ranks. Each rank evaluates
its own configuration (no collective in the data path); the only collectives
are the reductions of the timing and the atom count, which these tests run
over gloo exactly as the GPU ranks run them over NCCL."""
from __future__ import annotations

import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, tmpdir, q):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, REPO)
    import bench
    dev = torch.device("cpu")
    slowest = bench.reduce_over_ranks([3.0, 5.0][rank], "max", world, dev)
    total = bench.reduce_over_ranks([100, 120][rank], "sum", world, dev)
    _, nb, _ = bench.workload(2, os.path.join(tmpdir, f"r{rank}"), rank)
    atoms = bench.reduce_over_ranks(nb.natom, "sum", world, dev)
    q.put((rank, slowest, total, nb.natom, atoms, float(nb.dlist.sum())))
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()


def test_two_rank_reductions_and_independent_configurations(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    for r in range(2):
        os.makedirs(tmp_path / f"r{r}", exist_ok=True)
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, str(tmp_path), q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, s0, t0, n0, a0, d0), (_, s1, t1, n1, a1, d1) = out
    assert s0 == s1 == 5.0  # slowest rank's time on every rank
    assert t0 == t1 == 220.0
    assert a0 == a1 == n0 + n1  # whole-job units: the atoms of both ranks
    assert d0 != d1  # the ranks evaluate different configurations
    assert bench_rate(a0, s0) == pytest.approx((n0 + n1) / 5.0)


def bench_rate(units, seconds):
    sys.path.insert(0, REPO)
    import bench
    return bench.whole_job_rate(units, seconds)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    sys.path.insert(0, REPO)
    import bench

    class Args:
        ncell = 2
    called = []
    monkeypatch.setattr(bench, "workload", lambda *a, **k: called.append(a))
    bench.reference_arm(Args(), rank=1)
    assert called == [] and capsys.readouterr().out == ""


def test_reference_arm_never_loads_the_library(tmp_path):
    """The reference arm enumerates the seeded potential's basis with the
    oracle: its process maps the oracle's library and never libmagace.so."""
    import json
    import subprocess
    run = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--ncell", "2",
                          "--steps", "1", "--warmup", "1", "--cpu-seconds", "0.2"],
                         capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert run.returncode == 0, run.stderr
    line = json.loads(run.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    libs = line["native_libraries"]
    assert any("oracle" in p for p in libs), libs
    assert not any("libmagace" in p for p in libs), libs
