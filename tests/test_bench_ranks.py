"""The multi-rank host logic of bench.py on CPU: two ``gloo`` ranks started the
way torchrun starts them (RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* in the
environment). Covers the rank discovery, the barriers, the max-over-ranks of
the elapsed times, the whole-job throughput (units of every rank over the
slowest rank's time) and the reference arm's rank-0-only rule. No GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys, types
sys.path.insert(0, sys.argv[1])
import bench
world, rank, local = bench._dist()
bench._init_ranks(local, backend="gloo")
bench._barrier(world)
out = {
    "world": world, "rank": rank, "local": local,
    "max": bench._reduce_over_ranks(1.5 + rank, "max", world, device="cpu"),
    "sum": bench._reduce_over_ranks(100 * (rank + 1), "sum", world, device="cpu"),
    # rank r processed 1000 (r + 1) units in 2 (r + 1) s
    "rate": bench.job_throughput(1000.0 * (rank + 1), 2.0 * (rank + 1), world, device="cpu"),
}
bench._barrier(world)
import torch.distributed as dist
dist.destroy_process_group()
args = types.SimpleNamespace(workload="C1", steps=1, warmup=0)
out["reference_arm"] = bench.run_reference(args) if rank != 0 else "not run"
with open(sys.argv[2], "w") as f:
    json.dump(out, f)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script), ROOT, str(tmp_path / f"out{r}.json")],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    logs = []
    for pr in procs:
        try:
            logs.append(pr.communicate(timeout=240)[0])
        except subprocess.TimeoutExpired:
            pr.kill()
            logs.append(pr.communicate()[0])
    for r, pr in enumerate(procs):
        assert pr.returncode == 0, f"rank {r} failed:\n{logs[r]}"
    outs = [json.loads((tmp_path / f"out{r}.json").read_text()) for r in range(2)]
    for r, o in enumerate(outs):
        assert (o["world"], o["rank"], o["local"]) == (2, r, r)
        assert o["max"] == 2.5
        assert o["sum"] == 300.0
        # 3000 units over the slowest rank's 4 s
        assert o["rate"] == pytest.approx(750.0)
    # the reference arm: ranks other than 0 return at once, printing nothing
    assert outs[1]["reference_arm"] is None
    assert logs[1].strip() == ""


def test_single_rank_is_identity(monkeypatch):
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench._dist() == (1, 0, 0)
    assert bench._reduce_over_ranks(3.25, "max", 1) == 3.25
    assert bench.job_throughput(1000.0, 4.0, 1) == 250.0
