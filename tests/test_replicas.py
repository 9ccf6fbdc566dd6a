"""Replica runs (one process per GPU, no data-path collective): the group's
barrier and reductions on world_size 2 over gloo, on the CPU."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    from mczi_gb300.replicas import ReplicaGroup
    g = ReplicaGroup("gloo")
    g.barrier(sync_device=False)
    # rank r processed 1000 + r units in 10 + 5 r ms
    mx = g.max_over_ranks(10.0 + 5 * rank)
    sm = g.sum_over_ranks(1000 + rank)
    tp = g.throughput(1000 + rank, 10.0 + 5 * rank)
    g.barrier(sync_device=False)
    g.close()
    Path(out_dir, f"r{rank}").write_text(f"{g.world} {g.rank} {mx} {sm} {tp}")


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    world, port = 2, _free_port()
    torch.multiprocessing.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                                          start_method="spawn")
    for r in range(world):
        ws, rank, mx, sm, tp = (float(v) for v in (tmp_path / f"r{r}").read_text().split())
        assert (ws, rank) == (world, r)
        assert mx == 15.0 and sm == 2001.0
        assert tp == pytest.approx(2001.0 / 15e-3)  # every rank reports the same whole-job figure


def test_single_process_group_needs_no_rendezvous(monkeypatch):
    for v in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(v, raising=False)
    from mczi_gb300.replicas import ReplicaGroup
    g = ReplicaGroup("gloo")
    assert (g.world, g.rank) == (1, 0)
    assert g.max_over_ranks(3.5) == 3.5 and g.throughput(100, 2.0) == pytest.approx(5e4)
    g.close()


def test_reference_arm_prints_on_rank_zero_only():
    """Under torchrun every rank runs bench.py; the reference arm's CPU work
    and its JSON line belong to rank 0, the other ranks exit 0 at once."""
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
