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


def test_reference_arm_line_on_rank_zero():
    """Rank 0 (or a plain run) of the reference arm times the CPU
    restatement on a sample of the headline workload and prints one JSON line
    with the keys the benchmark line carries: the same metric and unit as the
    GPU arm, the sample's scale and bases in `config`, a `cpu_baseline`
    describing this run and an `e2e` with no host-device copies."""
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE")}
    scale = 0.0005  # 2 Mbp of the 4 Gbp long-read workload
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--ref-sample-scale", str(scale)], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert (d["metric"], d["unit"], d["higher_is_better"]) == ("MC Gbases/s", "Gbases/s", True)
    assert (d["steps"], d["warmup"], d["n_gpus"]) == (2, 1, 1)
    assert d["value"] > 0
    cfg = d["config"]
    assert cfg["workload"] == "mc_abundance_long_reads_4gbp_k63" and (cfg["k"], cfg["m"], cfg["x"]) == (63, 21, 3)
    assert cfg["scale"] == scale and cfg["bases"] == int(4_000_000_000 * scale)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert f"scale {scale}" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
