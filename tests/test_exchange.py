"""Several GPUs: MC counting's exchange plan (mczi_gb300/exchange.py, in
abundance and fof presence mode) and ZI's sharded queries
(mczi_gb300/zi.py::collect_absent_sharded) on two gloo ranks on the CPU, and
the record split.

The GPU routing step (mczi_route_superkmers) is replaced here by a CPU
stand-in with the property the plan relies on: every window goes to the rank
chosen by a function of its canonical k-mer (the GPU routes whole superkmers
by their minimizer bucket, which is such a function).  The per-rank count is
the oracle's.  The union of the ranks' records must equal the oracle's
single-rank result.  The real routing step is checked on one GPU in
tests/test_mc_gpu.py::test_route_superkmers_union_equals_single.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
K, X = 15, 1


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reads(seed=4, n=300):
    rng = np.random.default_rng(seed)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=3000)
    out = []
    for i in range(n):
        a = int(rng.integers(0, 2800))
        s = g[a:a + int(rng.integers(20, 200))].copy()
        if rng.random() < 0.5:
            s = np.frombuffer(bytes(s)[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA")), dtype=np.uint8).copy()
        if rng.random() < 0.2:
            s[int(rng.integers(0, s.size))] = ord("N")
        out.append(b">r%d\n" % i + s.tobytes() + b"\n")
    return b"".join(out)


def cpu_route(share, world, k=K):
    """Every window of the share as its own FASTA record, sent to the rank
    hash(canonical k-mer) mod world."""
    import oracle_ref
    groups = [[] for _ in range(world)]
    comp = {0: 3, 1: 2, 2: 1, 3: 0}
    for buf in share:
        codes, offs, _ = oracle_ref.fragments(bytes(buf), k)
        for f in range(len(offs) - 1):
            seq = codes[int(offs[f]):int(offs[f + 1])]
            for i in range(seq.size - k + 1):
                w = seq[i:i + k]
                fwd = int("".join("%d" % c for c in w), 4)
                rev = int("".join("%d" % comp[int(c)] for c in w[::-1]), 4)
                dest = (min(fwd, rev) * 0x9E3779B97F4A7C15 >> 17) % world
                groups[dest].append(b">\n" + bytes(b"ACGT"[int(c)] for c in w) + b"\n")
    return [np.frombuffer(b"".join(g), dtype=np.uint8) for g in groups]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch.distributed as dist
    import oracle_ref
    from mczi_gb300 import exchange
    from mczi_gb300.mc import CounterConfig
    dist.init_process_group("gloo", rank=rank, world_size=world)
    data = _reads()
    share = [exchange.split_records(data, world)[rank]]
    lo, hi, cnt = exchange.count_sharded(
        share, CounterConfig(K, 7, X), route=cpu_route,
        count=lambda received: (lambda r: (r[0], None, r[2]))(oracle_ref.count(received, K, X)))
    got = exchange.gather_records(lo, hi, cnt)
    if rank == 0:
        np.save(Path(out_dir, "lo.npy"), got[0])
        np.save(Path(out_dir, "cnt.npy"), got[2])
    Path(out_dir, f"n{rank}").write_text(str(lo.size))
    dist.barrier()
    dist.destroy_process_group()


def test_exchange_plan_two_gloo_ranks(tmp_path, oracle):
    torch = pytest.importorskip("torch")
    world, port = 2, _free_port()
    torch.multiprocessing.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                                          start_method="spawn")
    lo, hi, cnt = oracle.count([_reads()], K, X)
    assert np.array_equal(np.load(tmp_path / "lo.npy"), lo)
    assert np.array_equal(np.load(tmp_path / "cnt.npy"), cnt)
    # both ranks counted a share of the k-mers (a disjoint split)
    n = [int((tmp_path / f"n{r}").read_text()) for r in range(world)]
    assert all(v > 0 for v in n) and sum(n) == lo.size


def _datasets(n=4):
    """fof inputs: n read samples of one genome (presence counts up to n)."""
    rng = np.random.default_rng(11)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=1500)
    out = []
    for d in range(n):
        recs = []
        for i in range(60 + 20 * d):
            a = int(rng.integers(0, 1400))
            s = g[a:a + int(rng.integers(20, 120))].copy()
            if rng.random() < 0.5:
                s = np.frombuffer(bytes(s)[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA")), dtype=np.uint8)
            recs.append(b">d%dr%d\n" % (d, i) + s.tobytes() + b"\n")
        out.append(b"".join(recs))
    return out


def _fof_rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch.distributed as dist
    import oracle_ref
    from mczi_gb300 import exchange
    from mczi_gb300.mc import CounterConfig
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # every rank takes a share of every dataset; rank 1's share of the last
    # dataset is empty (a dataset need not reach every rank)
    shares = [[exchange.split_records(ds, world)[rank]] for ds in _datasets()]
    if rank == 1:
        shares[-1] = []
    if rank == 0:
        shares[-1] = [_datasets()[-1]]
    lo, hi, cnt = exchange.count_datasets_sharded(
        shares, CounterConfig(K, 7, X), route=cpu_route,
        count=lambda received: (lambda r: (r[0], None, r[2]))(oracle_ref.count(received, K, X, 1)))
    got = exchange.gather_records(lo, hi, cnt)
    if rank == 0:
        np.save(Path(out_dir, "lo.npy"), got[0])
        np.save(Path(out_dir, "cnt.npy"), got[2])
    Path(out_dir, f"n{rank}").write_text(str(lo.size))
    dist.barrier()
    dist.destroy_process_group()


def test_fof_exchange_plan_two_gloo_ranks(tmp_path, oracle):
    """fof mode: datasets split over two ranks, each dataset routed on its
    own, sizes per (destination, dataset) exchanged with the bytes, presence
    counted per rank; the union equals the oracle's presence count of the
    whole datasets."""
    torch = pytest.importorskip("torch")
    world, port = 2, _free_port()
    torch.multiprocessing.start_processes(_fof_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                                          start_method="spawn")
    lo, hi, cnt = oracle.count(_datasets(), K, X, 1)
    assert lo.size > 0 and int(cnt.max()) == 4  # k-mers in every dataset are kept
    assert np.array_equal(np.load(tmp_path / "lo.npy"), lo)
    assert np.array_equal(np.load(tmp_path / "cnt.npy"), cnt)
    n = [int((tmp_path / f"n{r}").read_text()) for r in range(world)]
    assert all(v > 0 for v in n) and sum(n) == lo.size


def _zi_inputs():
    """A ZI index (one genome) and three query sets: reads of the genome and
    of foreign sequence, some with an N."""
    rng = np.random.default_rng(21)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    g = rng.choice(acgt, size=4000)
    foreign = rng.choice(acgt, size=600)  # absent k-mers that recur across records and ranks
    index = b">idx\n" + g.tobytes() + b"\n"
    queries = []
    for q in range(3):
        recs = []
        for i in range(50 + 30 * q):
            src = g if rng.random() < 0.7 else foreign
            a = int(rng.integers(0, src.size - 150))
            s = src[a:a + int(rng.integers(30, 150))].copy()
            if rng.random() < 0.2:
                s[int(rng.integers(0, s.size))] = ord("N")
            recs.append(b">q%dr%d\n" % (q, i) + s.tobytes() + b"\n")
        queries.append(b"".join(recs))
    return index, queries


def _zi_rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch.distributed as dist
    import oracle_ref
    from mczi_gb300 import zi
    dist.init_process_group("gloo", rank=rank, world_size=world)
    index, queries = _zi_inputs()
    for k in (15, 41):
        def absent(share):
            lo, hi = oracle_ref.zi_absent(index, share, k)
            Path(out_dir, f"n{k}_{rank}").write_text(str(lo.size))
            return lo, hi
        got = zi.collect_absent_sharded(None, queries, absent=absent)
        if rank == 0:
            np.save(Path(out_dir, f"lo{k}.npy"), got[0])
            np.save(Path(out_dir, f"hi{k}.npy"), got[1])
        else:
            assert got is None
    dist.barrier()
    dist.destroy_process_group()


def test_zi_sharded_queries_two_gloo_ranks(tmp_path, oracle):
    """ZI on several GPUs: the index replicated, every query split over two
    ranks, the absent sets gathered and merged at rank 0; the merged set
    equals the oracle's absent set of the whole queries (k = 15 and 41)."""
    torch = pytest.importorskip("torch")
    world, port = 2, _free_port()
    torch.multiprocessing.start_processes(_zi_rank_main, args=(world, port, str(tmp_path)), nprocs=world,
                                          start_method="spawn")
    index, queries = _zi_inputs()
    for k in (15, 41):
        lo, hi = oracle.zi_absent(index, queries, k)
        assert lo.size > 0
        # the ranks' sets overlap, so the merge has duplicates to remove
        assert sum(int((tmp_path / f"n{k}_{r}").read_text()) for r in range(world)) > lo.size, k
        assert np.array_equal(np.load(tmp_path / f"lo{k}.npy"), lo), k
        assert np.array_equal(np.load(tmp_path / f"hi{k}.npy"), hi), k


def test_split_records_cuts_at_record_starts():
    from mczi_gb300 import exchange
    fa = _reads(7, 50)
    for parts in (1, 2, 3, 7, 60):
        sl = exchange.split_records(fa, parts)
        assert len(sl) == parts and b"".join(bytes(s) for s in sl) == fa
        assert all(s.size == 0 or s[0] == ord(">") for s in sl)
    fq = b"".join(b"@q%d\nACGTACGT\n+\nIIIIIIII\n" % i for i in range(40))
    sl = exchange.split_records(fq, 4)
    assert b"".join(bytes(s) for s in sl) == fq
    assert all(s.size == 0 or (s[0] == ord("@") and bytes(s).count(b"\n") % 4 == 0) for s in sl)
