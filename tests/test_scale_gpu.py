"""GPU parity at the benchmark configurations' own sizes.

The other GPU tests use scaled-down shapes; these compare the CUDA path
(through the C ABI) with the oracle on the workloads the benchmarks time:

* short reads: the full 150 Mbp workload (1.0 M x 150 bp reads of a 5 Mbp
  genome, k=31 m=21), x=5 through the KFF file (u8 counts saturated at
  min(x+1, 255), src/lib.rs:2489-2506) and x=0 as exact records;
* long reads: the 4 Gbp k=63 generator at scale 0.05 (200 Mbp; exact u64
  counts, src/lib.rs:2400-2425), record for record, and the full 4 Gbp run
  against the oracle digest committed in tests/golden/digests.json;
* fof: all 64 datasets of the presence workload over a 300 kbp base genome;
* ZI: the full 60 Mbp index with 100 Mbp of query reads (absent set digest
  against the oracle's, computed here), and the full 2 Gbp query against the
  committed digest.

Records are compared as sorted numpy arrays (bit-exact); digests are
mczi_gb300.digest's order-independent summary (record count, sum of counts,
wrapping sum and xor of a mixed word per record).
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "digests.json"


def kff_arrays(data: bytes):
    """(key_lo, key_hi, counts) of a KFF file's records, parsed with numpy."""
    assert data[:3] == b"KFF"
    p = 8
    p += 4 + int.from_bytes(data[p:p + 4], "big")
    assert data[p:p + 1] == b"v"
    nv = int.from_bytes(data[p + 1:p + 9], "big")
    p += 9
    vals = {}
    for _ in range(nv):
        e = data.index(b"\0", p)
        vals[data[p:e].decode()] = int.from_bytes(data[e + 1:e + 9], "big")
        p = e + 9
    assert data[p:p + 1] == b"r"
    n = int.from_bytes(data[p + 1:p + 9], "big")
    p += 9
    nb, cs = (vals["k"] + 3) // 4, vals["data_size"]
    rec = np.frombuffer(data, dtype=np.uint8, count=n * (nb + cs), offset=p).reshape(n, nb + cs)
    assert data[p + n * (nb + cs):] == b"KFF"
    key = np.zeros((n, 16), dtype=np.uint8)
    key[:, 16 - nb:] = rec[:, :nb]
    hi = key[:, :8].copy().view(">u8").ravel().astype(np.uint64)
    lo = key[:, 8:].copy().view(">u8").ravel().astype(np.uint64)
    cnt = np.zeros((n, 8), dtype=np.uint8)
    cnt[:, 8 - cs:] = rec[:, nb:]
    return lo, hi, cnt.view(">u8").ravel().astype(np.uint64)


def sort_records(lo, hi, cnt):
    order = np.lexsort((lo, hi))
    return lo[order], hi[order], cnt[order]


def golden_entry(name):
    if not GOLDEN.exists():
        pytest.skip("no committed digests")
    d = json.loads(GOLDEN.read_text())
    if name not in d:
        pytest.skip(f"no committed digest for {name}")
    return d[name]


def test_short_reads_full_size(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import gen
    from mczi_gb300.mc import CounterConfig
    data = gen.c1_reads(1.0)
    lo, hi, cnt = oracle.count([data], 31, 0)
    # x = 5 through the KFF file: every count byte is min(count, 6)
    gpu_ctx.count([data], CounterConfig(31, 21, 5))
    path = tmp_path / "c1.kff"
    gpu_ctx.write_kff(path)
    klo, khi, kc = sort_records(*kff_arrays(path.read_bytes()))
    keep = cnt > 5
    assert np.array_equal(klo, lo[keep]) and not khi.any()
    assert np.array_equal(kc, np.minimum(cnt[keep], 6))
    # x = 0: every distinct k-mer with its exact count
    n = gpu_ctx.count([data], CounterConfig(31, 21, 0))
    r = gpu_ctx.records(n, sorted=True)
    assert n == lo.size
    assert np.array_equal(r.lo, lo) and np.array_equal(r.count, cnt)


def test_long_reads_200mbp(gpu_ctx, oracle):
    from mczi_gb300 import digest, gen
    from mczi_gb300.mc import CounterConfig
    data = gen.c2_reads(0.05)
    lo, hi, cnt = oracle.count([data], 63, 3)
    n = gpu_ctx.count([data], CounterConfig(63, 21, 3))
    r = gpu_ctx.records(n, sorted=True)
    assert n == lo.size
    assert np.array_equal(r.lo, lo) and np.array_equal(r.hi, hi) and np.array_equal(r.count, cnt)
    assert digest.records_digest(r.lo, r.hi, r.count) == oracle.records_digest(lo, hi, cnt) == gpu_ctx.digest()


def test_long_reads_full_4gbp_digest(gpu_ctx):
    """The workload the headline benchmark times, against the committed
    oracle digest of the same generator output."""
    from mczi_gb300 import digest, gen
    from mczi_gb300.mc import CounterConfig
    g = golden_entry("mc_abundance_long_reads_4gbp_k63")
    data = gen.c2_reads(1.0)
    assert gen.fingerprint(data) == g["input_fingerprints"][0], "generator output differs from the fixture's"
    n = gpu_ctx.count([data], CounterConfig(63, 21, 3))
    del data
    assert gpu_ctx.digest() == g["digest"]
    r = gpu_ctx.records(n, sorted=False)
    assert digest.records_digest(r.lo, r.hi, r.count) == g["digest"]


def test_fof_64_datasets(gpu_ctx, oracle):
    from mczi_gb300 import gen
    ds = gen.c3_datasets(64, genome_len=300_000)
    for x in (5, 0):
        lo, hi, cnt = oracle.count(ds, 31, x, 1)
        from mczi_gb300.mc import CounterConfig
        n = gpu_ctx.count(ds, CounterConfig(31, 21, x), 1)
        r = gpu_ctx.records(n, sorted=True)
        assert n == lo.size, x
        assert np.array_equal(r.lo, lo) and np.array_equal(r.count, cnt), x


def test_zi_full_index_100mbp_query(gpu_ctx, oracle):
    from mczi_gb300 import digest, gen, zi
    index, query = gen.c4_index_and_query(genome_len=60_000_000, query_bases=100_000_000, k=31)
    zi.build_dictionary(index, 31, 19, ctx=gpu_ctx)
    n = zi.query(gpu_ctx, [query])
    r = gpu_ctx.records(n, sorted=False)
    got = digest.records_digest(r.lo, r.hi, np.ones(n, dtype=np.uint64))
    assert got == oracle.zi_absent_digest(index, [query], 31, None, 2)
    assert gpu_ctx.digest(unit_counts=True) == got


def test_zi_full_2gbp_digest(gpu_ctx):
    from mczi_gb300 import gen, zi
    g = golden_entry("zi_subtract_2gbp_k31")
    index, query = gen.c4_index_and_query(genome_len=60_000_000, query_bases=2_000_000_000, k=31)
    assert [gen.fingerprint(index), gen.fingerprint(query)] == g["input_fingerprints"]
    zi.build_dictionary(index, 31, 19, ctx=gpu_ctx)
    zi.query(gpu_ctx, [query])
    del query
    assert gpu_ctx.digest(unit_counts=True) == g["digest"]
