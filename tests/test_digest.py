"""The result digest (mczi_gb300.digest) and the oracle's hash-range digest
passes, on the CPU.

bench.py and the full-size GPU tests compare a GPU result with a digest the
oracle computed in passes over disjoint hash ranges
(tests/golden/make_digests.py).  Here the three definitions are pinned
against each other on small cases of every workload shape: the numpy digest
of the oracle's records, the oracle's digest of the same records, and the
oracle's pass-wise digest for several pass counts.
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "digests.json"


def test_digest_definitions_agree_mc(oracle):
    from mczi_gb300 import digest, gen
    cases = [([gen.c2_reads(0.001)], 63, 3, 0), ([gen.c1_reads(0.005)], 31, 0, 0), ([gen.c1_reads(0.005)], 31, 5, 0),
             (gen.c3_datasets(8, genome_len=60_000), 31, 2, 1), ([gen.c1_reads(0.002)], 64, 0, 0),
             ([gen.c1_reads(0.002)], 5, 1, 0)]
    for inputs, k, x, mode in cases:
        lo, hi, cnt = oracle.count(inputs, k, x, mode)
        ref = digest.records_digest(lo, hi if k > 32 else None, cnt)
        assert ref == oracle.records_digest(lo, hi, cnt)
        assert ref["records"] == lo.size and ref["count_sum"] == int(cnt.sum())
        for passes in (1, 3, 8):
            assert oracle.count_digest(inputs, k, x, mode, 4, passes) == ref, (k, x, mode, passes)


def test_digest_definitions_agree_zi(oracle):
    from mczi_gb300 import digest, gen
    index, query = gen.c4_index_and_query(genome_len=100_000, query_bases=1_000_000, k=31)
    lo, hi = oracle.zi_absent(index, [query], 31)
    ref = digest.records_digest(lo, hi, np.ones(lo.size, dtype=np.uint64))
    for passes in (1, 4):
        assert oracle.zi_absent_digest(index, [query], 31, 4, passes) == ref


def test_digest_is_order_independent_and_sensitive():
    from mczi_gb300 import digest
    rng = np.random.default_rng(1)
    lo = rng.integers(0, 2**63, size=1000, dtype=np.uint64)
    hi = rng.integers(0, 2**63, size=1000, dtype=np.uint64)
    cnt = rng.integers(1, 100, size=1000, dtype=np.uint64)
    d = digest.records_digest(lo, hi, cnt)
    p = rng.permutation(1000)
    assert digest.records_digest(lo[p], hi[p], cnt[p]) == d
    assert digest.records_digest(lo, hi, cnt, chunk=7) == d
    cnt2 = cnt.copy()
    cnt2[5] += 1
    assert digest.records_digest(lo, hi, cnt2)["sum"] != d["sum"]
    hi2 = hi.copy()
    hi2[9] ^= np.uint64(1)
    assert digest.records_digest(lo, hi2, cnt)["xor"] != d["xor"]


def test_committed_digests_are_well_formed():
    if not GOLDEN.exists():
        pytest.skip("no committed digests")
    d = json.loads(GOLDEN.read_text())
    for name, e in d.items():
        assert e["digest"]["records"] > 0, name
        assert len(e["digest"]["sum"]) == 16 and len(e["digest"]["xor"]) == 16
        assert all(len(f) == 16 for f in e["input_fingerprints"])
        assert e["scale"] == 1.0


def test_fingerprint_is_positional():
    from mczi_gb300 import gen
    a = np.frombuffer(b">r\n" + b"ACGT" * 1_000_000 + b"\n", dtype=np.uint8).copy()
    f = gen.fingerprint(a)
    assert f == gen.fingerprint(a.copy())
    b = a.copy()
    b[2_000_001], b[2_000_002] = a[2_000_002], a[2_000_001]
    assert gen.fingerprint(b) != f
    assert gen.fingerprint(a[:-1]) != f
