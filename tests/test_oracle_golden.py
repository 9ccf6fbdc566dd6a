"""The CPU oracle against the reference's own known-answer vectors.

The oracle is the parity checker for the GPU path, so it is pinned first:
every vector here is transcribed from the reference's unit tests (see the
`_source` fields of tests/golden/reference_vectors.json).
"""
import numpy as np
import pytest

from oracle_ref import decode, encode, parse_kff, to_int


def fa(seq):
    return f">s\n{seq}\n".encode()


def as_dict(lo, hi, cnt):
    return dict(zip(to_int(lo, hi), (int(c) for c in cnt)))


def test_ascii_counts(oracle, golden):
    for seq, k, expected in golden["ascii_counts"]["cases"]:
        got = as_dict(*oracle.count([fa(seq)], k, 0))
        assert got == {encode(km): c for km, c in expected}, (seq, k)


def test_count_inputs(oracle, golden):
    for case in golden["count_inputs"]["cases"]:
        got = as_dict(*oracle.count([case["fasta"].encode()], case["k"], case["x"]))
        if "exact" in case:
            assert got == {encode(km): c for km, c in case["exact"]}
        for km, c in case.get("contains", []):
            assert got[encode(km)] == c


def test_count_datasets(oracle, golden):
    for case in golden["count_datasets"]["cases"]:
        got = as_dict(*oracle.count([d.encode() for d in case["datasets"]], case["k"], case["x"], mode=1))
        if "exact" in case:
            assert got == {encode(km): c for km, c in case["exact"]}
        for km, c in case.get("contains", []):
            assert got[encode(km)] == c
        for km in case.get("absent", []):
            assert encode(km) not in got
        if "n_records" in case:
            assert len(got) == case["n_records"]


def test_simplitig_chains(oracle, golden, tmp_path):
    for k, kmers, expected in golden["simplitigs"]["chains"]:
        vals = sorted(encode(km) for km in kmers)
        lo = np.array(vals, dtype=np.uint64)
        hi = np.zeros_like(lo)
        p = tmp_path / "s.fa"
        oracle.write_simplitigs(p, lo, hi, k)
        text = p.read_text()
        seqs = [l for l in text.splitlines() if not l.startswith(">")]
        assert seqs == [expected], (k, kmers, text)


def test_simplitig_layout(oracle, golden, tmp_path):
    lay = golden["simplitigs"]["layout"]
    vals = sorted(encode(km) for km in lay["kmers"])
    lo = np.array(vals, dtype=np.uint64)
    hi = np.zeros_like(lo)
    p = tmp_path / "s.fa"
    last = oracle.write_simplitigs(p, lo, hi, lay["k"])
    text = p.read_text()
    assert lay["header"] in text and lay["line"] in text and last == 1
    last = oracle.write_simplitigs(p, lo, hi, lay["k"], lay["after_index"])
    assert lay["header_after"] in p.read_text() and last == lay["after_index"] + 1


def test_kff_signature(oracle, golden, tmp_path):
    g = golden["kff"]
    lo = np.array([encode(km) for km, _ in g["kmers"]], dtype=np.uint64)
    cnt = np.array([c for _, c in g["kmers"]], dtype=np.uint64)
    p = tmp_path / "o.kff"
    oracle.write_kff(p, lo, np.zeros_like(lo), cnt, g["k"], g["m"], g["x"], 8)
    data = p.read_bytes()
    assert data.startswith(g["starts_with"].encode()) and data.endswith(g["ends_with"].encode())
    head, recs, ok = parse_kff(data)
    assert ok and recs == {encode("ACG"): 4}
    assert head["values"] == {"k": 3, "max": 1, "data_size": 8, "ordered": 0, "m": 2, "threshold": 1}
    assert head["free_block"] == "producer=MC\nk=3\nm=2\nthreshold=1\nfilter=count>threshold\ncanonical=1\n"


def test_kff_u8_saturates_at_x_plus_one(oracle, tmp_path):
    # src/lib.rs:2489-2506: k <= 32 KFF counts saturate at min(x + 1, 255)
    lo, hi, cnt = oracle.count([fa("A" * 40)], 3, 5)
    assert int(cnt[0]) == 38
    p = tmp_path / "o.kff"
    oracle.write_kff(p, lo, hi, cnt, 3, 2, 5, 1)
    _, recs, ok = parse_kff(p.read_bytes())
    assert ok and recs == {0: 6}


def test_zi_subtract(oracle, golden):
    z = golden["zi"]
    lo, hi = oracle.zi_absent(z["subtract"]["index"].encode(), [z["subtract"]["query"].encode()], 3)
    assert sorted(to_int(lo, hi)) == sorted(encode(s) for s in z["subtract"]["absent"])
    lo, hi = oracle.zi_absent(z["dedup"]["index"].encode(), [z["dedup"]["query"].encode()], 3)
    assert to_int(lo, hi) == [encode("CCC")]


def test_mczi_subtraction_statistics(oracle, golden):
    """MCZI's scan statistics: every query window is scanned; the absent
    records' counts are their absent occurrences, so their sum is the number
    of windows not found in the index (the first case's index is MC's x = 0
    set of AAACG, i.e. all its k-mers)."""
    for c in golden["mczi_stats"]["cases"]:
        queries = [q.encode() for q in c["queries"]]
        scanned = 0
        for q in queries:
            _, offs, _ = oracle.fragments(q, c["k"])
            scanned += sum(int(offs[i + 1] - offs[i]) - c["k"] + 1 for i in range(len(offs) - 1))
        lo, hi, cnt = oracle.zi_absent_counts(c["index"].encode(), queries, c["k"])
        assert scanned == c["scanned_kmers"]
        assert int(cnt.sum()) == c["not_filtered_kmers"]
        assert scanned - int(cnt.sum()) == c["filtered_kmers"]


def test_zi_subtract_fasta_text(oracle, golden, tmp_path):
    z = golden["zi"]["subtract"]
    lo, hi = oracle.zi_absent(z["index"].encode(), [z["query"].encode()], 3)
    p = tmp_path / "out.fa"
    oracle.write_simplitigs(p, lo, hi, 3)
    text = p.read_text()
    assert any(s in text for s in z["fasta_contains_any"])


def test_reader_split(oracle, golden):
    r = golden["zi"]["reader_split"]
    codes, offs, skipped = oracle.fragments(r["fasta"].encode(), r["min_len"])
    frags = ["".join("ACGT"[c] for c in codes[offs[i]:offs[i + 1]]) for i in range(len(offs) - 1)]
    assert frags == r["fragments"] and skipped == 0


def test_reader_formats(oracle):
    # multi-line FASTA, lower case, CRLF, FASTQ; invalid record start is skipped
    codes, offs, _ = oracle.fragments(b">a\nACG\r\ntac\n>b\nGG\n", 1)
    frags = ["".join("ACGT"[c] for c in codes[offs[i]:offs[i + 1]]) for i in range(len(offs) - 1)]
    assert frags == ["ACGTAC", "GG"]
    codes, offs, _ = oracle.fragments(b"@r1\nACGNT\n+\nIIIII\n@r2\nTTT\n+\nIII\n", 1)
    frags = ["".join("ACGT"[c] for c in codes[offs[i]:offs[i + 1]]) for i in range(len(offs) - 1)]
    assert frags == ["ACG", "T", "TTT"]
    _, _, skipped = oracle.fragments(b"ACGT\n", 1)
    assert skipped == 1


def test_decode_roundtrip():
    for s in ["A", "C", "G", "T", "AC", "GT", "ACG", "TGA", "ACGT", "TTAA", "AAACG", "GATTACA", "ACGTACGT",
              "TTTTCCCC", "ACACACACAC", "ACGTACGTACGTACGT"]:
        assert decode(encode(s), len(s)) == s  # src/lib.rs:5160-5175


def test_oracle_threads_agree(oracle):
    from mczi_gb300 import gen
    data = gen.c1_reads(scale=0.001)
    a = oracle.count([data], 31, 1, threads=1)
    b = oracle.count([data], 31, 1, threads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
