"""The selected-k-mer FASTA (mczi_write_kmer_fasta; the files of the
reference's count_inputs_to_kmer_fasta_path / count_datasets_to_kmer_fasta_path,
src/lib.rs:306-425, records as src/lib.rs:1535-1544), on the CPU: the writer
is host code of libmczi_gpu, fed here with the oracle's records.  The GPU
entry points (mc.count_*_to_kmer_fasta_path) are the parity-tested count and
record copy followed by this writer.
"""
import numpy as np
import pytest


def _records(oracle, bufs, k, x, mode):
    from mczi_gb300.mc import Records
    lo, hi, cnt = oracle.count(bufs, k, x, mode)
    return Records(lo, hi if k > 32 else None, cnt, k)


def _write(tmp_path, rec, name="kmers.fa"):
    from mczi_gb300.mc import write_kmer_fasta
    out = tmp_path / name
    n = write_kmer_fasta(rec, out)
    return n, out.read_text()


def test_reference_known_answers(tmp_path, oracle):
    # src/lib.rs:6100-6135: one read AAAA, k=3 x=1 -> AAA seen twice
    n, text = _write(tmp_path, _records(oracle, [b">r\nAAAA\n"], 3, 1, 0))
    assert n == 1 and ">MC_kmer_1 count=2\nAAA\n" in text
    # src/lib.rs:6137-6170: two datasets holding AAAA, presence, x=1
    n, text = _write(tmp_path, _records(oracle, [b">d\nAAAA\n", b">d\nAAAA\n"], 3, 1, 1))
    assert n == 1 and ">MC_kmer_1 count=2\nAAA\n" in text
    # src/lib.rs:5805-5843: presence over three datasets, x=2: only ACG is in all three
    ds = [b">d1\nAAAACGACG\n", b">d2\nAAAACGTTT\n", b">d3\nGGGACGCCC\n"]
    n, text = _write(tmp_path, _records(oracle, ds, 3, 2, 1))
    assert n == 1 and "\nACG\n" in text and "\nAAA\n" not in text


@pytest.mark.parametrize("k,x,mode", [(31, 1, 0), (63, 0, 0), (21, 1, 1)])
def test_records_round_trip(tmp_path, oracle, k, x, mode):
    rng = np.random.default_rng(k)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=5000).tobytes()
    bufs = []
    for d in range(3 if mode else 1):
        recs = []
        for i in range(120):
            a = int(rng.integers(0, 4800))
            recs.append(b">r%d\n" % i + g[a:a + int(rng.integers(k, 200))] + b"\n")
        bufs.append(b"".join(recs))
    rec = _records(oracle, bufs, k, x, mode)
    n, text = _write(tmp_path, rec)
    assert n == len(rec) > 0
    lines = text.split("\n")
    assert lines[-1] == "" and len(lines) == 2 * n + 1
    code = {"A": 0, "C": 1, "G": 2, "T": 3}
    hi = rec.hi if rec.hi is not None else np.zeros_like(rec.lo)
    for i in range(n):
        assert lines[2 * i] == ">MC_kmer_%d count=%d" % (i + 1, int(rec.count[i]))
        seq = lines[2 * i + 1]
        assert len(seq) == k
        v = 0
        for ch in seq:
            v = (v << 2) | code[ch]
        assert v == (int(hi[i]) << 64) | int(rec.lo[i])


def test_empty_set_and_errors(tmp_path):
    from mczi_gb300 import _native as N
    from mczi_gb300.mc import Records
    e = np.empty(0, dtype=np.uint64)
    n, text = _write(tmp_path, Records(e, None, e, 31), "empty.fa")
    assert n == 0 and text == ""
    one = np.array([5], dtype=np.uint64)
    with pytest.raises(N.MCZIError, match="failed to create"):
        _write(tmp_path / "no-such-folder", Records(one, None, one, 31))
    with pytest.raises(N.MCZIError):
        _write(tmp_path, Records(one, None, one, 65))  # k beyond 64
    with pytest.raises(N.MCZIError):
        _write(tmp_path, Records(one, None, one, 33))  # k > 32 needs the high words


def test_many_records_across_blocks(tmp_path):
    """More records than one block of every host thread: the file is the
    records in order, each formatted as the reference formats it."""
    from mczi_gb300.mc import Records, write_kmer_fasta
    n = 700_001
    rng = np.random.default_rng(3)
    lo = rng.integers(0, 2**62, size=n, dtype=np.uint64)
    hi = rng.integers(0, 2**60, size=n, dtype=np.uint64)
    cnt = rng.integers(0, 2**64 - 1, size=n, dtype=np.uint64, endpoint=True)
    cnt[:3] = [0, 1, 2**64 - 1]
    k = 63
    out = tmp_path / "many.fa"
    assert write_kmer_fasta(Records(lo, hi, cnt, k), out) == n
    lines = out.read_bytes().split(b"\n")
    assert len(lines) == 2 * n + 1 and lines[-1] == b""
    for i in [0, 1, 2, 3, 131071, 131072, 131073, 262144, 699_999, n - 1] + list(rng.integers(0, n, size=200)):
        i = int(i)
        assert lines[2 * i] == b">MC_kmer_%d count=%d" % (i + 1, int(cnt[i]))
        v = (int(hi[i]) << 64) | int(lo[i])
        assert lines[2 * i + 1] == bytes(b"ACGT"[(v >> (2 * (k - 1 - j))) & 3] for j in range(k))
