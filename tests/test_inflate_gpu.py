"""gzip inputs decoded on the device (mczi_inflate_gzip and the counting /
ZI entry points), against Python's zlib and the oracle on the decoded bytes.

The reference decompresses gzip inputs in front of its FASTX parser
(src/lib.rs:3127-3143); inputs whose members carry their sizes (BGZF) are
decoded here in HBM, one warp per member, every member checked against its
ISIZE and CRC-32.  Covered: stored, fixed-Huffman and dynamic blocks, long
overlapping matches (distance 1), empty members, incompressible data, FASTQ
and non-FASTX content, corrupt members (an error, never a fault), and gzip
files without sizes (decoded on the host).
"""
import ctypes as C
import gzip
import zlib

import numpy as np
import pytest

from mczi_gb300 import bgzf
from oracle_ref import parse_kff, to_int

pytestmark = pytest.mark.gpu


def _inflate(ctx, gz: bytes):
    from mczi_gb300 import _native as N
    lib = N.load()
    n = C.c_uint64()
    rc = lib.mczi_inflate_gzip(ctx.handle, gz, len(gz), None, 0, C.byref(n))
    if rc != 0 and rc != N.MCZI_ERR_TOO_LARGE:
        return rc, None
    out = (C.c_uint8 * max(1, n.value))()
    rc = lib.mczi_inflate_gzip(ctx.handle, gz, len(gz), out, n.value, C.byref(n))
    return rc, bytes(out)[: n.value]


CASES = [
    ("default", 6, zlib.Z_DEFAULT_STRATEGY),
    ("stored", 0, zlib.Z_DEFAULT_STRATEGY),
    ("fast", 1, zlib.Z_DEFAULT_STRATEGY),
    ("best", 9, zlib.Z_DEFAULT_STRATEGY),
    ("fixed", 6, zlib.Z_FIXED),
    ("huffman_only", 6, zlib.Z_HUFFMAN_ONLY),
    ("rle", 6, zlib.Z_RLE),
    ("filtered", 6, zlib.Z_FILTERED),
]


@pytest.mark.parametrize("name,level,strategy", CASES)
def test_inflate_matches_zlib(gpu_ctx, name, level, strategy):
    from mczi_gb300 import gen
    rng = np.random.default_rng(7)
    fasta = gen.c1_reads(scale=0.002).tobytes()
    parts = [
        fasta,
        b"A" * 200_000,                                  # distance-1 matches of 258 bytes
        (b"ACGTTGCA" * 40_000),                           # short-period matches
        rng.integers(0, 256, 150_000, dtype=np.uint8).tobytes(),  # incompressible: stored blocks
        b"",
    ]
    data = b"".join(parts)
    gz = bgzf.compress(data, level, strategy)
    assert gzip.decompress(gz) == data
    rc, out = _inflate(gpu_ctx, gz)
    assert rc == 0
    assert out == data


def test_inflate_member_sizes_and_empty(gpu_ctx):
    # odd member sizes, one-byte members and an input that is only the end marker
    data = bytes(range(256)) * 3000
    for block in (1, 7, 4096, 65280):
        gz = bgzf.compress(data[: 20 * block + 3], block=block)
        rc, out = _inflate(gpu_ctx, gz)
        assert rc == 0 and out == data[: 20 * block + 3]
    rc, out = _inflate(gpu_ctx, bgzf.member(b""))
    assert rc == 0 and out == b""


def test_inflate_rejects_and_reports(gpu_ctx):
    from mczi_gb300 import _native as N
    data = b">r\n" + b"ACGT" * 100_000 + b"\n"
    # no sizes in the members: not decodable here
    rc, _ = _inflate(gpu_ctx, gzip.compress(data))
    assert rc == N.MCZI_ERR_INVALID_CONFIG
    # a member whose size runs past the buffer
    gz = bgzf.compress(data)
    rc, _ = _inflate(gpu_ctx, gz[: len(gz) - 40])
    assert rc == N.MCZI_ERR_INVALID_CONFIG
    # corrupt DEFLATE data, a wrong CRC, a wrong ISIZE: errors, never a fault
    m = bytearray(bgzf.member(data[:60_000]))
    for at, val in ((40, 0xFF), (len(m) - 8, m[len(m) - 8] ^ 1), (len(m) - 4, m[len(m) - 4] ^ 1)):
        bad = bytearray(m)
        bad[at] = val
        rc, _ = _inflate(gpu_ctx, bytes(bad))
        assert rc == N.MCZI_ERR_IO
    # random bytes as DEFLATE data
    rng = np.random.default_rng(3)
    for trial in range(20):
        junk = rng.integers(0, 256, 3000, dtype=np.uint8).tobytes()
        bsize = 10 + 2 + 6 + len(junk) + 8 - 1
        head = bytes([0x1F, 0x8B, 8, 4, 0, 0, 0, 0, 0, 0xFF, 6, 0, ord("B"), ord("C"), 2, 0]) + bsize.to_bytes(2, "little")
        fake = head + junk + (0).to_bytes(4, "little") + (5000).to_bytes(4, "little")
        rc, _ = _inflate(gpu_ctx, fake)
        assert rc == N.MCZI_ERR_IO
    # the context stays usable
    rc, out = _inflate(gpu_ctx, bgzf.compress(data))
    assert rc == 0 and out == data


def test_count_bgzf_inputs_in_memory(gpu_ctx, oracle):
    """mczi_count with BGZF, plain-gzip and plain inputs mixed: the result of
    the decoded bytes (FASTA and FASTQ; a non-FASTX input is skipped)."""
    from mczi_gb300 import gen
    from mczi_gb300.mc import CounterConfig
    fa = gen.c1_reads(scale=0.01)
    half = fa.size // 2
    cut = int(np.flatnonzero(fa[half:] == ord(">"))[0]) + half
    a, b = fa[:cut].tobytes(), fa[cut:].tobytes()
    # a FASTQ version of a's records
    lines = a.split(b"\n")
    fq = bytearray()
    for i in range(0, len(lines) - 1, 2):
        if lines[i].startswith(b">"):
            seq = lines[i + 1]
            fq += b"@" + lines[i][1:] + b"\n" + seq + b"\n+\n" + b"I" * len(seq) + b"\n"
    fq = bytes(fq)
    inputs = [bgzf.compress(a), gzip.compress(b), bgzf.compress(fq, level=1), bgzf.compress(b"not a fastx file\n")]
    cfg = CounterConfig(31, 21, 1)
    n = gpu_ctx.count(inputs, cfg)
    r = gpu_ctx.records(n, sorted=True)
    lo, hi, cnt = oracle.count([a, b, fq], 31, 1)
    assert np.array_equal(r.lo, lo) and np.array_equal(r.count, cnt)
    # the same bytes uncompressed give the same result
    n2 = gpu_ctx.count([a, b, fq], cfg)
    r2 = gpu_ctx.records(n2, sorted=True)
    assert np.array_equal(r.lo, r2.lo) and np.array_equal(r.count, r2.count)


def test_count_and_zi_bgzf_paths(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import _native as N, gen
    lib = N.load()
    data = gen.c2_reads(scale=0.002).tobytes()
    (tmp_path / "r.fa.gz").write_bytes(bgzf.compress(data))
    (tmp_path / "r.fa").write_bytes(data)
    cfg = N.CounterConfigC(63, 21, 2, 1024)
    outs = []
    for name in ("r.fa.gz", "r.fa"):
        out = tmp_path / (name + ".kff")
        arr = (C.c_char_p * 1)(str(tmp_path / name).encode())
        rc = lib.mczi_count_inputs_to_kff_path(gpu_ctx.handle, arr, 1, C.byref(cfg), str(out).encode())
        assert rc == 0, lib.mczi_last_error(gpu_ctx.handle)
        head, recs, ok = parse_kff(out.read_bytes())
        assert ok
        outs.append(recs)
    assert outs[0] == outs[1]  # the same record set (emission order may differ)
    lo, hi, cnt = oracle.count([data], 63, 2)
    exp = dict(zip(to_int(lo, hi), (int(c) for c in cnt)))
    if head["values"]["data_size"] == 1:  # one-byte counts saturate at x + 1
        exp = {e: min(c, 3) for e, c in exp.items()}
    assert outs[0] == exp
    # ZI build and query paths with BGZF index and query files
    index, query = gen.c4_index_and_query(genome_len=200_000, query_bases=2_000_000, k=31)
    (tmp_path / "idx.fa.gz").write_bytes(bgzf.compress(index.tobytes()))
    (tmp_path / "q.fa.gz").write_bytes(bgzf.compress(query.tobytes()))
    assert lib.mczi_zi_build_path(gpu_ctx.handle, str(tmp_path / "idx.fa.gz").encode(), 31, 19) == 0
    n = C.c_uint64()
    arr = (C.c_char_p * 1)(str(tmp_path / "q.fa.gz").encode())
    rc = lib.mczi_zi_query_paths(gpu_ctx.handle, arr, 1, C.byref(n))
    assert rc == 0, lib.mczi_last_error(gpu_ctx.handle)
    gpu_ctx.k = 31
    r = gpu_ctx.records(n.value, sorted=True)
    lo, hi = oracle.zi_absent(index, [query], 31)
    assert np.array_equal(r.lo, lo)
