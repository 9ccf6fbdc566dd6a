"""Compressed inputs of the path-based entry points, on the CPU.

MC and ZI read gzip, xz and zstd inputs (src/lib.rs:3127-3143, 3218-3226).
The library recognises the format by magic bytes and decodes it with the
system's zlib / liblzma / libzstd loaded at run time (csrc/decompress.cpp);
mczi_read_input_file is the host-only entry point these tests call (no
device needed).  Covered: plain, multi-member gzip, concatenated xz streams,
multi-frame zstd, a compressed file with a misleading name, an empty file,
and truncated or corrupt streams, which must fail with MCZI_ERR_IO and a
message, not return partial data; and the reference's own gzip, xz and
invalid-input cases counted by the oracle.
"""
import ctypes as C
import ctypes.util
import gzip
import lzma

import numpy as np
import pytest


def payload(seed=0, n=300_000):
    rng = np.random.default_rng(seed)
    seq = rng.choice(np.frombuffer(b"ACGTN", dtype=np.uint8), size=n).tobytes()
    return b"".join(b">r%d\n%s\n" % (i, seq[i * 150:(i + 1) * 150]) for i in range(n // 150))


def read(path):
    from mczi_gb300 import mc
    return mc.read_input(path)


def zstd_compress(data: bytes, level=3):
    name = ctypes.util.find_library("zstd")
    if not name:
        pytest.skip("libzstd not on this host")
    z = C.CDLL(name)
    z.ZSTD_compressBound.restype = C.c_size_t
    z.ZSTD_compressBound.argtypes = [C.c_size_t]
    z.ZSTD_compress.restype = C.c_size_t
    z.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
    cap = z.ZSTD_compressBound(len(data))
    out = C.create_string_buffer(cap)
    n = z.ZSTD_compress(out, cap, data, len(data), level)
    return out.raw[:n]


@pytest.fixture(scope="module", autouse=True)
def lib():
    from mczi_gb300 import build
    build.build_gpu_lib()


def test_plain_and_empty(tmp_path):
    d = payload(1)
    (tmp_path / "a.fa").write_bytes(d)
    (tmp_path / "e.fa").write_bytes(b"")
    assert read(tmp_path / "a.fa") == d
    assert read(tmp_path / "e.fa") == b""


def test_gzip_multi_member(tmp_path):
    a, b = payload(2), payload(3)
    (tmp_path / "x.fa.gz").write_bytes(gzip.compress(a) + gzip.compress(b, compresslevel=1))
    assert read(tmp_path / "x.fa.gz") == a + b


def test_xz_concatenated(tmp_path):
    a, b = payload(4), payload(5)
    (tmp_path / "x.fa.xz").write_bytes(lzma.compress(a) + lzma.compress(b))
    assert read(tmp_path / "x.fa.xz") == a + b


def test_zstd_frames(tmp_path):
    a, b = payload(6), payload(7)
    (tmp_path / "x.fa.zst").write_bytes(zstd_compress(a) + zstd_compress(b, 9))
    assert read(tmp_path / "x.fa.zst") == a + b


def test_format_by_magic_not_name(tmp_path):
    d = payload(8)
    (tmp_path / "looks_plain.fa").write_bytes(gzip.compress(d))
    assert read(tmp_path / "looks_plain.fa") == d
    (tmp_path / "looks_gz.gz").write_bytes(d)  # plain text under a .gz name
    assert read(tmp_path / "looks_gz.gz") == d


@pytest.mark.parametrize("kind", ["gz", "xz", "zst"])
def test_truncated_and_corrupt_fail(tmp_path, kind):
    from mczi_gb300 import MCZIError, _native as N
    d = payload(9)
    comp = {"gz": gzip.compress, "xz": lzma.compress, "zst": zstd_compress}[kind](d)
    (tmp_path / f"t.{kind}").write_bytes(comp[: len(comp) // 2])
    with pytest.raises(MCZIError) as e:
        read(tmp_path / f"t.{kind}")
    assert e.value.code == N.MCZI_ERR_IO and str(e.value)
    bad = bytearray(comp)
    for i in range(len(bad) // 3, len(bad) // 3 + 64):
        bad[i] ^= 0x5A
    (tmp_path / f"c.{kind}").write_bytes(bytes(bad))
    with pytest.raises(MCZIError) as e:
        read(tmp_path / f"c.{kind}")
    assert e.value.code == N.MCZI_ERR_IO


def test_missing_file(tmp_path):
    from mczi_gb300 import MCZIError
    with pytest.raises(MCZIError, match="failed to open"):
        read(tmp_path / "nope.fa")


def test_reference_compressed_and_invalid_inputs(tmp_path, oracle):
    """The reference's own cases (src/lib.rs:5609-5740): ACGTACGT through
    gzip and xz counts to ACG:4, GTA:2 at k=3 x=1; an input that is not
    FASTA/FASTQ, plain or gzip-compressed, is skipped, not an error."""
    from oracle_ref import encode
    fa = b">read\nACGTACGT\n"
    want = {encode("ACG"): 4, encode("GTA"): 2}
    (tmp_path / "r.fa.gz").write_bytes(gzip.compress(fa))
    (tmp_path / "r.fa.xz").write_bytes(lzma.compress(fa))
    (tmp_path / "bad.txt").write_bytes(b"not a FASTA or FASTQ file\n")
    (tmp_path / "bad.fa.gz").write_bytes(gzip.compress(b"not a FASTA or FASTQ file\n"))
    for name in ("r.fa.gz", "r.fa.xz"):
        lo, hi, cnt = oracle.count([read(tmp_path / name)], 3, 1)
        assert dict(zip((int(v) for v in lo), (int(c) for c in cnt))) == want, name
    for bad in ("bad.txt", "bad.fa.gz"):
        data = [read(tmp_path / bad), read(tmp_path / "r.fa.gz")]
        assert data[0] == b"not a FASTA or FASTQ file\n"  # decoded, then skipped by the parser
        lo, hi, cnt = oracle.count(data, 3, 1)
        assert dict(zip((int(v) for v in lo), (int(c) for c in cnt))) == want, bad


@pytest.mark.parametrize("ext", [".gz", ".gzip", ".xz", ".zst", ".zstd", ".fa"])
def test_outputs_compressed_by_extension(tmp_path, ext):
    """Outputs are compressed by their extension as MC's output writer does
    (src/lib.rs:1355-1405); each reads back through the library's readers."""
    from mczi_gb300.mc import _write_through
    d = payload(3, 60_000)
    out = tmp_path / ("out.fa" + ext if ext != ".fa" else "out.fa")
    _write_through(out, lambda p: p.write_bytes(d))
    raw = out.read_bytes()
    magic = {".gz": b"\x1f\x8b", ".gzip": b"\x1f\x8b", ".xz": b"\xfd7zXZ\x00", ".zst": b"\x28\xb5\x2f\xfd",
             ".zstd": b"\x28\xb5\x2f\xfd", ".fa": b">"}[ext]
    assert raw.startswith(magic)
    assert read(out) == d
    assert not list(tmp_path.glob("*.tmp-plain"))


@pytest.mark.parametrize("ext", [".gz", ".GZIP", ".xz", ".zst", ".zstd", ".kff"])
@pytest.mark.parametrize("size", [0, 1, 3_000_000])
def test_native_compress_output(tmp_path, ext, size):
    """mczi_compress_output, the reference's compress_existing_file step
    (src/lib.rs:1355-1405): the output reads back through the library's own
    readers to the plain bytes, whatever its size."""
    from mczi_gb300 import _native as N
    lib = N.load()
    d = payload(5, max(size, 150))[:size]
    plain, out = tmp_path / "plain.bin", tmp_path / ("out" + ext)
    plain.write_bytes(d)
    err = C.create_string_buffer(512)
    assert lib.mczi_compress_output(str(plain).encode(), str(out).encode(), err, len(err)) == 0, err.value
    raw = out.read_bytes()
    magic = {".gz": b"\x1f\x8b", ".GZIP": b"\x1f\x8b", ".xz": b"\xfd7zXZ\x00", ".zst": b"\x28\xb5\x2f\xfd",
             ".zstd": b"\x28\xb5\x2f\xfd", ".kff": d[:1]}[ext]
    assert raw.startswith(magic)
    if ext == ".kff":
        assert raw == d
    assert read(out) == d


def test_native_compress_output_errors(tmp_path):
    from mczi_gb300 import _native as N
    lib = N.load()
    err = C.create_string_buffer(512)
    rc = lib.mczi_compress_output(str(tmp_path / "missing").encode(), str(tmp_path / "o.gz").encode(), err, len(err))
    assert rc == N.MCZI_ERR_IO and b"failed to open" in err.value
    (tmp_path / "p").write_bytes(b">r\nACGT\n")
    rc = lib.mczi_compress_output(str(tmp_path / "p").encode(), str(tmp_path / "no" / "o.xz").encode(), err,
                                  len(err))
    assert rc == N.MCZI_ERR_IO and b"failed to create" in err.value
