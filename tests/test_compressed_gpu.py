"""Compressed inputs through the C ABI's path-based entry points, against the
oracle on the decompressed bytes.

mczi_count_inputs_to_kff_path / mczi_count_datasets_to_kff_path (MC's
count_inputs_to_kff_path src/lib.rs:457 and count_datasets_to_kff_path :509)
and mczi_zi_build_path / mczi_zi_query_paths (ZI's build_dictionary
src/zi.rs:114 and collect_query_kmers_absent_from_index :152) take gzip, xz
and zstd files as the reference's readers do.
"""
import ctypes as C
import gzip
import lzma

import numpy as np
import pytest

from oracle_ref import parse_kff, to_int
from test_decompress import zstd_compress

pytestmark = pytest.mark.gpu


def _paths(ps):
    arr = (C.c_char_p * len(ps))(*[str(p).encode() for p in ps])
    return arr


def test_compressed_inputs_count_to_kff(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import _native as N, gen
    lib = N.load()
    data = gen.c1_reads(scale=0.01)
    half = len(data) // 2
    cut = int(np.flatnonzero(data[half:] == ord(">"))[0]) + half
    a, b = data[:cut].tobytes(), data[cut:].tobytes()
    (tmp_path / "a.fa.gz").write_bytes(gzip.compress(a))
    (tmp_path / "b.fa.xz").write_bytes(lzma.compress(b))
    cfg = N.CounterConfigC(31, 21, 2, 1024)
    out = tmp_path / "out.kff"
    rc = lib.mczi_count_inputs_to_kff_path(gpu_ctx.handle, _paths([tmp_path / "a.fa.gz", tmp_path / "b.fa.xz"]), 2,
                                           C.byref(cfg), str(out).encode())
    assert rc == 0, lib.mczi_last_error(gpu_ctx.handle)
    _, recs, ok = parse_kff(out.read_bytes())
    assert ok
    lo, hi, cnt = oracle.count([a, b], 31, 2)
    assert recs == {e: min(c, 3) for e, c in zip(to_int(lo, hi), (int(c) for c in cnt))}
    # fof mode over a zstd and a gzip dataset
    (tmp_path / "c.fa.zst").write_bytes(zstd_compress(a))
    rc = lib.mczi_count_datasets_to_kff_path(gpu_ctx.handle, _paths([tmp_path / "c.fa.zst", tmp_path / "a.fa.gz"]),
                                             2, C.byref(N.CounterConfigC(31, 21, 1, 1024)), str(out).encode())
    assert rc == 0, lib.mczi_last_error(gpu_ctx.handle)
    _, recs, ok = parse_kff(out.read_bytes())
    lo, hi, cnt = oracle.count([a, a], 31, 1, 1)
    assert recs == dict(zip(to_int(lo, hi), (int(c) for c in cnt)))
    # a truncated input fails with MCZI_ERR_IO and a message
    (tmp_path / "bad.gz").write_bytes(gzip.compress(a)[:1000])
    rc = lib.mczi_count_inputs_to_kff_path(gpu_ctx.handle, _paths([tmp_path / "bad.gz"]), 1, C.byref(cfg),
                                           str(out).encode())
    assert rc == N.MCZI_ERR_IO and b"bad.gz" in lib.mczi_last_error(gpu_ctx.handle)


def test_compressed_zi_paths(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import _native as N, gen
    lib = N.load()
    index, query = gen.c4_index_and_query(genome_len=200_000, query_bases=2_000_000, k=31)
    (tmp_path / "idx.fa.xz").write_bytes(lzma.compress(index.tobytes()))
    (tmp_path / "q.fa.gz").write_bytes(gzip.compress(query.tobytes()))
    (tmp_path / "q2.fa.zst").write_bytes(zstd_compress(query[: query.size // 3].tobytes()))
    assert lib.mczi_zi_build_path(gpu_ctx.handle, str(tmp_path / "idx.fa.xz").encode(), 31, 19) == 0
    n = C.c_uint64()
    rc = lib.mczi_zi_query_paths(gpu_ctx.handle, _paths([tmp_path / "q.fa.gz", tmp_path / "q2.fa.zst"]), 2,
                                 C.byref(n))
    assert rc == 0, lib.mczi_last_error(gpu_ctx.handle)
    gpu_ctx.k = 31
    r = gpu_ctx.records(n.value, sorted=True)
    lo, hi = oracle.zi_absent(index, [query, query[: query.size // 3]], 31)
    assert np.array_equal(r.lo, lo)
