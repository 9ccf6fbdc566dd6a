"""ctypes wrapper of the CPU oracle (oracle/libmczi_oracle.so).

Test infrastructure only: the parity checker for the GPU library and the
source of the CPU-baseline timing.  The product never imports this.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    so = ORACLE_DIR / "libmczi_oracle.so"
    src = ORACLE_DIR / "mczi_oracle.c"
    if not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    lib = C.CDLL(str(so))
    lib.oracle_count.restype = C.c_void_p
    lib.oracle_count.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_int, C.c_int, C.c_uint64,
                                 C.c_int, C.c_int]
    lib.oracle_zi_absent.restype = C.c_void_p
    lib.oracle_zi_absent.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_int,
                                     C.c_int]
    lib.oracle_result_status.argtypes = [C.c_void_p]
    lib.oracle_result_len.restype = C.c_uint64
    lib.oracle_result_len.argtypes = [C.c_void_p]
    lib.oracle_result_skipped.restype = C.c_uint64
    lib.oracle_result_skipped.argtypes = [C.c_void_p]
    lib.oracle_result_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.oracle_result_free.argtypes = [C.c_void_p]
    lib.oracle_fragments.restype = C.c_int
    lib.oracle_fragments.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.oracle_write_kff.restype = C.c_int
    lib.oracle_write_kff.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_int,
                                     C.c_uint64, C.c_int]
    lib.oracle_write_simplitigs.restype = C.c_int64
    lib.oracle_write_simplitigs.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_uint64]
    lib.oracle_count_digest.restype = C.c_int
    lib.oracle_count_digest.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_int, C.c_int, C.c_uint64,
                                        C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.oracle_zi_absent_digest.restype = C.c_int
    lib.oracle_zi_absent_digest.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                            C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint64)]
    lib.oracle_records_digest.restype = None
    lib.oracle_records_digest.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    _lib = lib
    return lib


def _arrays(bufs):
    arrs = [np.frombuffer(b, dtype=np.uint8) if not isinstance(b, np.ndarray) else np.ascontiguousarray(b)
            for b in bufs]
    ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data if a.size else None for a in arrs])
    lens = (C.c_uint64 * len(arrs))(*[a.size for a in arrs])
    return arrs, ptrs, lens


def _take(h):
    lib = load()
    try:
        if lib.oracle_result_status(h) != 0:
            raise ValueError("oracle rejected the configuration")
        n = lib.oracle_result_len(h)
        lo = np.empty(n, dtype=np.uint64)
        hi = np.empty(n, dtype=np.uint64)
        cnt = np.empty(n, dtype=np.uint64)
        if n:
            lib.oracle_result_copy(h, lo.ctypes.data, hi.ctypes.data, cnt.ctypes.data)
        return lo, hi, cnt
    finally:
        lib.oracle_result_free(h)


def count(bufs, k: int, x: int, mode: int = 0, threads: int = 4):
    """Sorted (lo, hi, count) of canonical k-mers with count > x."""
    arrs, ptrs, lens = _arrays(bufs)
    h = load().oracle_count(ptrs, lens, len(arrs), k, x, mode, threads)
    return _take(h)


def zi_absent_counts(index, queries, k: int):
    """Sorted (lo, hi, count) of the canonical query k-mers absent from the
    index; count = the k-mer's absent occurrences over the queries."""
    ia = np.frombuffer(index, dtype=np.uint8) if not isinstance(index, np.ndarray) else index
    arrs, ptrs, lens = _arrays(queries)
    h = load().oracle_zi_absent(ia.ctypes.data if ia.size else None, ia.size, ptrs, lens, len(arrs), k)
    return _take(h)


def zi_absent(index, queries, k: int):
    """Sorted (lo, hi) of the canonical query k-mers absent from the index."""
    lo, hi, _ = zi_absent_counts(index, queries, k)
    return lo, hi


def fragments(buf, min_len: int):
    a = np.frombuffer(buf, dtype=np.uint8) if not isinstance(buf, np.ndarray) else buf
    nc, nf = C.c_uint64(), C.c_uint64()
    lib = load()
    lib.oracle_fragments(a.ctypes.data if a.size else None, a.size, min_len, None, None, C.byref(nc), C.byref(nf))
    codes = np.empty(nc.value, dtype=np.uint8)
    offs = np.empty(nf.value + 1, dtype=np.uint64)
    skipped = lib.oracle_fragments(a.ctypes.data if a.size else None, a.size, min_len,
                                   codes.ctypes.data if nc.value else None, offs.ctypes.data, C.byref(nc),
                                   C.byref(nf))
    return codes, offs, skipped


def write_kff(path, lo, hi, cnt, k, m, x, count_size):
    lo = np.ascontiguousarray(lo, dtype=np.uint64)
    hi = np.ascontiguousarray(hi, dtype=np.uint64)
    cnt = np.ascontiguousarray(cnt, dtype=np.uint64)
    rc = load().oracle_write_kff(str(path).encode(), lo.ctypes.data, hi.ctypes.data, cnt.ctypes.data, lo.size, k, m,
                                 x, count_size)
    assert rc == 0


def write_simplitigs(path, lo, hi, k, first_index=0):
    lo = np.ascontiguousarray(lo, dtype=np.uint64)
    hi = np.ascontiguousarray(hi, dtype=np.uint64)
    return load().oracle_write_simplitigs(str(path).encode(), lo.ctypes.data, hi.ctypes.data, lo.size, k,
                                          first_index)


def encode(seq: str) -> int:
    v = 0
    for ch in seq:
        v = (v << 2) | "ACGT".index(ch)
    return v


def decode(v: int, k: int) -> str:
    return "".join("ACGT"[(v >> (2 * (k - 1 - i))) & 3] for i in range(k))


def to_int(lo, hi):
    return [(int(h) << 64) | int(l) for l, h in zip(lo, hi)]


def parse_kff(data: bytes):
    """Returns (header dict, records as {encoded: count}, trailer ok)."""
    assert data[:3] == b"KFF"
    p = 3 + 5
    fbl = int.from_bytes(data[p:p + 4], "big")
    p += 4
    free_block = data[p:p + fbl].decode()
    p += fbl
    assert data[p:p + 1] == b"v"
    p += 1
    nv = int.from_bytes(data[p:p + 8], "big")
    p += 8
    vals = {}
    for _ in range(nv):
        e = data.index(b"\0", p)
        name = data[p:e].decode()
        p = e + 1
        vals[name] = int.from_bytes(data[p:p + 8], "big")
        p += 8
    assert data[p:p + 1] == b"r"
    p += 1
    n = int.from_bytes(data[p:p + 8], "big")
    p += 8
    hdr_end = p
    k = vals["k"]
    nb = (k + 3) // 4
    cs = vals["data_size"]
    recs = {}
    for _ in range(n):
        key = int.from_bytes(data[p:p + nb], "big")
        p += nb
        c = int.from_bytes(data[p:p + cs], "big")
        p += cs
        recs[key] = c
    trailer = data[p:] == b"KFF"
    return {"free_block": free_block, "values": vals, "n": n, "head": data[:hdr_end]}, recs, trailer


def _digest_dict(out) -> dict:
    return {"records": int(out[0]), "count_sum": int(out[1]), "sum": "%016x" % out[2], "xor": "%016x" % out[3]}


def count_digest(bufs, k: int, x: int, mode: int = 0, threads: int | None = None, passes: int = 1) -> dict:
    """Digest (mczi_gb300.digest's definition) of what count() would return,
    computed in `passes` hash-range passes so that memory stays bounded."""
    from mczi_gb300._native import default_threads
    arrs, ptrs, lens = _arrays(bufs)
    out = (C.c_uint64 * 4)()
    skipped = C.c_uint64()
    rc = load().oracle_count_digest(ptrs, lens, len(arrs), k, x, mode, threads or default_threads(), passes, out,
                                    C.byref(skipped))
    if rc != 0:
        raise ValueError("oracle rejected the configuration")
    return _digest_dict(out)


def records_digest(lo, hi, cnt) -> dict:
    lo = np.ascontiguousarray(lo, dtype=np.uint64)
    cnt = np.ascontiguousarray(cnt, dtype=np.uint64)
    hi = None if hi is None else np.ascontiguousarray(hi, dtype=np.uint64)
    out = (C.c_uint64 * 4)()
    load().oracle_records_digest(lo.ctypes.data, hi.ctypes.data if hi is not None else None, cnt.ctypes.data, lo.size,
                                 out)
    return _digest_dict(out)


def zi_absent_digest(index, queries, k: int, threads: int | None = None, passes: int = 1) -> dict:
    """Digest of zi_absent()'s set (every record with count 1), in `passes`
    hash-range passes over the queries."""
    from mczi_gb300._native import default_threads
    ia = np.frombuffer(index, dtype=np.uint8) if not isinstance(index, np.ndarray) else index
    arrs, ptrs, lens = _arrays(queries)
    out = (C.c_uint64 * 4)()
    rc = load().oracle_zi_absent_digest(ia.ctypes.data if ia.size else None, ia.size, ptrs, lens, len(arrs), k,
                                        threads or default_threads(), passes, out)
    if rc != 0:
        raise ValueError("oracle rejected k")
    return _digest_dict(out)
