"""Order-independent digest of a count's kept records.

A result set of (canonical k-mer, count) records -- from MC counting or a ZI
subtraction -- is summarised by four numbers: the record count, the sum of
the counts, and the wrapping 64-bit sum and the xor of one mixed word per
record, ``mix64(mix64(mix64(lo) ^ hi) + count)`` with ``mix64`` the
murmur3 64-bit finaliser.  Two runs that kept the same records give the same
digest in any record order, so a large result (billions of input bases) can
be compared with a digest computed elsewhere without moving the records.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xff51afd7ed558ccd)
_M2 = np.uint64(0xc4ceb9fe1a85ec53)
_S = np.uint64(33)


def _mix64(x: np.ndarray) -> np.ndarray:
    x = x ^ (x >> _S)
    x = x * _M1
    x ^= x >> _S
    x *= _M2
    return x ^ (x >> _S)


def records_digest(key_lo, key_hi, counts, chunk: int = 1 << 22) -> dict:
    """Digest of records given as arrays (key_hi None for k <= 32)."""
    lo = np.asarray(key_lo, dtype=np.uint64)
    cnt = np.asarray(counts, dtype=np.uint64)
    hi = np.asarray(key_hi, dtype=np.uint64) if key_hi is not None else None
    n = lo.size
    s = np.uint64(0)
    x = np.uint64(0)
    csum = 0
    with np.errstate(over="ignore"):
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            h = _mix64(lo[a:b].copy())
            if hi is not None:
                h ^= hi[a:b]
            w = _mix64(_mix64(h) + cnt[a:b])
            s = np.uint64(s + np.add.reduce(w, dtype=np.uint64))
            x = np.uint64(x ^ np.bitwise_xor.reduce(w))
            csum += int(np.add.reduce(cnt[a:b], dtype=np.uint64))
    return {"records": int(n), "count_sum": int(csum), "sum": "%016x" % int(s), "xor": "%016x" % int(x)}
