"""ZI on the GPU: subtract a device-resident k-mer index from query k-mers.

Mirrors ZI (``src/zi.rs``): ``validate_k`` (:103-107), ``default_minimizer_size``
(:109-112), ``build_dictionary`` (:114-141), ``collect_query_kmers_absent_from_index``
(:152-175) and ``write_novel_simplitigs`` (:177-189).  The dictionary lives in
HBM inside a :class:`mczi_gb300.mc.Context` and is reused by every query until
the next build.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

from . import _native as N
from .mc import Context, Records, _inputs_c, _write_through, default_context, read_input


def validate_k(k: int) -> None:
    if not 3 <= k <= 63:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "k must be in [3, 63] for sshash-rs")
    if k % 2 == 0:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "k must be odd for sshash-rs")


def default_minimizer_size(k: int) -> int:
    m = min(19, k - 2)
    return m if m % 2 == 1 else m - 1


def _bytes(x):
    if isinstance(x, (bytes, bytearray, memoryview, np.ndarray, tuple)):
        return x
    return read_input(x)


def build_dictionary(index, k: int, m: int | None = None, ctx: Context | None = None) -> Context:
    """Builds the device dictionary of the canonical k-mers of `index`
    (a FASTA path or bytes)."""
    validate_k(k)
    m = default_minimizer_size(k) if m is None else m
    if not 0 < m < k:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k")
    ctx = ctx or default_context()
    data = _bytes(index)
    arr, keep = _inputs_c([data])
    ctx._ck(ctx._lib.mczi_zi_build(ctx.handle, arr[0].data, arr[0].len, k, m))
    del keep
    ctx.k = k
    return ctx


def build_dictionary_from_result(ctx: Context, m: int | None = None) -> Context:
    """Builds the device dictionary from the context's last count (its kept
    k-mers), without moving them off the device."""
    k = ctx.k
    validate_k(k)
    m = default_minimizer_size(k) if m is None else m
    if not 0 < m < k:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k")
    ctx._ck(ctx._lib.mczi_zi_build_from_result(ctx.handle, m))
    return ctx


def query(ctx: Context, queries: Sequence) -> int:
    """Runs the subtraction; the absent set stays on the device as the
    context's result.  Returns its size."""
    data = [_bytes(q) for q in queries]
    arr, keep = _inputs_c(data)
    n = C.c_uint64()
    ctx._ck(ctx._lib.mczi_zi_query(ctx.handle, arr, len(data), C.byref(n)))
    del keep
    return n.value


def collect_query_kmers_absent_from_index(ctx: Context, queries: Sequence) -> Records:
    """Distinct canonical query k-mers absent from the index, sorted."""
    n = query(ctx, queries)
    return ctx.records(n, sorted=True)


def collect_absent_sharded(ctx: Context | None, queries: Sequence, group=None, absent=None):
    """ZI on several GPUs, one process per GPU.  Every rank holds the same
    dictionary (each builds it from the same index: ZI's index is small, so
    it is replicated, not split) and takes a share of every query, cut at
    record boundaries; the ranks' absent sets are gathered and merged at rank
    0, the only collective.  Whether a k-mer is absent does not depend on the
    other queries, so the merged set is the single-GPU result.  Returns the
    sorted distinct (lo, hi) at rank 0 (hi None for k <= 32), None elsewhere.
    `absent(share)` -> (lo, hi) replaces the GPU query (the CPU tests pass a
    stand-in)."""
    import torch.distributed as dist
    from .exchange import split_records
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    share = [s for s in (split_records(_bytes(q), world)[rank] for q in queries) if s.size]
    if absent is None:
        def absent(qs):
            r = collect_query_kmers_absent_from_index(ctx, qs)
            return r.lo, r.hi
    lo, hi = absent(share) if share else (np.empty(0, dtype=np.uint64), None)
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(lo, dtype=np.uint64), hi), group=group)
    if rank != 0:
        return None
    lo = np.concatenate([p[0] for p in parts])
    if all(p[1] is None for p in parts):
        return np.unique(lo), None
    hi = np.concatenate([np.asarray(p[1], dtype=np.uint64) if p[1] is not None else np.zeros(p[0].size, np.uint64)
                         for p in parts])
    u = np.unique(np.stack([hi, lo], axis=1), axis=0)  # sorted by (hi, lo), duplicates removed
    return np.ascontiguousarray(u[:, 1]), np.ascontiguousarray(u[:, 0])


def query_per_input(ctx: Context, queries: Sequence) -> int:
    """One batch of independent requests; returns the number of records."""
    data = [_bytes(q) for q in queries]
    arr, keep = _inputs_c(data)
    n = C.c_uint64()
    ctx._ck(ctx._lib.mczi_zi_query_per_input(ctx.handle, arr, len(data), C.byref(n)))
    del keep
    return n.value


def input_result(ctx: Context, i: int) -> list[int]:
    """Sorted absent canonical k-mers of input `i` of the last per-input batch."""
    n = C.c_uint64()
    ctx._ck(ctx._lib.mczi_zi_input_result(ctx.handle, i, None, None, 0, C.byref(n)))
    lo = np.empty(n.value, dtype=np.uint64)
    hi = np.empty(n.value, dtype=np.uint64)
    if n.value:
        ctx._ck(ctx._lib.mczi_zi_input_result(ctx.handle, i, lo.ctypes.data, hi.ctypes.data, n.value, C.byref(n)))
    return [(int(h) << 64) | int(l) for l, h in zip(lo, hi)]


def batch_results(ctx: Context, n_inputs: int) -> list[np.ndarray]:
    """Every input's absent set from the last per-input batch (unordered, as
    ZI's set), split in one pass by the library.  k <= 32: 1-D uint64 arrays;
    k > 32: (n, 2) arrays of (lo, hi)."""
    total = C.c_uint64()
    offs = np.empty(n_inputs + 1, dtype=np.uint64)
    ctx._ck(ctx._lib.mczi_zi_batch_split(ctx.handle, None, None, offs.ctypes.data, 0, C.byref(total)))
    lo = np.empty(total.value, dtype=np.uint64)
    hi = np.empty(total.value, dtype=np.uint64)
    if total.value:
        ctx._ck(ctx._lib.mczi_zi_batch_split(ctx.handle, lo.ctypes.data, hi.ctypes.data, offs.ctypes.data,
                                             total.value, C.byref(total)))
    o = offs.astype(np.int64)
    if ctx.k <= 32:
        return [lo[o[i]:o[i + 1]] for i in range(n_inputs)]
    return [np.stack([lo[o[i]:o[i + 1]], hi[o[i]:o[i + 1]]], axis=1) for i in range(n_inputs)]


def write_novel_simplitigs(ctx: Context, output_path) -> None:
    """Simplitig FASTA of the last query's absent set (src/zi.rs:177-189)."""
    _write_through(output_path, ctx.write_fasta)


def info(ctx: Context) -> dict:
    buf = (C.c_uint64 * 8)()
    ctx._ck(ctx._lib.mczi_zi_info(ctx.handle, buf, 8))
    keys = ["built", "k", "m", "index_bases", "superkmers", "minimizers", "mphf_levels", "build_us"]
    return {k: int(buf[i]) for i, k in enumerate(keys)}


def subtract(index, queries: Sequence, k: int, m: int | None = None, output=None,
             ctx: Context | None = None) -> Records:
    """ZI's main flow: build, query, write the absent k-mers as simplitigs."""
    ctx = build_dictionary(index, k, m, ctx)
    rec = collect_query_kmers_absent_from_index(ctx, queries)
    if output is not None:
        write_novel_simplitigs(ctx, output)
    return rec
