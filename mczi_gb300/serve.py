"""ZI serving: continuous batching of subtraction requests on one GPU.

The loop itself is native (``mczi_serve_*`` in ``include/mczi_gpu.h``,
``csrc/serve.cpp``): worker threads in the library each own a context (its
own CUDA stream and device buffers) holding the ZI dictionary, built once and
kept resident.  A request is one query FASTA.  Whenever a worker is idle it
takes every waiting request that fits -- at most ``max_batch`` requests and at
most its share of the free HBM, estimated per query byte -- and runs them as
ONE batch of launches (``mczi_zi_query_per_input``); each absent k-mer carries
the set of requests it is absent from, so every request gets exactly the
result it gets alone.  Batches of different workers overlap on the device.

This module wraps the native server in futures: ``submit`` returns a
``concurrent.futures.Future`` whose result is the request's absent set (k <=
32: a uint64 array; k > 32: an (n, 2) array of (lo, hi)), or only its size
with ``keep_results=False``; the future carries ``latency_ms`` and
``queue_ms`` once done.

No counterpart exists in the reference (ZI is a one-shot CLI, src/zi.rs:64-101).
"""
from __future__ import annotations

import ctypes as C
import threading
from concurrent.futures import Future

import numpy as np

from . import _native as N
from . import zi
from .mc import _as_bytes


class ZIServer:
    def __init__(self, index, k: int, m: int | None = None, workers: int = 2, device: int = 0,
                 max_batch: int = 64, hbm_budget: int | None = None, hbm_free_fn=None, keep_results: bool = True):
        zi.validate_k(k)
        m = zi.default_minimizer_size(k) if m is None else m
        if not 0 < m < k:
            raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k")
        self.k = k
        # keep_results=False: futures give only the absent-set size and the
        # native server releases each request without copying its k-mers
        self.keep_results = keep_results
        self._lib = N.load()
        if hbm_budget is None:
            hbm_budget = int(0.6 * hbm_free_fn()) if hbm_free_fn else 0  # 0: the library asks the device
        idx = _as_bytes(zi._bytes(index))
        buf = (C.c_uint8 * len(idx)).from_buffer_copy(idx) if len(idx) else None
        h = C.c_void_p()
        rc = self._lib.mczi_serve_open(device, buf, len(idx), k, m, workers, max_batch, int(hbm_budget), C.byref(h))
        if rc < 0:
            msg = self._lib.mczi_serve_error(None, 0)
            raise N.MCZIError(rc, msg.decode() if msg else "mczi_serve_open failed")
        self._h = h
        self._lock = threading.Lock()
        self._pending: dict[int, tuple[Future, object]] = {}
        self._stop = False
        self._poller = threading.Thread(target=self._poll, daemon=True)
        self._poller.start()

    # ---- client side
    def submit(self, fasta) -> Future:
        data = np.frombuffer(_as_bytes(fasta), dtype=np.uint8) if not isinstance(fasta, np.ndarray) else \
            np.ascontiguousarray(fasta).view(np.uint8).reshape(-1)
        fut: Future = Future()
        rid = C.c_uint64()
        with self._lock:  # the poller looks the future up under this lock
            rc = self._lib.mczi_serve_submit(self._h, data.ctypes.data if data.size else None, data.size,
                                             C.byref(rid))
            if rc < 0:
                raise N.MCZIError(rc, "the server is closed")
            self._pending[rid.value] = (fut, data)  # the bytes stay alive until answered
        return fut

    def stats(self) -> dict:
        out = (C.c_double * 7)()
        n = self._lib.mczi_serve_stats(self._h, out, 7)
        keys = ["batches", "requests", "largest_batch", "query_s", "results_s", "waiting", "worker_bytes"]
        return {keys[i]: out[i] for i in range(n)}

    @property
    def batches(self) -> int:
        return int(self.stats()["batches"])

    def close(self) -> None:
        if self._h is None:
            return
        with self._lock:
            futs = [f for f, _ in self._pending.values()]
        for f in futs:  # the workers answer everything queued
            try:
                f.result()
            except Exception:
                pass
        self._stop = True
        self._poller.join()
        self._lib.mczi_serve_close(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- completions
    def _poll(self) -> None:
        rid, st, n = C.c_uint64(), C.c_int32(), C.c_uint64()
        lat, wait = C.c_double(), C.c_double()
        while not self._stop:
            rc = self._lib.mczi_serve_next(self._h, 50, C.byref(rid), C.byref(st), C.byref(n), C.byref(lat),
                                           C.byref(wait))
            if rc == N.MCZI_ERR_TIMEOUT:
                continue
            with self._lock:
                fut, _ = self._pending.pop(rid.value)
            fut.latency_ms = lat.value  # type: ignore[attr-defined]
            fut.queue_ms = wait.value  # type: ignore[attr-defined]
            if st.value < 0:
                msg = self._lib.mczi_serve_error(self._h, rid.value)
                err = N.MCZIError(st.value, msg.decode() if msg else "")
                self._lib.mczi_serve_result(self._h, rid.value, _EMPTY.ctypes.data, None, 0, None)  # release
                fut.set_exception(err)
                continue
            if not self.keep_results:
                self._lib.mczi_serve_release(self._h, rid.value)
                fut.set_result(int(n.value))
                continue
            lo = np.empty(n.value, dtype=np.uint64)
            hi = np.empty(n.value, dtype=np.uint64) if self.k > 32 else None
            # a non-NULL key_lo copies and releases the request, an empty one too
            self._lib.mczi_serve_result(self._h, rid.value, lo.ctypes.data if n.value else _EMPTY.ctypes.data,
                                        hi.ctypes.data if (hi is not None and n.value) else None, n.value,
                                        C.byref(n))
            fut.set_result(lo if hi is None else np.stack([lo, hi], axis=1))


_EMPTY = np.empty(1, dtype=np.uint64)


def percentile(xs: list[float], p: float) -> float:
    if not xs:
        return float("nan")
    s = sorted(xs)
    i = min(len(s) - 1, max(0, int(round(p / 100.0 * (len(s) - 1)))))
    return s[i]
