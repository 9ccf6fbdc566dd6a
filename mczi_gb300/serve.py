"""ZI serving loop: continuous batching of subtraction requests on one GPU.

Each worker owns a :class:`~mczi_gb300.mc.Context` (its own CUDA stream and
device buffers) holding the ZI dictionary, built once and kept resident.  A
request is one query FASTA.  Whenever a worker is idle it takes every waiting
request that fits -- at most ``max_batch`` requests and at most its share of
the free HBM, estimated per query byte -- and runs them as ONE batch of
launches (``mczi_zi_query_per_input``); each absent k-mer carries the set of
requests it is absent from, so every request gets exactly the result it gets
alone.  Requests that arrive while batches are running wait only until a
worker frees up, and the batches of different workers overlap on the device
(separate streams; the host threads release the GIL inside the library).

No counterpart exists in the reference (ZI is a one-shot CLI, src/zi.rs:64-101).
"""
from __future__ import annotations

import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field

from . import zi
from .mc import Context

# device bytes needed per query byte during a batch: text, 2-bit stream,
# fragment bits, superkmer descriptors (double-buffered) and keys, absent runs
HBM_BYTES_PER_QUERY_BYTE = 8.0


@dataclass
class Request:
    data: bytes
    arrival: float
    future: Future = field(default_factory=Future)
    started: float = 0.0
    finished: float = 0.0


class ZIServer:
    def __init__(self, index, k: int, m: int | None = None, workers: int = 2, device: int = 0,
                 max_batch: int = 64, hbm_budget: int | None = None, hbm_free_fn=None):
        self.k = k
        self.max_batch = max_batch
        self._q: deque[Request] = deque()
        self._cv = threading.Condition()
        self._stop = False
        self._ctxs = []
        for _ in range(workers):
            ctx = Context(device)
            zi.build_dictionary(index, k, m, ctx=ctx)
            self._ctxs.append(ctx)
        if hbm_budget is None:
            free = hbm_free_fn() if hbm_free_fn else _free_hbm(device)
            hbm_budget = int(0.6 * free)
        self.per_worker_bytes = max(1 << 20, int(hbm_budget / workers / HBM_BYTES_PER_QUERY_BYTE))
        self.batches = 0
        self.batch_sizes: list[int] = []
        self.t_query = 0.0    # seconds inside mczi_zi_query_per_input
        self.t_results = 0.0  # seconds splitting a batch's result per request
        self._threads = [threading.Thread(target=self._run, args=(c,), daemon=True) for c in self._ctxs]
        for t in self._threads:
            t.start()

    # ---- client side
    def submit(self, fasta: bytes) -> Future:
        r = Request(fasta, time.perf_counter())
        with self._cv:
            self._q.append(r)
            self._cv.notify()
        r.future.request = r  # type: ignore[attr-defined]
        return r.future

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        for c in self._ctxs:
            c.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- worker side
    def _take(self) -> list[Request]:
        """Admits waiting requests up to max_batch and this worker's HBM share
        (a request larger than the share runs alone)."""
        batch, size = [], 0
        while self._q and len(batch) < self.max_batch:
            n = len(self._q[0].data)
            if batch and size + n > self.per_worker_bytes:
                break
            batch.append(self._q.popleft())
            size += n
        return batch

    def _run(self, ctx: Context) -> None:
        while True:
            with self._cv:
                while not self._q and not self._stop:
                    self._cv.wait()
                if self._stop and not self._q:
                    return
                batch = self._take()
            t0 = time.perf_counter()
            for r in batch:
                r.started = t0
            try:
                zi.query_per_input(ctx, [r.data for r in batch])
                tq = time.perf_counter()
                results = zi.batch_results(ctx, len(batch))
                t1 = time.perf_counter()
                with self._cv:
                    self.batches += 1
                    self.batch_sizes.append(len(batch))
                    self.t_query += tq - t0
                    self.t_results += t1 - tq
                for r, res in zip(batch, results):
                    r.finished = t1
                    r.future.set_result(res)
            except Exception as e:  # the error reaches every request of the batch
                for r in batch:
                    r.finished = time.perf_counter()
                    r.future.set_exception(e)


def _free_hbm(device: int) -> int:
    try:
        import torch
        free, _ = torch.cuda.mem_get_info(device)
        return int(free)
    except Exception:
        return 8 << 30


def percentile(xs: list[float], p: float) -> float:
    if not xs:
        return float("nan")
    s = sorted(xs)
    i = min(len(s) - 1, max(0, int(round(p / 100.0 * (len(s) - 1)))))
    return s[i]
