"""The Python futures over the native serving loop (mczi_gb300/serve.py),
on the CPU against a fake of the mczi_serve_* entry points: every request
gets its own result, a failed request's error reaches its future, and close
waits for what was submitted."""
import ctypes as C
import queue
import threading

import numpy as np
import pytest

from mczi_gb300 import _native as N


class FakeServeLib:
    """mczi_serve_* semantics: requests finish in submission order on a
    worker thread; a request whose bytes start with b'!' fails."""

    def __init__(self):
        self.done = queue.Queue()
        self.results, self.errors, self.closed = {}, {}, False
        self.next_id = 1
        self.lock = threading.Lock()

    @staticmethod
    def _set(ref, v):
        ref._obj.value = v

    def mczi_serve_open(self, device, index, length, k, m, workers, max_batch, budget, out):
        self._set(out, 1234)
        return N.MCZI_OK

    def mczi_serve_submit(self, h, data, length, rid):
        with self.lock:
            i = self.next_id
            self.next_id += 1
        self._set(rid, i)
        raw = C.string_at(data, length) if length else b""

        def work():
            if raw.startswith(b"!"):
                self.errors[i] = b"request rejected"
            else:  # the "absent set": the request's distinct bytes
                self.results[i] = np.unique(np.frombuffer(raw, dtype=np.uint8)).astype(np.uint64)
            self.done.put(i)
        threading.Thread(target=work).start()
        return N.MCZI_OK

    def mczi_serve_next(self, h, timeout_ms, rid, st, n, lat, wait):
        try:
            i = self.done.get(timeout=timeout_ms / 1000.0)
        except queue.Empty:
            return N.MCZI_ERR_TIMEOUT
        self._set(rid, i)
        self._set(st, N.MCZI_ERR_DEVICE if i in self.errors else N.MCZI_OK)
        self._set(n, len(self.results.get(i, [])))
        self._set(lat, 2.0)
        self._set(wait, 1.0)
        return N.MCZI_OK

    def mczi_serve_result(self, h, i, lo, hi, cap, n):
        if i in self.errors:
            return N.MCZI_ERR_DEVICE
        r = self.results.pop(i)
        if len(r):
            C.memmove(lo, r.ctypes.data, r.nbytes)
        return N.MCZI_OK

    def mczi_serve_release(self, h, i):
        self.results.pop(i, None)
        return N.MCZI_ERR_DEVICE if i in self.errors else N.MCZI_OK

    def mczi_serve_error(self, h, i):
        return self.errors.get(i, b"")

    def mczi_serve_stats(self, h, out, cap):
        return 0

    def mczi_serve_close(self, h):
        self.closed = True
        return N.MCZI_OK


def test_futures_results_errors_and_close(monkeypatch):
    fake = FakeServeLib()
    monkeypatch.setattr(N, "load", lambda required=True: fake)
    from mczi_gb300.serve import ZIServer
    srv = ZIServer(b">i\nACGTACGT\n", 5, 3, workers=1)
    reqs = [bytes([65 + (i % 7)]) * (i + 1) + b"xyz" for i in range(40)]
    futs = [srv.submit(r) for r in reqs]
    bad = srv.submit(b"!broken")
    for r, f in zip(reqs, futs):
        assert list(f.result(timeout=10)) == sorted(set(r))
        assert f.latency_ms == 2.0 and f.queue_ms == 1.0
    with pytest.raises(N.MCZIError, match="request rejected"):
        bad.result(timeout=10)
    late = srv.submit(b"late")  # still answered: close waits for it
    srv.close()
    assert fake.closed and late.done() and list(late.result()) == sorted(set(b"late"))
    assert not srv._pending


def test_sizes_only_client(monkeypatch):
    """keep_results=False: futures give the absent-set size and the requests
    are released without copying their k-mers."""
    fake = FakeServeLib()
    monkeypatch.setattr(N, "load", lambda required=True: fake)
    from mczi_gb300.serve import ZIServer
    with ZIServer(b">i\nACGTACGT\n", 5, 3, workers=1, keep_results=False) as srv:
        reqs = [bytes([65 + (i % 5)]) * (i + 1) + b"q" for i in range(20)]
        futs = [srv.submit(r) for r in reqs]
        assert [f.result(timeout=10) for f in futs] == [len(set(r)) for r in reqs]
    assert not fake.results
