"""The autotuner's host logic (mczi_gb300/autotune.py) on the CPU, with a
stand-in context: the fastest candidate wins and is left applied, a
candidate that changes the record count is rejected, and the choice is
cached per (GPU, key width, mode, threshold class), a corrupt cache being
ignored.  The GPU counterpart (tests/test_mc_gpu.py) checks that tuning
keeps the oracle's results."""
import json

import pytest


class FakeCtx:
    """Records the knobs applied; a count's time depends on them."""

    def __init__(self, slow_fill=None, wrong=None):
        self.knobs = {}
        self.staged = 0
        self.counts = 0
        self.slow_fill, self.wrong = slow_fill, wrong

    def set_count_tuning(self, threads, slots, ctas_per_sm):
        self.knobs.update(threads=threads, ctas_per_sm=ctas_per_sm)

    def set_count_options(self, chunk, fill):
        self.knobs.update(chunk=chunk, fill=fill)

    def set_count_filter(self, f):
        self.knobs.update(filter=f)

    def set_minimizer_precount(self, on):
        self.knobs.update(precount=bool(on))

    def stage(self, sample):
        self.staged += 1

    def count_staged(self, config, mode=0):
        self.counts += 1
        kn = self.knobs
        if self.wrong is not None and (kn["threads"], kn["fill"]) == self.wrong:
            return 999
        return 1000

    def phase_times(self):
        kn = self.knobs
        # the fastest: 1024 threads x 1 CTA, fill 0.7, chunk 2, filter on, no pre-count
        t = 10.0
        t -= 1.0 if kn["threads"] == 1024 else 0.0
        t -= 0.5 if kn["fill"] == 0.7 else 0.0
        t -= 0.25 if kn["chunk"] == 2 else 0.0
        t -= 0.125 if kn["filter"] == 1 else 0.0
        t += 5.0 if kn["precount"] else 0.0
        return [t, 0.0, 0.0, 0.0]


@pytest.fixture
def cache(tmp_path, monkeypatch):
    p = tmp_path / "tune.json"
    monkeypatch.setenv("MCZI_TUNE_CACHE", str(p))
    return p


def test_candidates():
    from mczi_gb300 import autotune as at
    wide = at.candidates(63, 3)
    assert wide[0] == at.DEFAULT and len(wide) == 1 + 3 * 3 * 2 * 2 + 1
    assert {c.filter for c in wide[1:]} == {0, 1}
    assert {c.filter for c in at.candidates(63, 0)[1:]} == {0}  # x = 0: no filtered rounds
    assert sum(c.precount for c in wide) == 1


def test_fastest_wins_and_is_cached(cache):
    from mczi_gb300 import autotune as at
    from mczi_gb300.mc import CounterConfig
    cfg = CounterConfig(63, 21, 3)
    ctx = FakeCtx()
    best, rep = at.tune(ctx, [b">r\nACGT\n"], cfg)
    assert (best.threads, best.ctas_per_sm, best.fill, best.chunk, best.filter, best.precount) == \
        (1024, 1, 0.7, 2, 1, False)
    assert ctx.knobs == {"threads": 1024, "ctas_per_sm": 1, "chunk": 2, "fill": 0.7, "filter": 1, "precount": False}
    assert rep["cached"] is False and rep["records"] == 1000 and rep["candidates"] == len(at.candidates(63, 3))
    assert rep["best_ms"] < rep["default_ms"]
    saved = json.loads(cache.read_text())
    assert list(saved) == [at.cache_key(63, 0, 3)]
    # a second tune of the same class reads the cache: nothing is staged or counted
    ctx2 = FakeCtx()
    best2, rep2 = at.tune(ctx2, [b">r\nACGT\n"], CounterConfig(45, 21, 7))
    assert rep2["cached"] is True and best2 == best and ctx2.staged == 0 and ctx2.counts == 0
    assert ctx2.knobs == ctx.knobs
    # another class (k <= 32) is tuned afresh
    ctx3 = FakeCtx()
    _, rep3 = at.tune(ctx3, [b">r\nACGT\n"], CounterConfig(31, 21, 3))
    assert rep3["cached"] is False and ctx3.staged == 1


def test_corrupt_cache_is_ignored(cache):
    from mczi_gb300 import autotune as at
    from mczi_gb300.mc import CounterConfig
    cache.write_text("{not json")
    _, rep = at.tune(FakeCtx(), [b">r\n"], CounterConfig(63, 21, 3))
    assert rep["cached"] is False
    assert at.cache_key(63, 0, 3) in json.loads(cache.read_text())


def test_candidate_changing_results_is_rejected(cache):
    from mczi_gb300 import autotune as at
    from mczi_gb300.mc import CounterConfig
    with pytest.raises(RuntimeError, match="changed the result"):
        at.tune(FakeCtx(wrong=(384, 0.6)), [b">r\n"], CounterConfig(63, 21, 3), use_cache=False)
    assert not cache.exists()
