"""Autotuner for the counting pipeline's runtime knobs.

Results never depend on these knobs (the kernels split overfull rounds and
every configuration counts the same canonical k-mers), so tuning is a pure
speed search: each candidate runs on a sample of the caller's workload, its
record count must equal the first candidate's (a cheap invariance check), and
the fastest device time wins.  The choice is cached per (GPU name, key width,
mode, threshold class) in ``~/.cache/mczi_gb300/tune.json`` (override with
MCZI_TUNE_CACHE).

Knobs: threads per counting CTA and CTAs per SM (block size and table size
follow), target table fill, windows per work item, two-pass filtered rounds,
and the pass-1 minimizer pre-count.  The pack tile (8 KiB), the scan tile
(4096 windows) and the partition digits (12 + 11 bits) size shared-memory
arrays and unrolled loops, so they are compile-time constants; builds with
other tiles measured no faster on GB300 (4 Gbp, k = 63: scan 12.04 ms at 4096
windows, 12.84 at 2048; pack 7.41 ms at 8 KiB, 7.30 at 4 KiB, 7.92 at 16 KiB;
identical results).
"""
from __future__ import annotations

import itertools
import json
import os
from dataclasses import asdict, dataclass
from pathlib import Path

from .mc import Context, CounterConfig


@dataclass(frozen=True)
class Tuning:
    threads: int = 0
    ctas_per_sm: int = 0
    fill: float = 0.0
    chunk: int = 0
    filter: int = -1
    precount: bool = False

    def apply(self, ctx: Context) -> None:
        ctx.set_count_tuning(self.threads, 0, self.ctas_per_sm)
        ctx.set_count_options(self.chunk, self.fill)
        ctx.set_count_filter(self.filter)
        ctx.set_minimizer_precount(self.precount)


DEFAULT = Tuning()


def _cache_path() -> Path:
    p = os.environ.get("MCZI_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "mczi_gb300" / "tune.json"


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown-gpu"


def cache_key(k: int, mode: int, threshold: int) -> str:
    return f"{_gpu_name()}|k{'64' if k <= 32 else '128'}|mode{mode}|x{'0' if threshold == 0 else 'ge1'}"


def candidates(k: int, threshold: int) -> list[Tuning]:
    wide = k > 32
    shapes = [(512, 2), (1024, 1), (384, 2)] if wide else [(512, 2), (1024, 1), (256, 4)]
    fills = [0.8, 0.7, 0.6]
    chunks = [4, 2] if wide else [2, 4]
    filters = [1, 0] if threshold >= 1 else [0]
    out = [DEFAULT]
    for (t, c), f, ch, fl in itertools.product(shapes, fills, chunks, filters):
        out.append(Tuning(t, c, f, ch, fl, False))
    out.append(Tuning(shapes[0][0], shapes[0][1], fills[0], chunks[0], filters[0], True))
    return out


def tune(ctx: Context, sample: list, config: CounterConfig, mode: int = 0, repeats: int = 2,
         use_cache: bool = True) -> tuple[Tuning, dict]:
    """Times every candidate on `sample` (FASTA inputs) and applies the best.
    Returns (best, report)."""
    key = cache_key(config.k, mode, config.threshold)
    path = _cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            best = Tuning(**cache[key]["tuning"])
            best.apply(ctx)
            return best, {"cached": True, **cache[key]}
    ctx.stage(sample)
    ref = None
    results = []
    for cand in candidates(config.k, config.threshold):
        cand.apply(ctx)
        times = []
        for _ in range(repeats + 1):
            n = ctx.count_staged(config, mode)
            times.append(sum(ctx.phase_times()))
        if ref is None:
            ref = n
        if n != ref:
            raise RuntimeError(f"tuning candidate {cand} changed the result ({n} != {ref} records)")
        results.append((min(times[1:]), cand))
    results.sort(key=lambda r: r[0])
    best_ms, best = results[0]
    best.apply(ctx)
    report = {"tuning": asdict(best), "best_ms": round(best_ms, 4),
              "default_ms": round(next(t for t, c in results if c == DEFAULT), 4),
              "candidates": len(results), "records": ref, "cached": False}
    if use_cache:
        cache[key] = {k: v for k, v in report.items() if k != "cached"}
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best, report
