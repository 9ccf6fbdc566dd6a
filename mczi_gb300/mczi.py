"""MCZI orchestration on one GPU: MC indexing and ZI subtraction in one process.

Follows the reference's MCZI run (src/mczi.rs:238-454): the index inputs are
counted by MC with (k, m, x); the kept canonical k-mers become the
dictionary's sequences on the device, each k-mer its own sequence
(``mczi_zi_build_from_result``; the reference writes MC's k-mer set to FASTA
and compacts it before its SSHash build: the k-mer set is the same); the
query inputs are subtracted; the absent
k-mers are written as simplitig FASTA, one file for all queries or, with
``query_fofn``, one per query file named ``<stem>.<suffix><ext>`` beside it or
in the output folder (src/mczi.rs:770-871).  The index stays on the device
between the two steps.  Out of scope (kept on the CPU by the reference):
GGCAT compaction of the output (the absent k-mer set is the same; only its
tiling into simplitigs differs), the R reformer and the "regular" output mode.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

from . import _native as N
from . import mc, zi


def _ensure(cond: bool, msg: str) -> None:
    if not cond:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, msg)


def normalized_output_suffix(output_suffix: str) -> str:
    s = output_suffix.strip()
    s = s[1:] if s.startswith(".") else s
    _ensure(bool(s), "--output-suffix must not be empty")
    _ensure(os.sep not in s, "--output-suffix must be a filename suffix, not a path")
    return s


def _split_known_suffix(name: str, suffixes: Sequence[str]) -> tuple[str, str] | None:
    for suf in suffixes:
        if len(name) > len(suf) and name[-len(suf):].lower() == suf:
            return name[:-len(suf)], name[-len(suf):]
    return None


def suffixed_query_file_name(file_name: str, suffix: str) -> str:
    """reads.fq.gz -> reads.<suffix>.fq.gz"""
    base, comp = _split_known_suffix(file_name, [".zstd", ".gzip", ".zst", ".gz", ".xz"]) or (file_name, "")
    stem, seq_ext = _split_known_suffix(base, [".fasta", ".fastq", ".fna", ".fa", ".fq"]) or (base, "")
    return f"{stem}.{suffix}{seq_ext}{comp}"


@dataclass
class Job:
    inputs: list[Path]
    output: Path | None


def query_output_plan(query_fofn: bool, query_inputs: Sequence[Path], output: Path | None,
                      output_suffix: str) -> list[Job]:
    if not query_fofn:
        _ensure(output is not None, "--output is required unless --query-fofn is set")
        return [Job(list(query_inputs), output)]
    if output is not None and str(output) == "/dev/null":
        return [Job(list(query_inputs), output)]
    suffix = normalized_output_suffix(output_suffix)
    if output is not None:
        if output.exists():
            _ensure(output.is_dir(), "--output must be a directory in --query-fofn mode")
        else:
            output.mkdir(parents=True)
    jobs, seen = [], set()
    for q in query_inputs:
        q = Path(q)
        _ensure(bool(q.name), f"query input {q} has no filename")
        out = (output if output is not None else (q.parent if str(q.parent) else Path("."))) / \
            suffixed_query_file_name(q.name, suffix)
        _ensure(out != q, f"output path {out} would overwrite query input {q}; choose a non-empty --output-suffix")
        _ensure(out not in seen, f"multiple query inputs map to the same output path {out}; "
                                 "use --output or --output-suffix to disambiguate")
        seen.add(out)
        jobs.append(Job([q], out))
    return jobs


def run(index_inputs: Sequence, query_inputs: Sequence, k: int, m: int, x: int = 1, output=None,
        query_fofn: bool = False, output_suffix: str = "filtered", output_mode: str = "simplitig",
        partition_count: int = mc.DEFAULT_PARTITION_COUNT, ctx: mc.Context | None = None) -> dict:
    """Returns {"index_kmers": n, "absent": [n per output job]}."""
    zi.validate_k(k)
    _ensure(0 < m < k, "minimizer size must be > 0 and < k")
    _ensure(output_mode in ("simplitig", "no-output"),
            f"--output-mode {output_mode} is not supported (simplitig or no-output)")
    _ensure(output_mode != "no-output" or output is None, "--output is not used with --output-mode no-output")
    _ensure(output_mode == "no-output" or query_fofn or output is not None,
            "--output is required unless --query-fofn or --output-mode no-output is set")
    _ensure(len(index_inputs) > 0, "at least one index input is required")
    _ensure(len(query_inputs) > 0, "at least one query input is required")
    output = Path(output) if output is not None else None
    jobs = [Job(list(query_inputs), None)] if output_mode == "no-output" else \
        query_output_plan(query_fofn, [Path(q) for q in query_inputs], output, output_suffix)
    ctx = ctx or mc.default_context()
    # 1. MC on the index set
    cfg = mc.CounterConfig(k, m, x, partition_count)
    ctx.validate(cfg)
    data = [mc.read_input(p) if not isinstance(p, (bytes, bytearray, memoryview)) else p for p in index_inputs]
    n_index = ctx.count(data, cfg)
    # 2. the kept k-mers -> the dictionary, built where they are (on the device)
    if n_index == 0:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "index FASTA did not contain any sequence of length >= k")
    zi.build_dictionary_from_result(ctx, m)
    # 3. the subtraction, per output job
    absent = []
    for job in jobs:
        n = zi.query(ctx, [mc.read_input(q) if not isinstance(q, (bytes, bytearray, memoryview)) else q
                           for q in job.inputs])
        absent.append(n)
        if job.output is not None:
            zi.write_novel_simplitigs(ctx, job.output)
    return {"index_kmers": n_index, "absent": absent}
