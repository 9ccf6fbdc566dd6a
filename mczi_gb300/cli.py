"""Command lines of MC and ZI over the GPU library.

``python -m mczi_gb300.cli mc|zi|mczi ...`` take the flags of the reference's
binaries (MC: src/main.rs:10-101, ZI: src/zi.rs:13-101, MCZI:
src/mczi.rs:140-230) with the same defaults and validation messages, and run
the same library entry points (count_inputs_to_{kff,fasta}_path,
count_datasets_to_{kff,fasta}_path; build_dictionary,
collect_query_kmers_absent_from_index, write_novel_simplitigs; mczi.run).  Errors print
as ``Error: <message>`` with exit status 1.  ``--threads`` is accepted and
validated; the device work does not use host threads, and ZI's
``--ram-limit-gib`` only bounded the reference's external-memory build.
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

from . import _native as N
from . import mc, zi


def _mc_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="MC", description="Parallel two-pass pseudo k-mer counter using minimizer "
                                                        "pre-counting (GB300)")
    ap.add_argument("-i", "--input", nargs="+", required=True, type=Path,
                    help="Input FASTA/FASTQ file(s), optionally gzip, xz or zstd compressed")
    ap.add_argument("--fofn", action="store_true",
                    help="Treat --input path(s) as file-of-filenames; -x is a dataset-presence threshold")
    ap.add_argument("-k", "--kmer-size", type=int, required=True, help="K-mer size; must be <= 64")
    ap.add_argument("-m", "--minimizer-size", type=int, required=True, help="Minimizer size; must be <= k")
    ap.add_argument("-x", "--threshold", type=int, default=1, help="Emit k-mers seen more than this many times")
    ap.add_argument("-o", "--output", type=Path, required=True,
                    help="Output FASTA or KFF file; .gz and .xz are compressed")
    ap.add_argument("--format", choices=["fasta", "kff"], default="fasta", help="Output format")
    ap.add_argument("-t", "--threads", type=int, default=None, help="Host worker threads (validated only)")
    ap.add_argument("--partition-count", type=int, default=mc.DEFAULT_PARTITION_COUNT,
                    help="Partition count of the reference's temporary files (validated only)")
    return ap


def _zi_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="ZI", description="Subtract an SSHash-style indexed k-mer set from FASTA/FOFN "
                                                        "FASTA input (GB300)")
    ap.add_argument("--index", type=Path, required=True,
                    help="FASTA containing k-mers/simplitigs to index and subtract; gzip, xz and zstd accepted")
    ap.add_argument("-i", "--input", nargs="+", required=True, type=Path,
                    help="Query FASTA file(s), or FOFN path(s) when --fofn is set")
    ap.add_argument("--fofn", action="store_true", help="Treat --input path(s) as file-of-filenames")
    ap.add_argument("-k", "--kmer-size", type=int, required=True, help="K-mer size; must be odd and in [3, 63]")
    ap.add_argument("-m", "--minimizer-size", type=int, default=None,
                    help="Minimizer size; defaults to 19, adjusted below k")
    ap.add_argument("-o", "--output", type=Path, required=True,
                    help="Output FASTA of the query k-mers absent from the index; .gz and .xz are compressed")
    ap.add_argument("-t", "--threads", type=int, default=0, help="Build threads (validated only)")
    ap.add_argument("--ram-limit-gib", type=int, default=8, help="Build RAM limit of the reference (unused)")
    return ap


def _mczi_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="MCZI", description="Run MC indexing and ZI subtraction in one process (GB300)")
    ap.add_argument("--index-input", nargs="+", required=True, type=Path,
                    help="MC index-set input FASTA/FASTQ file(s), or FOFN path(s) with --index-fofn")
    ap.add_argument("--index-fofn", action="store_true", help="Treat --index-input path(s) as MC file-of-filenames")
    ap.add_argument("--query-input", nargs="+", required=True, type=Path,
                    help="Query FASTA/FASTQ file(s), or FOFN path(s) with --query-fofn")
    ap.add_argument("--query-fofn", action="store_true", help="Treat --query-input path(s) as file-of-filenames")
    ap.add_argument("-k", "--kmer-size", type=int, required=True, help="K-mer size; must be odd and in [3, 63]")
    ap.add_argument("-m", "--minimizer-size", type=int, required=True, help="MC minimizer size; also used for the index")
    ap.add_argument("-x", "--threshold", type=int, default=1, help="MC threshold for the index set")
    ap.add_argument("-o", "--output", type=Path, default=None,
                    help="Output FASTA path (a folder in --query-fofn mode)")
    ap.add_argument("--output-suffix", default="filtered", help="Suffix of each output name in --query-fofn mode")
    ap.add_argument("--output-mode", default="simplitig", help="simplitig or no-output")
    ap.add_argument("--reform-output", action="store_true", help="R-style reforming (not available here)")
    ap.add_argument("-t", "--threads", type=int, default=None, help="Host worker threads (validated only)")
    ap.add_argument("--partition-count", type=int, default=mc.DEFAULT_PARTITION_COUNT)
    ap.add_argument("--ram-limit-gib", type=int, default=8, help="Build RAM limit of the reference (unused)")
    return ap


def mczi_main(argv: list[str]) -> None:
    from . import mczi
    a = _mczi_parser().parse_args(argv)
    if a.reform_output:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "--reform-output (the R unitig reformer) is not part of this library")
    if a.threads is not None and a.threads <= 0:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "--threads must be greater than 0")
    index_inputs = mc.expand_fofns(a.index_input) if a.index_fofn else list(a.index_input)
    query_inputs = mc.expand_fofns(a.query_input) if a.query_fofn else list(a.query_input)
    started = time.perf_counter()
    stats = mczi.run(index_inputs, query_inputs, a.kmer_size, a.minimizer_size, a.threshold, a.output,
                     a.query_fofn, a.output_suffix, a.output_mode, a.partition_count)
    print(f"MCZI_STAT\tindex_kmers\t{stats['index_kmers']}\tabsent_kmers\t{sum(stats['absent'])}", file=sys.stderr)
    _phase("total", started)


def _phase(name: str, t0: float) -> None:
    print(f"ZI_PHASE\t{name}\t{time.perf_counter() - t0:.6f}s", file=sys.stderr)


def mc_main(argv: list[str]) -> None:
    a = _mc_parser().parse_args(argv)
    if a.threads is not None and a.threads <= 0:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "--threads must be greater than 0")
    cfg = mc.CounterConfig(a.kmer_size, a.minimizer_size, a.threshold, a.partition_count)
    if a.fofn:
        datasets = mc.expand_fofns(a.input)
        run = mc.count_datasets_to_kff_path if a.format == "kff" else mc.count_datasets_to_fasta_path
        run(datasets, cfg, a.output)
    else:
        run = mc.count_inputs_to_kff_path if a.format == "kff" else mc.count_inputs_to_fasta_path
        run(list(a.input), cfg, a.output)


def zi_main(argv: list[str]) -> None:
    a = _zi_parser().parse_args(argv)
    k = a.kmer_size
    zi.validate_k(k)
    m = a.minimizer_size if a.minimizer_size is not None else zi.default_minimizer_size(k)
    if not (0 < m < k):
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k")
    queries = mc.expand_fofns(a.input) if a.fofn else list(a.input)
    if not queries:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "at least one query FASTA is required")
    started = time.perf_counter()
    ctx = zi.build_dictionary(mc.read_input(a.index), k, m)
    _phase("1_index", started)
    t = time.perf_counter()
    zi.query(ctx, [mc.read_input(q) for q in queries])
    _phase("2_query_subtraction", t)
    t = time.perf_counter()
    zi.write_novel_simplitigs(ctx, a.output)
    _phase("3_simplitig_output", t)
    _phase("total", started)


def main(argv: list[str] | None = None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    mains = {"mc": mc_main, "zi": zi_main, "mczi": mczi_main}
    if not argv or argv[0] not in mains:
        print("usage: python -m mczi_gb300.cli {mc,zi,mczi} [flags of the MC / ZI / MCZI binaries]", file=sys.stderr)
        return 2
    try:
        mains[argv[0]](argv[1:])
    except N.MCZIError as e:
        print(f"Error: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
