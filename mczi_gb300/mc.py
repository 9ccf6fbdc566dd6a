"""MC on the GPU: the k-mer counting entry points of the reference library.

Names, argument meaning, validation messages and result order follow the MC
library (``src/lib.rs``): ``CounterConfig`` (:48-53), ``CountedKmer`` (:63-66),
``count_inputs`` (:278, sorted by encoded k-mer), ``count_datasets`` (:289),
``count_inputs_to_kff_path`` (:457), ``count_inputs_to_fasta_path`` (:427),
``count_datasets_to_kff_path`` (:509), ``count_datasets_to_fasta_path``
(:442), ``count_inputs_to_kmer_fasta_path`` (:306),
``count_datasets_to_kmer_fasta_path`` (:357), ``expand_fofns`` (:242-276),
``decode_kmer`` (:3056-3069).

All counting runs in ``libmczi_gpu.so`` on the GPU; this module only moves
bytes and records across the C ABI.  Input files given by path are read with
the library's readers (``read_input``): plain, gzip, xz or zstd, decoded on
host threads, as MC's readers decode them.  Compressed bytes handed to
``Context.count`` directly, and the C ABI's path entry points, decode BGZF
gzip on the device instead (``Context.inflate_gzip`` decodes such a buffer
alone).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Iterable, Sequence

import numpy as np

from . import _native as N

DEFAULT_PARTITION_COUNT = 1024


@dataclass(frozen=True)
class CounterConfig:
    k: int
    minimizer: int
    threshold: int = 1
    partition_count: int = DEFAULT_PARTITION_COUNT

    def c(self) -> N.CounterConfigC:
        if min(self.k, self.minimizer, self.threshold, self.partition_count) < 0:
            raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "negative configuration value")
        return N.CounterConfigC(self.k, self.minimizer, self.threshold, self.partition_count)


@dataclass(frozen=True, order=True)
class CountedKmer:
    encoded: int
    count: int


class Records:
    """Kept (canonical k-mer, count) records of one run, as numpy arrays."""

    def __init__(self, lo: np.ndarray, hi: np.ndarray | None, count: np.ndarray, k: int):
        self.lo, self.hi, self.count, self.k = lo, hi, count, k

    def __len__(self) -> int:
        return int(self.lo.shape[0])

    def encoded(self) -> list[int]:
        if self.hi is None:
            return [int(v) for v in self.lo]
        return [(int(h) << 64) | int(l) for h, l in zip(self.hi, self.lo)]

    def counted(self) -> list[CountedKmer]:
        return [CountedKmer(e, int(c)) for e, c in zip(self.encoded(), self.count)]


def _as_bytes(x) -> memoryview:
    if isinstance(x, (bytes, bytearray)):
        return memoryview(x)
    if isinstance(x, memoryview):
        return x
    if isinstance(x, np.ndarray):
        return memoryview(np.ascontiguousarray(x).view(np.uint8).reshape(-1))
    raise TypeError(f"unsupported input type {type(x)!r}")


def _inputs_c(inputs: Sequence) -> tuple[C.Array, list]:
    keep = []
    arr = (N.InputC * len(inputs))()
    for i, x in enumerate(inputs):
        if isinstance(x, tuple):  # (address, length) of caller-owned memory, e.g. pinned
            arr[i].data = int(x[0]) if x[1] else None
            arr[i].len = int(x[1])
            continue
        if isinstance(x, np.ndarray):
            a = np.ascontiguousarray(x).view(np.uint8).reshape(-1)
            keep.append(a)
            arr[i].data = a.ctypes.data if a.size else None
            arr[i].len = a.size
        else:
            mv = _as_bytes(x)
            if mv.nbytes == 0:
                arr[i].data = None
                arr[i].len = 0
                continue
            buf = (C.c_char * mv.nbytes).from_buffer_copy(mv) if mv.readonly else (C.c_char * mv.nbytes).from_buffer(mv)
            keep.append(buf)
            arr[i].data = C.addressof(buf)
            arr[i].len = mv.nbytes
    return arr, keep


class Context:
    """One ``mczi_ctx``: a CUDA device, a stream and the device buffers."""

    def __init__(self, device: int = 0):
        self._lib = N.load()
        h = C.c_void_p()
        rc = self._lib.mczi_open(device, C.byref(h))
        if rc != 0:
            raise N.MCZIError(rc, f"cannot open CUDA device {device} (no CPU fallback)")
        self._h = h
        self.device = device
        self.k = 0

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            self._lib.mczi_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc: int) -> int:
        return N.check(self._h, rc)

    def set_stream(self, stream_ptr: int | None) -> None:
        self._ck(self._lib.mczi_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def validate(self, config: CounterConfig, mode: int = N.MODE_ABUNDANCE) -> None:
        cc = config.c()
        self._ck(self._lib.mczi_validate_config(self._h, C.byref(cc), mode))

    def count(self, inputs: Sequence, config: CounterConfig, mode: int = N.MODE_ABUNDANCE) -> int:
        arr, keep = _inputs_c(inputs)
        cc = config.c()
        n = C.c_uint64()
        self._ck(self._lib.mczi_count(self._h, C.byref(cc), mode, arr, len(inputs), C.byref(n)))
        del keep
        self.k = config.k
        return n.value

    def stage(self, inputs: Sequence) -> None:
        arr, keep = _inputs_c(inputs)
        self._ck(self._lib.mczi_stage(self._h, arr, len(inputs)))
        del keep

    def count_staged(self, config: CounterConfig, mode: int = N.MODE_ABUNDANCE) -> int:
        cc = config.c()
        n = C.c_uint64()
        self._ck(self._lib.mczi_count_staged(self._h, C.byref(cc), mode, C.byref(n)))
        self.k = config.k
        return n.value

    def records(self, n: int | None = None, sorted: bool = True, out=None) -> Records:
        """The last result's records.  sorted=False keeps the kernels' emission
        order and copies straight from the device into the arrays; `out` =
        (lo, hi, counts) uint64 arrays of >= n entries (e.g. views of pinned
        host memory, reused across calls; hi may be None for k <= 32)."""
        if n is None:
            st = self.run_stats()
            n = int(st[5])
        if out is not None:
            lo, hi, cnt = out
            lo, cnt = lo[:n], cnt[:n]
            hi = hi[:n] if (hi is not None and self.k > 32) else None
        else:
            lo = np.empty(n, dtype=np.uint64)
            cnt = np.empty(n, dtype=np.uint64)
            hi = np.empty(n, dtype=np.uint64) if self.k > 32 else None
        self._ck(self._lib.mczi_result_copy(self._h, lo.ctypes.data if n else None,
                                            hi.ctypes.data if (hi is not None and n) else None,
                                            cnt.ctypes.data if n else None, n, 1 if sorted else 0))
        return Records(lo, hi, cnt, self.k)

    def digest(self, unit_counts: bool = False) -> dict:
        """Order-independent digest of the last result, computed on the device
        (the definition of mczi_gb300.digest.records_digest; unit_counts
        digests every count as 1, for ZI absent sets)."""
        out = (C.c_uint64 * 4)()
        self._ck(self._lib.mczi_result_digest(self._h, 1 if unit_counts else 0, out))
        return {"records": int(out[0]), "count_sum": int(out[1]), "sum": "%016x" % out[2], "xor": "%016x" % out[3]}

    def write_kff(self, path: str | os.PathLike) -> None:
        self._ck(self._lib.mczi_result_write_kff(self._h, os.fsencode(str(path))))

    def write_fasta(self, path: str | os.PathLike) -> None:
        self._ck(self._lib.mczi_result_write_fasta(self._h, os.fsencode(str(path))))

    def inflate_gzip(self, gz) -> bytes:
        """Decodes a gzip buffer whose members carry their sizes (BGZF, see
        mczi_gb300.bgzf) on the device; phase_times()[5] is the decode time."""
        mv = _as_bytes(gz)
        src = (C.c_char * mv.nbytes).from_buffer_copy(mv) if mv.nbytes else None
        n = C.c_uint64()
        rc = self._lib.mczi_inflate_gzip(self._h, src, mv.nbytes, None, 0, C.byref(n))
        if rc not in (0, N.MCZI_ERR_TOO_LARGE):
            self._ck(rc)
        out = np.empty(max(1, n.value), dtype=np.uint8)
        self._ck(self._lib.mczi_inflate_gzip(self._h, src, mv.nbytes, out.ctypes.data, n.value, C.byref(n)))
        return out[: n.value].tobytes()

    def phase_times(self) -> list[float]:
        buf = (C.c_float * 8)()
        n = self._ck(self._lib.mczi_phase_times(self._h, buf, 8))
        return [float(buf[i]) for i in range(n)]

    def run_stats(self) -> list[int]:
        buf = (C.c_uint64 * 10)()
        n = self._ck(self._lib.mczi_run_stats(self._h, buf, 10))
        return [int(buf[i]) for i in range(n)]

    def set_count_tuning(self, threads: int, table_slots: int = 0, ctas_per_sm: int = 2) -> None:
        self._ck(self._lib.mczi_set_count_tuning(self._h, threads, table_slots, ctas_per_sm))

    def set_count_options(self, chunk: int = 0, fill: float = 0.0) -> None:
        self._ck(self._lib.mczi_set_count_options(self._h, chunk, fill))

    def set_count_filter(self, mode: int) -> None:
        """-1 auto (two-pass rounds when threshold >= 1), 0 single pass, 1 two-pass."""
        self._ck(self._lib.mczi_set_count_filter(self._h, mode))

    def set_graph_replay(self, enable: bool) -> None:
        """Replay the counting pipeline from a captured CUDA graph."""
        self._ck(self._lib.mczi_set_graph_replay(self._h, 1 if enable else 0))

    def set_key_range_passes(self, passes: int) -> None:
        """0 = automatic; n forces n passes over disjoint minimizer-key ranges."""
        self._ck(self._lib.mczi_set_key_range_passes(self._h, passes))

    def set_streamed_staging(self, enable: bool = True, segment_bytes: int = 0) -> None:
        """count() copies its inputs in segments overlapped with pack + scan
        (default on; segment_bytes a multiple of 8192, 0 = automatic)."""
        self._ck(self._lib.mczi_set_streamed_staging(self._h, 1 if enable else 0, segment_bytes))

    def set_zi_bucket_records(self, records: int = 0) -> None:
        """Records per final bucket of the ZI deduplication (0 = automatic,
        half a shared-memory table); smaller values only add partition work."""
        self._ck(self._lib.mczi_set_zi_bucket_records(self._h, records))

    def set_minimizer_precount(self, enable: bool) -> None:
        self._ck(self._lib.mczi_set_minimizer_precount(self._h, 1 if enable else 0))

    def debug_packed(self) -> tuple[np.ndarray, np.ndarray]:
        nb = C.c_uint64()
        self._ck(self._lib.mczi_debug_packed(self._h, None, None, 0, C.byref(nb)))
        codes = np.empty(nb.value, dtype=np.uint8)
        starts = np.empty(nb.value, dtype=np.uint8)
        if nb.value:
            self._ck(self._lib.mczi_debug_packed(self._h, codes.ctypes.data, starts.ctypes.data, nb.value,
                                                 C.byref(nb)))
        return codes, starts


_default: Context | None = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default


# ------------------------------------------------------------------ helpers

def read_input(path: str | os.PathLike) -> bytes:
    """Reads a FASTA/FASTQ file as MC does: plain, or gzip / xz / zstd
    compressed (recognised by magic bytes; src/lib.rs:3127-3143) and decoded
    by the library's host-side readers (mczi_read_input_file)."""
    lib = N.load()
    data = C.c_void_p()
    n = C.c_uint64()
    err = C.create_string_buffer(1024)
    rc = lib.mczi_read_input_file(os.fsencode(str(path)), C.byref(data), C.byref(n), err, len(err))
    if rc < 0:
        raise N.MCZIError(rc, err.value.decode(errors="replace"))
    try:
        return C.string_at(data, n.value) if n.value else b""
    finally:
        lib.mczi_free_input(data)


def expand_fofns(fofns: Iterable[str | os.PathLike]) -> list[Path]:
    """File-of-filenames expansion (src/lib.rs:242-276): blank lines and '#'
    comments are skipped, relative paths resolve against the FOFN's folder."""
    out: list[Path] = []
    for fofn in fofns:
        fofn = Path(fofn)
        try:
            text = fofn.read_text()
        except OSError as e:
            raise N.MCZIError(N.MCZI_ERR_IO, f"failed to read FOFN {fofn}") from e
        base = fofn.parent if str(fofn.parent) else Path(".")
        for line_no, raw in enumerate(text.splitlines()):
            line = raw.strip()
            if not line or line.startswith("#"):
                continue
            p = Path(line)
            out.append(p if p.is_absolute() else base / p)
    if not out:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG, "no inputs found in FOFN(s)")
    return out


def validate_config(config: CounterConfig) -> None:
    default_context().validate(config, N.MODE_ABUNDANCE)


def decode_kmer(encoded: int, k: int) -> bytes:
    return bytes(b"ACGT"[(encoded >> (2 * (k - 1 - i))) & 3] for i in range(k))


def encode(seq: bytes) -> int:
    v = 0
    for b in seq:
        v = (v << 2) | {65: 0, 67: 1, 71: 2, 84: 3}[b]
    return v


def _compressed_output(path: Path) -> str | None:
    ext = path.suffix.lower()
    if ext in (".gz", ".gzip"):
        return "gz"
    if ext == ".xz":
        return "xz"
    if ext in (".zst", ".zstd"):
        return "zst"
    return None


def _write_through(path: str | os.PathLike, writer) -> None:
    """Writes through `writer` and compresses by the output's extension as
    MC's output writer does (src/lib.rs:1355-1405): .gz/.gzip gzip level 1,
    .xz preset 6, .zst/.zstd level 1 -- the plain file first, then the
    library's mczi_compress_output (compress_existing_file, :1397)."""
    p = Path(path)
    if _compressed_output(p) is None:
        writer(p)
        return
    tmp = p.with_name(p.name + ".tmp-plain")
    try:
        writer(tmp)
        err = C.create_string_buffer(1024)
        rc = N.load().mczi_compress_output(os.fsencode(str(tmp)), os.fsencode(str(p)), err, len(err))
        if rc < 0:
            raise N.MCZIError(rc, err.value.decode(errors="replace"))
    finally:
        tmp.unlink(missing_ok=True)


def _run(inputs, config: CounterConfig, mode: int, ctx: Context | None) -> Context:
    ctx = ctx or default_context()
    ctx.validate(config, mode)
    if not inputs:
        raise N.MCZIError(N.MCZI_ERR_INVALID_CONFIG,
                          "at least one dataset file is required" if mode else "at least one input file is required")
    data = [x if isinstance(x, (bytes, bytearray, memoryview, np.ndarray)) else read_input(x) for x in inputs]
    ctx.count(data, config, mode)
    return ctx


# ------------------------------------------------------------------ entry points

def count_inputs(inputs, config: CounterConfig, ctx: Context | None = None) -> list[CountedKmer]:
    """Canonical k-mers with count > threshold, sorted by encoded value."""
    return _run(inputs, config, N.MODE_ABUNDANCE, ctx).records(sorted=True).counted()


def count_datasets(inputs, config: CounterConfig, ctx: Context | None = None) -> list[CountedKmer]:
    """fof mode: number of inputs containing each k-mer, kept if > threshold."""
    return _run(inputs, config, N.MODE_PRESENCE, ctx).records(sorted=True).counted()


def count_inputs_to_kff_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> None:
    c = _run(inputs, config, N.MODE_ABUNDANCE, ctx)
    _write_through(output_path, c.write_kff)


def count_inputs_to_fasta_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> None:
    c = _run(inputs, config, N.MODE_ABUNDANCE, ctx)
    _write_through(output_path, c.write_fasta)


def count_datasets_to_kff_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> None:
    c = _run(inputs, config, N.MODE_PRESENCE, ctx)
    _write_through(output_path, c.write_kff)


def count_datasets_to_fasta_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> None:
    c = _run(inputs, config, N.MODE_PRESENCE, ctx)
    _write_through(output_path, c.write_fasta)


def write_kmer_fasta(records: Records, output_path) -> int:
    """The selected-k-mer FASTA of `records` (src/lib.rs:1535-1544): record i
    (from 1) is ">MC_kmer_<i> count=<count>" and the k-mer's bases on one
    line, in the records' order; written by the library
    (mczi_write_kmer_fasta, host only).  Returns the number of records."""
    n = len(records)
    lo = np.ascontiguousarray(records.lo, dtype=np.uint64)
    cnt = np.ascontiguousarray(records.count, dtype=np.uint64)
    hi = np.ascontiguousarray(records.hi, dtype=np.uint64) if records.hi is not None else None
    err = C.create_string_buffer(1024)
    rc = N.load().mczi_write_kmer_fasta(os.fsencode(str(output_path)), lo.ctypes.data if n else None,
                                        hi.ctypes.data if hi is not None and n else None,
                                        cnt.ctypes.data if n else None, n, records.k, err, len(err))
    if rc < 0:
        raise N.MCZIError(rc, err.value.decode(errors="replace") or "invalid k-mer FASTA request")
    return n


def count_inputs_to_kmer_fasta_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> int:
    """Every kept k-mer as a FASTA record (src/lib.rs:306-311), in ascending
    encoded order (the reference writes its partitions' order); returns the
    number of selected k-mers."""
    return write_kmer_fasta(_run(inputs, config, N.MODE_ABUNDANCE, ctx).records(sorted=True), output_path)


def count_datasets_to_kmer_fasta_path(inputs, config: CounterConfig, output_path, ctx: Context | None = None) -> int:
    """fof mode of count_inputs_to_kmer_fasta_path (src/lib.rs:357-363): the
    count of a k-mer is the number of datasets containing it."""
    return write_kmer_fasta(_run(inputs, config, N.MODE_PRESENCE, ctx).records(sorted=True), output_path)
