"""Seeded synthetic workloads with the shapes of the MC/ZI benchmark configs.

No public dataset is used: genomes are i.i.d. uniform A/C/G/T and reads are
sampled from them with seeded errors (``gen/mczi_gen.c``).  Each builder
returns FASTA bytes as numpy uint8 arrays, or writes into a caller buffer
(e.g. pinned host memory) when ``out`` is given.

Shapes (full size; tests and the CPU baseline use scaled-down variants):
  c1  5 Mbp genome, 1.0 M x 150 bp reads (30x), 0.5 % substitutions; k31 m21 x5
  c2  100 Mbp genome with twenty 5 kbp segments present 20x each; log-normal
      long reads (median 8 kbp, sigma 0.8, 500 bp..100 kbp) to 40x (4 Gbp),
      5 % errors split 60/20/20 substitution/insertion/deletion; k63 m21 x3
  c3  64 datasets from a 20 Mbp base genome, 0.1 % private SNPs each, 150 bp
      reads at coverage U[5, 30], 0.5 % errors; k31 m21 x5 (fof)
  c4  index = the k-mers of a 60 Mbp genome (as overlapping chunks); query =
      150 bp reads, half from that genome and half from an independent one,
      1 % errors; k31 m19
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = N.gen_lib()
    return _lib


def genome(length: int, seed: int, threads: int | None = None) -> np.ndarray:
    g = np.empty(length, dtype=np.uint8)
    lib().gen_genome(seed, length, g.ctypes.data, threads or N.default_threads())
    return g


def insert_repeats(g: np.ndarray, seed: int, n_segments: int, seg_len: int, copies: int) -> None:
    lib().gen_insert_repeats(g.ctypes.data, g.size, seed, n_segments, seg_len, copies)


def variant(g: np.ndarray, seed: int, rate: float) -> np.ndarray:
    out = np.empty_like(g)
    lib().gen_variant(g.ctypes.data, g.size, seed, rate, out.ctypes.data)
    return out


def reads_fasta(g: np.ndarray, seed: int, total_bases: int, *, read_len: float = 150.0, lognormal: bool = False,
                sigma: float = 0.0, min_len: int = 1, max_len: int = 1 << 30, p_sub: float = 0.0,
                p_ins: float = 0.0, p_del: float = 0.0, threads: int | None = None,
                out: tuple[int, int] | None = None) -> np.ndarray | int:
    """Reads as one-line FASTA.  With ``out=(address, capacity)`` writes there
    and returns the byte count; otherwise returns a new array."""
    L = lib()
    nreads = C.c_uint64()
    args = (g.ctypes.data, g.size, seed, total_bases, 1 if lognormal else 0, float(read_len), float(sigma),
            int(min_len), int(max_len), float(p_sub), float(p_ins), float(p_del), threads or N.default_threads())
    need = L.gen_reads_fasta(*args, None, 0, C.byref(nreads))
    if out is not None:
        addr, cap = out
        if cap < need:
            raise ValueError(f"output buffer of {cap} bytes is smaller than {need}")
        L.gen_reads_fasta(*args, C.c_void_p(addr), cap, C.byref(nreads))
        return int(need)
    buf = np.empty(need, dtype=np.uint8)
    L.gen_reads_fasta(*args, buf.ctypes.data, need, C.byref(nreads))
    return buf


def reads_fasta_size(g: np.ndarray, seed: int, total_bases: int, **kw) -> int:
    L = lib()
    nreads = C.c_uint64()
    return int(L.gen_reads_fasta(g.ctypes.data, g.size, seed, total_bases, 1 if kw.get("lognormal") else 0,
                                 float(kw.get("read_len", 150.0)), float(kw.get("sigma", 0.0)),
                                 int(kw.get("min_len", 1)), int(kw.get("max_len", 1 << 30)), float(kw.get("p_sub", 0.0)),
                                 float(kw.get("p_ins", 0.0)), float(kw.get("p_del", 0.0)), 1, None, 0,
                                 C.byref(nreads)))


def chunked_fasta(g: np.ndarray, chunk: int, overlap: int) -> np.ndarray:
    L = lib()
    need = L.gen_chunked_fasta(g.ctypes.data, g.size, chunk, overlap, None, 0)
    buf = np.empty(need, dtype=np.uint8)
    L.gen_chunked_fasta(g.ctypes.data, g.size, chunk, overlap, buf.ctypes.data, need)
    return buf


def fingerprint(buf) -> str:
    """64-bit fingerprint (hex) of a generated workload's bytes: equal on two
    machines iff they generated the same input (the generator is
    arithmetic-only, so x86_64 and aarch64 hosts agree)."""
    a = buf if isinstance(buf, np.ndarray) else np.frombuffer(buf, dtype=np.uint8)
    return "%016x" % lib().gen_fingerprint(a.ctypes.data if a.size else None, a.size, N.default_threads())


def fingerprint_ptr(address: int, nbytes: int) -> str:
    """fingerprint() of `nbytes` bytes at a host address (e.g. a pinned buffer)."""
    return "%016x" % lib().gen_fingerprint(C.c_void_p(address), nbytes, N.default_threads())


@dataclass(frozen=True)
class Workload:
    name: str
    k: int
    m: int
    x: int
    mode: int


C1 = Workload("c1_mc_short_reads_k31", 31, 21, 5, N.MODE_ABUNDANCE)
C2 = Workload("c2_mc_long_reads_k63", 63, 21, 3, N.MODE_ABUNDANCE)
C3 = Workload("c3_mc_fof_64_datasets_k31", 31, 21, 5, N.MODE_PRESENCE)


def c1_reads(scale: float = 1.0, seed: int = 0xC1, out=None):
    g = genome(max(1000, int(5_000_000 * scale)), seed)
    return reads_fasta(g, seed + 1, int(150_000_000 * scale), read_len=150, p_sub=0.005, out=out)


def c2_genome(scale: float = 1.0, seed: int = 0xC2) -> np.ndarray:
    glen = max(200_000, int(100_000_000 * scale))
    g = genome(glen, seed)
    insert_repeats(g, seed + 7, 20, 5000, 20)
    return g


def c2_reads(scale: float = 1.0, seed: int = 0xC2, out=None):
    g = c2_genome(scale, seed)
    return reads_fasta(g, seed + 1, int(4_000_000_000 * scale), lognormal=True, read_len=8000, sigma=0.8,
                       min_len=500, max_len=100_000, p_sub=0.03, p_ins=0.01, p_del=0.01, out=out)


def c2_reads_size(scale: float = 1.0, seed: int = 0xC2) -> int:
    g = c2_genome(scale, seed)
    return reads_fasta_size(g, seed + 1, int(4_000_000_000 * scale), lognormal=True, read_len=8000, sigma=0.8,
                            min_len=500, max_len=100_000, p_sub=0.03, p_ins=0.01, p_del=0.01)


def c3_datasets(n_datasets: int = 64, genome_len: int = 20_000_000, seed: int = 0xC3,
                coverage: tuple[float, float] = (5.0, 30.0)) -> list[np.ndarray]:
    base = genome(genome_len, seed)
    rng = np.random.default_rng(seed)
    covs = rng.uniform(coverage[0], coverage[1], size=n_datasets)
    out = []
    for d in range(n_datasets):
        v = variant(base, seed + 1000 + d, 0.001)
        out.append(reads_fasta(v, seed + 2000 + d, int(genome_len * covs[d]), read_len=150, p_sub=0.005))
    return out


def c4_index_and_query(genome_len: int = 60_000_000, query_bases: int = 2_000_000_000, k: int = 31,
                       seed: int = 0xC4) -> tuple[np.ndarray, np.ndarray]:
    g = genome(genome_len, seed)
    other = genome(genome_len, seed + 99)
    index = chunked_fasta(g, 100_000, k - 1)
    q1 = reads_fasta(g, seed + 1, query_bases // 2, read_len=150, p_sub=0.01)
    q2 = reads_fasta(other, seed + 2, query_bases - query_bases // 2, read_len=150, p_sub=0.01)
    return index, np.concatenate([q1, q2])
