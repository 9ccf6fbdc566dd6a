"""ctypes binding of ``libmczi_gpu.so`` (the C ABI in ``include/mczi_gpu.h``).

The shared library is built in-tree by :mod:`mczi_gb300.build`.  There is no
Python or CPU fallback: if the library or a CUDA device is missing, calls fail
with :class:`MCZIError`.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"

MCZI_OK = 0
MCZI_ERR_INVALID_CONFIG = -1
MCZI_ERR_IO = -2
MCZI_ERR_OOM = -3
MCZI_ERR_DEVICE = -4
MCZI_ERR_TIMEOUT = -5
MCZI_ERR_STATE = -6
MCZI_ERR_TOO_LARGE = -7

MODE_ABUNDANCE = 0
MODE_PRESENCE = 1

_CODE_NAMES = {
    MCZI_ERR_INVALID_CONFIG: "invalid config",
    MCZI_ERR_IO: "I/O error",
    MCZI_ERR_OOM: "out of device memory",
    MCZI_ERR_DEVICE: "device error",
    MCZI_ERR_TIMEOUT: "device wait timed out",
    MCZI_ERR_STATE: "call out of order",
    MCZI_ERR_TOO_LARGE: "input larger than the fixed maximum",
}


class MCZIError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message or _CODE_NAMES.get(code, f"error {code}"))
        self.code = code


class CounterConfigC(C.Structure):
    _fields_ = [("k", C.c_uint32), ("minimizer", C.c_uint32), ("threshold", C.c_uint64),
                ("partition_count", C.c_uint32)]


class InputC(C.Structure):
    _fields_ = [("data", C.c_void_p), ("len", C.c_uint64)]


# (name, restype, argtypes) of every symbol declared in include/mczi_gpu.h
SIGNATURES = [
    ("mczi_open", C.c_int32, [C.c_int32, C.POINTER(C.c_void_p)]),
    ("mczi_close", C.c_int32, [C.c_void_p]),
    ("mczi_last_error", C.c_char_p, [C.c_void_p]),
    ("mczi_set_stream", C.c_int32, [C.c_void_p, C.c_void_p]),
    ("mczi_validate_config", C.c_int32, [C.c_void_p, C.POINTER(CounterConfigC), C.c_int32]),
    ("mczi_count", C.c_int32, [C.c_void_p, C.POINTER(CounterConfigC), C.c_int32, C.POINTER(InputC), C.c_size_t,
                                C.POINTER(C.c_uint64)]),
    ("mczi_stage", C.c_int32, [C.c_void_p, C.POINTER(InputC), C.c_size_t]),
    ("mczi_count_staged", C.c_int32, [C.c_void_p, C.POINTER(CounterConfigC), C.c_int32, C.POINTER(C.c_uint64)]),
    ("mczi_result_copy", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int32]),
    ("mczi_result_digest", C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64)]),
    ("mczi_result_write_kff", C.c_int32, [C.c_void_p, C.c_char_p]),
    ("mczi_result_write_fasta", C.c_int32, [C.c_void_p, C.c_char_p]),
    ("mczi_route_superkmers", C.c_int32, [C.c_void_p, C.POINTER(CounterConfigC), C.POINTER(InputC), C.c_size_t,
                                          C.c_uint32, C.POINTER(C.c_uint64)]),
    ("mczi_route_copy", C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64]),
    ("mczi_count_inputs_to_kff_path", C.c_int32, [C.c_void_p, C.POINTER(C.c_char_p), C.c_size_t,
                                                  C.POINTER(CounterConfigC), C.c_char_p]),
    ("mczi_count_inputs_to_fasta_path", C.c_int32, [C.c_void_p, C.POINTER(C.c_char_p), C.c_size_t,
                                                    C.POINTER(CounterConfigC), C.c_char_p]),
    ("mczi_count_datasets_to_kff_path", C.c_int32, [C.c_void_p, C.POINTER(C.c_char_p), C.c_size_t,
                                                    C.POINTER(CounterConfigC), C.c_char_p]),
    ("mczi_count_datasets_to_fasta_path", C.c_int32, [C.c_void_p, C.POINTER(C.c_char_p), C.c_size_t,
                                                      C.POINTER(CounterConfigC), C.c_char_p]),
    ("mczi_phase_times", C.c_int32, [C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    ("mczi_run_stats", C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int32]),
    ("mczi_set_count_tuning", C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    ("mczi_set_count_options", C.c_int32, [C.c_void_p, C.c_int32, C.c_float]),
    ("mczi_set_count_filter", C.c_int32, [C.c_void_p, C.c_int32]),
    ("mczi_set_key_range_passes", C.c_int32, [C.c_void_p, C.c_int32]),
    ("mczi_set_graph_replay", C.c_int32, [C.c_void_p, C.c_int32]),
    ("mczi_set_minimizer_precount", C.c_int32, [C.c_void_p, C.c_int32]),
    ("mczi_set_streamed_staging", C.c_int32, [C.c_void_p, C.c_int32, C.c_uint64]),
    ("mczi_set_zi_bucket_records", C.c_int32, [C.c_void_p, C.c_uint32]),
    ("mczi_debug_packed", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("mczi_debug_set_bucket_window_limit", C.c_int32, [C.c_void_p, C.c_uint64]),
    ("mczi_zi_build", C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32]),
    ("mczi_zi_query", C.c_int32, [C.c_void_p, C.POINTER(InputC), C.c_size_t, C.POINTER(C.c_uint64)]),
    ("mczi_zi_build_from_result", C.c_int32, [C.c_void_p, C.c_uint32]),
    ("mczi_zi_build_path", C.c_int32, [C.c_void_p, C.c_char_p, C.c_uint32, C.c_uint32]),
    ("mczi_zi_query_paths", C.c_int32, [C.c_void_p, C.POINTER(C.c_char_p), C.c_size_t, C.POINTER(C.c_uint64)]),
    ("mczi_read_input_file", C.c_int32, [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_char_p,
                                         C.c_uint64]),
    ("mczi_free_input", None, [C.c_void_p]),
    ("mczi_compress_output", C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint64]),
    ("mczi_write_kmer_fasta", C.c_int32, [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                          C.c_char_p, C.c_uint64]),
    ("mczi_inflate_gzip", C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                      C.POINTER(C.c_uint64)]),
    ("mczi_zi_query_per_input", C.c_int32, [C.c_void_p, C.POINTER(InputC), C.c_size_t, C.POINTER(C.c_uint64)]),
    ("mczi_zi_input_result", C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64,
                                         C.POINTER(C.c_uint64)]),
    ("mczi_zi_result_masks", C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_int32)]),
    ("mczi_zi_batch_split", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                        C.POINTER(C.c_uint64)]),
    ("mczi_zi_info", C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int32]),
    ("mczi_pack_fastx_noalloc", C.c_int32, [C.c_void_p, C.c_uint64, C.c_int32, C.c_void_p, C.c_uint64, C.c_void_p,
                                            C.c_uint64, C.POINTER(C.c_uint64), C.c_void_p]),
    ("mczi_serve_open", C.c_int32, [C.c_int32, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32,
                                    C.c_uint64, C.POINTER(C.c_void_p)]),
    ("mczi_serve_submit", C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("mczi_serve_next", C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("mczi_serve_result", C.c_int32, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64,
                                      C.POINTER(C.c_uint64)]),
    ("mczi_serve_release", C.c_int32, [C.c_void_p, C.c_uint64]),
    ("mczi_serve_error", C.c_char_p, [C.c_void_p, C.c_uint64]),
    ("mczi_serve_stats", C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    ("mczi_serve_close", C.c_int32, [C.c_void_p]),
]

_lib = None


def lib_path() -> Path:
    return LIB_DIR / "libmczi_gpu.so"


def load(required: bool = True):
    """Loads libmczi_gpu.so; raises MCZIError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        if not required:
            return None
        raise MCZIError(MCZI_ERR_DEVICE, f"{p} is missing: run `python -m mczi_gb300.build` (no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(ctx, rc: int) -> int:
    if rc < 0:
        msg = load().mczi_last_error(ctx)
        raise MCZIError(rc, msg.decode() if msg else "")
    return rc


def gen_lib():
    p = LIB_DIR / "libmczi_gen.so"
    if not p.exists():
        raise MCZIError(MCZI_ERR_STATE, f"{p} is missing: run `python -m mczi_gb300.build`")
    lib = C.CDLL(str(p))
    lib.gen_genome.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p, C.c_int]
    lib.gen_genome.restype = None
    lib.gen_insert_repeats.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_int]
    lib.gen_insert_repeats.restype = None
    lib.gen_variant.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_double, C.c_void_p]
    lib.gen_variant.restype = None
    lib.gen_reads_fasta.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_double,
                                    C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    lib.gen_reads_fasta.restype = C.c_uint64
    lib.gen_chunked_fasta.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64]
    lib.gen_chunked_fasta.restype = C.c_uint64
    lib.gen_fingerprint.argtypes = [C.c_void_p, C.c_uint64, C.c_int]
    lib.gen_fingerprint.restype = C.c_uint64
    return lib


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))
