"""The no-allocation packer (mczi_pack_fastx_noalloc) against the packer of
the regular entry point and the oracle.

Callers that cannot allocate device memory -- services that only hand out
HBM from their own pre-sized arena, or paths where a cudaMalloc and its
synchronisation are not allowed -- call mczi_pack_fastx_noalloc with their
own device buffers; its scratch is a fixed static device array.  This test
runs it twice in a row (so the second call sees the first call's leftovers in
the shared scratch) and checks both outputs bit for bit against the codes and
fragment starts produced by mczi_count, and the codes against the oracle's
fragments.  It lives in its own file, collected last, and passes both alone
in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILE = 8192


def _fasta(seed, n_reads, fastq=False):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_reads):
        L = int(rng.integers(1, 900))
        s = rng.choice(np.frombuffer(b"ACGTN", dtype=np.uint8), size=L, p=[0.24, 0.24, 0.24, 0.24, 0.04]).tobytes()
        if fastq:
            out.append(b"@r%d\n%s\n+\n%s\n" % (i, s, b"I" * L))
        else:
            out.append(b">r%d\n%s\n" % (i, b"\n".join(s[j:j + 70] for j in range(0, L, 70))))
    return b"".join(out)


def _unpack(packed, fbits, n):
    idx = np.arange(n, dtype=np.uint64)
    words = packed[(idx >> 4).astype(np.int64)]
    codes = ((words >> (30 - 2 * (idx & 15)).astype(np.uint32)) & 3).astype(np.uint8)
    bw = fbits[(idx >> 5).astype(np.int64)]
    starts = ((bw >> (idx & 31).astype(np.uint32)) & 1).astype(np.uint8)
    return codes, starts


def test_noalloc_packer_matches_count_entry_point():
    torch = pytest.importorskip("torch")
    import oracle_ref
    from mczi_gb300 import build
    build.build_gpu_lib()
    from mczi_gb300 import _native
    from mczi_gb300.mc import Context, CounterConfig
    lib = _native.load()
    ctx = Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    try:
        for seed, fastq in ((1, False), (2, True)):
            raw = _fasta(seed, 4000, fastq)
            # reference: the regular entry point's packed stream
            ctx.count([raw], CounterConfig(1, 1, 0))
            exp_codes, exp_starts = ctx.debug_packed()
            # no-allocation entry point on the caller's device buffers
            padded = raw + b"\n" * ((-len(raw)) % TILE)
            d_text = torch.frombuffer(bytearray(padded), dtype=torch.uint8).to("cuda")
            pw, fw = len(padded) // 16 + 8, len(padded) // 32 + 8
            d_packed = torch.full((pw,), -1, dtype=torch.int32, device="cuda")  # garbage: the call clears it
            d_fbits = torch.full((fw,), -1, dtype=torch.int32, device="cuda")
            nb = C.c_uint64()
            rc = lib.mczi_pack_fastx_noalloc(C.c_void_p(d_text.data_ptr()), len(padded), 1 if fastq else 0,
                                             C.c_void_p(d_packed.data_ptr()), pw, C.c_void_p(d_fbits.data_ptr()), fw,
                                             C.byref(nb), C.c_void_p(stream.cuda_stream))
            assert rc == 0
            assert nb.value == exp_codes.size
            codes, starts = _unpack(d_packed.cpu().numpy().view(np.uint32), d_fbits.cpu().numpy().view(np.uint32),
                                    nb.value)
            assert np.array_equal(codes, exp_codes)
            assert np.array_equal(starts, exp_starts)
            # and directly against the oracle's fragments of the same bytes
            o_codes, o_offs, _ = oracle_ref.fragments(raw, 1)
            o_starts = np.zeros(o_codes.size, dtype=np.uint8)
            o_starts[o_offs[:-1].astype(np.int64)] = 1
            assert np.array_equal(codes, o_codes)
            assert np.array_equal(starts, o_starts)
        # sizes beyond the fixed maximum and unpadded lengths are rejected
        rc = lib.mczi_pack_fastx_noalloc(C.c_void_p(d_text.data_ptr()), (65536 + 1) * TILE, 0,
                                         C.c_void_p(d_packed.data_ptr()), (1 << 40), C.c_void_p(d_fbits.data_ptr()),
                                         (1 << 40), C.byref(nb), C.c_void_p(stream.cuda_stream))
        assert rc == _native.MCZI_ERR_TOO_LARGE
        rc = lib.mczi_pack_fastx_noalloc(C.c_void_p(d_text.data_ptr()), TILE + 1, 0, C.c_void_p(d_packed.data_ptr()),
                                         pw, C.c_void_p(d_fbits.data_ptr()), fw, C.byref(nb),
                                         C.c_void_p(stream.cuda_stream))
        assert rc == _native.MCZI_ERR_INVALID_CONFIG
    finally:
        ctx.close()
