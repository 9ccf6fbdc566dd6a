"""GPU parity: libmczi_gpu (through its C ABI) against the CPU oracle.

Bit-exact set equality of (canonical k-mer, count) records is required for
every case; the oracle itself is pinned by test_oracle_golden.py.
"""
import numpy as np
import pytest

from oracle_ref import encode, parse_kff, to_int

pytestmark = pytest.mark.gpu


def fa(seq):
    return f">s\n{seq}\n".encode()


def gpu_dict(ctx, inputs, k, m, x, mode=0, sorted_=False):
    from mczi_gb300.mc import CounterConfig
    n = ctx.count(inputs, CounterConfig(k, m, x), mode)
    r = ctx.records(n, sorted=sorted_)
    hi = r.hi if r.hi is not None else np.zeros_like(r.lo)
    d = dict(zip(to_int(r.lo, hi), (int(c) for c in r.count)))
    assert len(d) == n, "duplicate k-mer in GPU output"
    return d


def oracle_dict(oracle, inputs, k, x, mode=0):
    lo, hi, cnt = oracle.count(inputs, k, x, mode)
    return dict(zip(to_int(lo, hi), (int(c) for c in cnt)))


def random_fasta(rng, n_reads, lo, hi, n_rate=0.0, lower=0.0):
    out = []
    for i in range(n_reads):
        L = int(rng.integers(lo, hi + 1))
        s = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=L)
        if n_rate:
            s[rng.random(L) < n_rate] = ord("N")
        if lower:
            mask = rng.random(L) < lower
            s[mask] = s[mask] + 32
        out.append(b">r%d\n" % i + s.tobytes() + b"\n")
    return b"".join(out)


def test_golden_count_inputs(gpu_ctx, golden):
    for case in golden["count_inputs"]["cases"]:
        got = gpu_dict(gpu_ctx, [case["fasta"].encode()], case["k"], case["m"], case["x"])
        if "exact" in case:
            assert got == {encode(km): c for km, c in case["exact"]}
        for km, c in case.get("contains", []):
            assert got[encode(km)] == c


def test_golden_ascii_counts(gpu_ctx, golden):
    for seq, k, expected in golden["ascii_counts"]["cases"]:
        got = gpu_dict(gpu_ctx, [fa(seq)], k, min(2, k), 0)
        assert got == {encode(km): c for km, c in expected}, (seq, k)


def test_golden_count_datasets(gpu_ctx, golden):
    for case in golden["count_datasets"]["cases"]:
        got = gpu_dict(gpu_ctx, [d.encode() for d in case["datasets"]], case["k"], case["m"], case["x"], mode=1)
        if "exact" in case:
            assert got == {encode(km): c for km, c in case["exact"]}
        for km, c in case.get("contains", []):
            assert got[encode(km)] == c
        for km in case.get("absent", []):
            assert encode(km) not in got


def test_validation_matches_reference(gpu_ctx, golden):
    from mczi_gb300 import MCZIError
    from mczi_gb300.mc import CounterConfig
    for k, m, x, ds, ok in golden["validation"]["cases"]:
        try:
            gpu_ctx.validate(CounterConfig(k, m, x), 1 if ds else 0)
            passed = True
        except MCZIError:
            passed = False
        assert passed == ok, (k, m, x, ds)


@pytest.mark.parametrize("k,m", [(1, 1), (2, 1), (3, 2), (5, 3), (11, 5), (16, 9), (21, 11), (31, 21), (32, 19),
                                 (33, 21), (45, 31), (63, 21), (64, 64), (31, 31), (25, 40 // 2)])
def test_random_parity(gpu_ctx, oracle, k, m):
    rng = np.random.default_rng(1000 + k * 100 + m)
    data = random_fasta(rng, 300, 1, 400, n_rate=0.01, lower=0.05)
    for x in (0, 1, 3):
        assert gpu_dict(gpu_ctx, [data], k, m, x) == oracle_dict(oracle, [data], k, x), (k, m, x)


def test_low_complexity_parity(gpu_ctx, oracle):
    # homopolymers and short tandem repeats give long superkmers and heavy keys
    parts = [b">h\n" + b"A" * 20000 + b"\n", b">t\n" + b"ACGTTG" * 3000 + b"\n", b">c\n" + b"C" * 33 + b"\n",
             b">d\n" + b"AT" * 9000 + b"\n"]
    data = b"".join(parts)
    for k, m in ((31, 21), (63, 21), (15, 7)):
        for x in (0, 2):
            assert gpu_dict(gpu_ctx, [data], k, m, x) == oracle_dict(oracle, [data], k, x)


def test_formats_and_edges(gpu_ctx, oracle):
    rng = np.random.default_rng(7)
    seq = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=50000).tobytes()
    wrapped = b">long\n" + b"\n".join(seq[i:i + 61] for i in range(0, len(seq), 61)) + b"\n"
    crlf = b">c\r\n" + seq[:3000] + b"\r\n" + seq[3000:5000] + b"\r\n"
    fastq = b"".join(b"@q%d\n%s\n+\n%s\n" % (i, seq[i * 150:(i + 1) * 150], b"I" * 150) for i in range(40))
    longline = b">ll\n" + seq + b"\n"  # one line much longer than a tile
    inputs = [wrapped, crlf, fastq, b"", b"not a fasta file\n", b">empty\n", b">allN\n" + b"N" * 9000 + b"\n",
              longline, b">short\nACGTA\n"]
    for k, m, x in ((31, 21, 0), (17, 9, 1), (63, 21, 0)):
        assert gpu_dict(gpu_ctx, inputs, k, m, x) == oracle_dict(oracle, inputs, k, x)
    # the skipped input is reported like MC_WARN
    assert gpu_ctx.run_stats()[7] == 1


def test_packer_parity(gpu_ctx, oracle):
    rng = np.random.default_rng(11)
    a = random_fasta(rng, 2000, 1, 700, n_rate=0.02, lower=0.1)
    b = b"@x\nACGTNNAC\n+\nIIIIIIII\n@y\nGGTT\n+\nIIII\n"
    c = b">z\nAC\nGT\n\n>w\nTTTT\r\n"
    from mczi_gb300.mc import CounterConfig
    gpu_ctx.count([a, b, c], CounterConfig(1, 1, 0))
    codes, starts = gpu_ctx.debug_packed()
    exp_codes, exp_starts = [], []
    for buf in (a, b, c):
        cc, offs, _ = oracle.fragments(buf, 1)
        exp_codes.append(cc)
        st = np.zeros(cc.size, dtype=np.uint8)
        st[offs[:-1].astype(np.int64)] = 1
        exp_starts.append(st)
    assert np.array_equal(codes, np.concatenate(exp_codes))
    assert np.array_equal(starts, np.concatenate(exp_starts))


def test_bucket_window_guard(gpu_ctx, oracle):
    """The counting kernel's 32-bit counters are bounded by one minimizer
    bucket's k-mer windows; a bucket above the limit fails the count with
    MCZI_ERR_TOO_LARGE instead of wrapping.  The test hook lowers the limit
    (default 2^32 - 1) so the path runs on a small input."""
    from mczi_gb300 import MCZIError, _native as N, gen
    from mczi_gb300.mc import CounterConfig
    lib = N.load()
    data = gen.c1_reads(scale=0.002)
    homopolymer = b">a\n" + b"A" * 5000 + b"\n"  # every window in one bucket
    try:
        for limit, inputs in ((10, [data]), (4000, [homopolymer])):
            assert lib.mczi_debug_set_bucket_window_limit(gpu_ctx.handle, limit) == 0
            for k in (31, 63):
                with pytest.raises(MCZIError) as e:
                    gpu_ctx.count(inputs, CounterConfig(k, 21, 1))
                assert e.value.code == N.MCZI_ERR_TOO_LARGE and "32-bit" in str(e.value)
        assert lib.mczi_debug_set_bucket_window_limit(gpu_ctx.handle, 1 << 33) == N.MCZI_ERR_INVALID_CONFIG
        # 4972 windows fit a limit of 5000
        assert lib.mczi_debug_set_bucket_window_limit(gpu_ctx.handle, 5000) == 0
        assert gpu_dict(gpu_ctx, [homopolymer], 29, 21, 1) == oracle_dict(oracle, [homopolymer], 29, 1)
    finally:
        lib.mczi_debug_set_bucket_window_limit(gpu_ctx.handle, 0)
    assert gpu_dict(gpu_ctx, [data], 31, 21, 1) == oracle_dict(oracle, [data], 31, 1)


def test_tuning_invariance(gpu_ctx, oracle):
    from mczi_gb300 import gen
    data = gen.c1_reads(scale=0.004)
    ref = oracle_dict(oracle, [data], 31, 1)
    try:
        for threads, slots, cps in ((512, 0, 2), (1024, 0, 1), (256, 0, 4), (128, 1024, 2), (256, 300 * 1 + 212, 2)):
            gpu_ctx.set_count_tuning(threads, slots, cps)
            for chunk, fill in ((1, 0.3), (2, 0.6), (7, 0.85)):
                gpu_ctx.set_count_options(chunk, fill)
                for filt in (0, 1):
                    gpu_ctx.set_count_filter(filt)
                    assert gpu_dict(gpu_ctx, [data], 31, 21, 1) == ref, (threads, slots, cps, chunk, fill, filt)
        gpu_ctx.set_count_options(0, 0.0)
        gpu_ctx.set_count_filter(-1)
    finally:
        gpu_ctx.set_count_tuning(0, 0, 0)


def test_c1_shape_parity(gpu_ctx, oracle):
    from mczi_gb300 import gen
    data = gen.c1_reads(scale=0.02)
    for x in (5, 0):
        assert gpu_dict(gpu_ctx, [data], 31, 21, x) == oracle_dict(oracle, [data], 31, x)


def test_c2_shape_parity(gpu_ctx, oracle):
    from mczi_gb300 import gen
    data = gen.c2_reads(scale=0.002)
    try:
        for filt in (-1, 0, 1):
            gpu_ctx.set_count_filter(filt)
            for x in (3, 1, 0):
                assert gpu_dict(gpu_ctx, [data], 63, 21, x) == oracle_dict(oracle, [data], 63, x), (filt, x)
    finally:
        gpu_ctx.set_count_filter(-1)


def test_fof_parity(gpu_ctx, oracle):
    from mczi_gb300 import gen
    ds = gen.c3_datasets(n_datasets=6, genome_len=200_000, coverage=(2.0, 6.0))
    ds.insert(2, np.frombuffer(b"", dtype=np.uint8))  # an empty dataset still counts as a dataset
    for x in (0, 2, 5, 7):
        assert gpu_dict(gpu_ctx, ds, 31, 21, x, mode=1) == oracle_dict(oracle, ds, 31, x, mode=1), x


def test_fof_many_datasets(gpu_ctx, oracle):
    rng = np.random.default_rng(5)
    base = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=3000).tobytes()
    ds = []
    for d in range(130):  # more than 64 datasets: multi-word presence masks
        a, b = sorted(rng.integers(0, 3000, size=2))
        ds.append(b">d\n" + base[a:b + 40] + b"\n")
    for x in (0, 10, 64, 100):
        assert gpu_dict(gpu_ctx, ds, 21, 11, x, mode=1) == oracle_dict(oracle, ds, 21, x, mode=1), x


def test_kff_output(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import gen
    from mczi_gb300.mc import CounterConfig
    data = gen.c1_reads(scale=0.004)
    half = data[: data.size // 2]
    # (k, m, x, mode, count bytes): 1-byte saturated, 8-byte, 4-byte presence,
    # 16-byte keys, 2-byte keys, and an empty result
    cases = [(31, 21, 2, 0, 1), (45, 21, 1, 0, 8), (21, 11, 1, 1, 4), (63, 21, 1, 0, 8), (5, 3, 3, 0, 1),
             (31, 21, 254, 0, 1)]
    for k, m, x, mode, cs in cases:
        ins = [data, half] if mode else [data]
        gpu_ctx.count(ins, CounterConfig(k, m, x), mode)
        p = tmp_path / f"g{k}_{x}.kff"
        gpu_ctx.write_kff(p)
        head, recs, ok = parse_kff(p.read_bytes())
        assert ok
        lo, hi, cnt = oracle.count(ins, k, x, mode)
        exp = dict(zip(to_int(lo, hi), (int(c) for c in cnt)))
        if cs == 1:
            exp = {e: min(c, x + 1, 255) for e, c in exp.items()}
        assert recs == exp
        q = tmp_path / f"o{k}_{x}.kff"
        oracle.write_kff(q, lo, hi, cnt, k, m, x, cs)
        ohead, _, _ = parse_kff(q.read_bytes())
        assert head["head"] == ohead["head"]  # header bytes identical, record count included
        assert p.stat().st_size == q.stat().st_size


def test_fasta_output_byte_identical(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import gen
    from mczi_gb300.mc import CounterConfig
    data = gen.c1_reads(scale=0.002)
    gpu_ctx.count([data], CounterConfig(31, 21, 1))
    p = tmp_path / "g.fa"
    gpu_ctx.write_fasta(p)
    lo, hi, cnt = oracle.count([data], 31, 1)
    q = tmp_path / "o.fa"
    oracle.write_simplitigs(q, lo, hi, 31)
    assert p.read_bytes() == q.read_bytes()


def test_path_entry_points(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import mc
    a = tmp_path / "a.fa"
    a.write_bytes(b">r\nACGTACGTTTGCA\n>s\nAAAANAAAA\n")
    fofn = tmp_path / "in.fofn"
    fofn.write_text("# comment\n\na.fa\n")
    inputs = mc.expand_fofns([fofn])
    assert inputs == [a]
    cfg = mc.CounterConfig(3, 2, 1)
    got = mc.count_inputs(inputs, cfg, ctx=gpu_ctx)
    assert got == [mc.CountedKmer(e, c) for e, c in sorted(oracle_dict(oracle, [a.read_bytes()], 3, 1).items())]
    out = tmp_path / "o.kff"
    mc.count_inputs_to_kff_path(inputs, cfg, out, ctx=gpu_ctx)
    assert out.read_bytes()[:3] == b"KFF"


def test_minimizer_precount_is_conservative(gpu_ctx, oracle):
    """With the pass-1 minimizer table on, results are unchanged and the
    filter removes work (superkmers) only."""
    from mczi_gb300 import gen
    data = gen.c2_reads(scale=0.001)
    ds = gen.c3_datasets(n_datasets=5, genome_len=100_000, coverage=(2.0, 5.0))
    try:
        for k, m, x in ((63, 21, 3), (31, 21, 2), (25, 11, 0)):
            gpu_ctx.set_minimizer_precount(False)
            off = gpu_dict(gpu_ctx, [data], k, m, x)
            n_off = gpu_ctx.run_stats()[1]
            gpu_ctx.set_minimizer_precount(True)
            on = gpu_dict(gpu_ctx, [data], k, m, x)
            n_on = gpu_ctx.run_stats()[1]
            assert on == off == oracle_dict(oracle, [data], k, x)
            assert n_on <= n_off
        for x in (0, 1, 3):
            gpu_ctx.set_minimizer_precount(True)
            on = gpu_dict(gpu_ctx, ds, 31, 21, x, mode=1)
            assert on == oracle_dict(oracle, ds, 31, x, mode=1)
    finally:
        gpu_ctx.set_minimizer_precount(False)


def test_key_range_passes_identical(gpu_ctx, oracle):
    """Counting in passes over disjoint minimizer-key ranges gives the same
    records (abundance and fof, filtered and single-pass rounds)."""
    from mczi_gb300 import gen
    data = gen.c1_reads(scale=0.003)
    ds = gen.c3_datasets(n_datasets=4, genome_len=60_000, coverage=(2.0, 4.0))
    ref31 = oracle_dict(oracle, [data], 31, 1)
    ref63 = oracle_dict(oracle, [data], 63, 0)
    reff = oracle_dict(oracle, ds, 31, 1, mode=1)
    try:
        for passes in (1, 2, 3, 7):
            gpu_ctx.set_key_range_passes(passes)
            for filt in (0, 1):
                gpu_ctx.set_count_filter(filt)
                assert gpu_dict(gpu_ctx, [data], 31, 21, 1) == ref31, (passes, filt)
                assert gpu_dict(gpu_ctx, ds, 31, 21, 1, mode=1) == reff, (passes, filt)
            assert gpu_dict(gpu_ctx, [data], 63, 21, 0) == ref63, passes
    finally:
        gpu_ctx.set_key_range_passes(0)
        gpu_ctx.set_count_filter(-1)


def test_autotuner_keeps_results(gpu_ctx, oracle, tmp_path, monkeypatch):
    from mczi_gb300 import autotune, gen
    from mczi_gb300.mc import CounterConfig
    monkeypatch.setenv("MCZI_TUNE_CACHE", str(tmp_path / "tune.json"))
    data = gen.c2_reads(scale=0.001)
    cfg = CounterConfig(63, 21, 3)
    best, rep = autotune.tune(gpu_ctx, [data], cfg, 0, repeats=1)
    assert rep["candidates"] > 5 and rep["best_ms"] <= rep["default_ms"]
    try:
        assert gpu_dict(gpu_ctx, [data], 63, 21, 3) == oracle_dict(oracle, [data], 63, 3)
        best2, rep2 = autotune.tune(gpu_ctx, [data], cfg, 0)
        assert rep2["cached"] and best2 == best
    finally:
        autotune.DEFAULT.apply(gpu_ctx)


def test_graph_replay_identical(gpu_ctx, oracle):
    """Counts replayed from a captured CUDA graph equal the plain path, also
    for new inputs of the same layout and across key-range passes."""
    from mczi_gb300 import gen
    a = gen.c1_reads(scale=0.002, seed=11)
    b = gen.c1_reads(scale=0.002, seed=12)  # same size and layout, other reads
    try:
        gpu_ctx.set_graph_replay(True)
        for passes in (1, 2):
            gpu_ctx.set_key_range_passes(passes)
            for data in (a, b, a):
                for _ in range(2):
                    assert gpu_dict(gpu_ctx, [data], 31, 21, 1) == oracle_dict(oracle, [data], 31, 1), passes
        big = gen.c1_reads(scale=0.004, seed=13)  # other layout: plain path, then a new capture
        assert gpu_dict(gpu_ctx, [big], 31, 21, 1) == oracle_dict(oracle, [big], 31, 1)
        assert gpu_dict(gpu_ctx, [big], 31, 21, 1) == oracle_dict(oracle, [big], 31, 1)
    finally:
        gpu_ctx.set_graph_replay(False)
        gpu_ctx.set_key_range_passes(0)


@pytest.mark.parametrize("k,m", [(31, 15), (45, 17)])
def test_records_into_caller_buffers(gpu_ctx, k, m):
    """Unsorted records copied straight into caller-owned (oversized, reused)
    arrays equal the sorted host path, record for record."""
    from mczi_gb300.mc import CounterConfig
    rng = np.random.default_rng(k)
    data = random_fasta(rng, 300, 100, 900)
    n = gpu_ctx.count([data], CounterConfig(k, m, 1))
    ref = gpu_ctx.records(n, sorted=True)
    bufs = [np.full(n + 17, 7, dtype=np.uint64) for _ in range(3)]
    for _ in range(2):
        r = gpu_ctx.records(n, sorted=False, out=(bufs[0], bufs[1] if k > 32 else None, bufs[2]))
        assert len(r.lo) == n and len(r.count) == n
        hi = r.hi if r.hi is not None else np.zeros_like(r.lo)
        rhi = ref.hi if ref.hi is not None else np.zeros_like(ref.lo)
        order = np.lexsort((r.lo, hi))
        assert np.array_equal(r.lo[order], ref.lo) and np.array_equal(hi[order], rhi)
        assert np.array_equal(r.count[order], ref.count)
        assert (bufs[0][n:] == 7).all() and (bufs[2][n:] == 7).all()


def _fastq(rng, n, L):
    seqs = [rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=L).tobytes() for _ in range(n)]
    return b"".join(b"@q%d\n%s\n+\n%s\n" % (i, s, b"I" * L) for i, s in enumerate(seqs))


@pytest.mark.parametrize("seg", [8192, 3 * 8192, 65536])
def test_streamed_staging_identical(gpu_ctx, oracle, seg):
    """mczi_count with the staging streamed in small segments (copies
    overlapped with pack + scan) gives exactly the records of the fully staged
    path: several files, reads longer than a segment, FASTQ, fof mode."""
    from mczi_gb300.mc import CounterConfig
    rng = np.random.default_rng(seg)
    genome = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=60_000).tobytes()
    long_reads = b"".join(b">L%d\n%s\n" % (i, genome[s:s + 20_000]) for i, s in enumerate((0, 7_000, 33_000)))
    files = [random_fasta(rng, 200, 100, 600), long_reads, _fastq(rng, 150, 150), random_fasta(rng, 50, 20, 90)]
    shared = files + [b">g\n" + genome[5_000:15_000] + b"\n"]  # fof: k-mers in two datasets
    cases = [(files, 31, 21, 1, 0), (files, 45, 17, 1, 0), (files[:2], 63, 25, 0, 0), (shared, 21, 11, 1, 1)]
    try:
        for inputs, k, m, x, mode in cases:
            gpu_ctx.set_streamed_staging(False)
            plain = gpu_dict(gpu_ctx, inputs, k, m, x, mode)
            gpu_ctx.set_streamed_staging(True, seg)
            streamed = gpu_dict(gpu_ctx, inputs, k, m, x, mode)
            assert streamed == plain, (k, m, x, mode)
            assert len(plain) > 0
            # the streamed call leaves the inputs staged: a recount of them agrees
            n = gpu_ctx.count_staged(CounterConfig(k, m, x), mode)
            assert n == len(plain)
        assert plain == oracle_dict(oracle, shared, 21, 1, 1)
    finally:
        gpu_ctx.set_streamed_staging(True, 0)


def test_packer_markers_inside_lines(gpu_ctx, oracle):
    """'>' / '@' inside a sequence line are breaks, not record starts -- also
    when they follow an all-ACGT 32-byte chunk that began at a line start (the
    packer's fast path), at every 32-byte phase of the tile."""
    from mczi_gb300.mc import CounterConfig
    rng = np.random.default_rng(5)
    bufs = []
    for off in (0, 1, 31, 32, 33, 63, 64, 65, 96, 127, 128):
        head = b">" + b"h" * max(0, off - 2) + b"\n" if off >= 2 else b""
        lines = []
        for j in range(6):
            s = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=200).tobytes()
            cut = 32 * (j % 3 + 1)
            lines.append(s[:cut] + (b">" if j % 2 else b"@") + s[cut:])
        bufs.append((head if off >= 2 else b">r\n") + b"\n".join(lines) + b"\n")
    fq = b"@q\n" + b"A" * 32 + b">" + b"C" * 40 + b"\n+\n" + b"I" * 73 + b"\n"
    bufs.append(fq)
    gpu_ctx.count(bufs, CounterConfig(1, 1, 0))
    codes, starts = gpu_ctx.debug_packed()
    exp_codes, exp_starts = [], []
    for buf in bufs:
        cc, offs, _ = oracle.fragments(buf, 1)
        exp_codes.append(cc)
        st = np.zeros(cc.size, dtype=np.uint8)
        st[offs[:-1].astype(np.int64)] = 1
        exp_starts.append(st)
    assert np.array_equal(codes, np.concatenate(exp_codes))
    assert np.array_equal(starts, np.concatenate(exp_starts))
    for k in (5, 31):
        assert gpu_dict(gpu_ctx, bufs, k, min(k, 3), 0) == oracle_dict(oracle, bufs, k, 0)


@pytest.mark.parametrize("k,m,x", [(31, 21, 1), (16, 9, 0), (4, 3, 0), (63, 25, 1), (64, 31, 0), (22, 11, 1)])
def test_simplitig_fasta_byte_identical(gpu_ctx, oracle, tmp_path, k, m, x):
    """The simplitig FASTA (device extension table + host walk) equals the
    oracle's greedy writer byte for byte: odd and even k (palindromes), 64-
    and 128-bit keys, repeat-rich input with branching paths."""
    from mczi_gb300.mc import CounterConfig
    rng = np.random.default_rng(k * 7 + x)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=3000).tobytes()
    reads = [g[s:s + 400] for s in rng.integers(0, 2600, size=40)]
    reads += [g[100:300] + b"A" + g[301:500], (b"AC" * 60), (b"AAAT" * 40)]
    data = b"".join(b">r%d\n%s\n" % (i, r) for i, r in enumerate(reads))
    n = gpu_ctx.count([data], CounterConfig(k, m, x))
    assert n > 0
    p = tmp_path / "g.fa"
    gpu_ctx.write_fasta(p)
    lo, hi, _ = oracle.count([data], k, x)
    q = tmp_path / "o.fa"
    oracle.write_simplitigs(q, lo, hi, k)
    assert p.read_bytes() == q.read_bytes()


def test_route_superkmers_union_equals_single(gpu_ctx, oracle):
    """The multi-GPU plan's local step (mczi_route_superkmers) on one GPU: the
    reads split in three shares, each share routed to three destinations,
    every destination counts what it received; the union of the three
    results equals the single count and the oracle, record for record."""
    from mczi_gb300 import exchange, gen
    from mczi_gb300.mc import CounterConfig
    for k, m, x, buf in ((31, 21, 1, gen.c1_reads(scale=0.004)), (63, 21, 2, gen.c2_reads(0.001))):
        world = 3
        cfg = CounterConfig(k, m, x)
        received = [[] for _ in range(world)]
        for share in exchange.split_records(buf, world):
            for d, g in enumerate(exchange.route_superkmers(gpu_ctx, [share], cfg, world)):
                if g.size:
                    received[d].append(g)
        parts = []
        for d in range(world):
            assert received[d], d  # every destination gets superkmers
            n = gpu_ctx.count(received[d], cfg)
            r = gpu_ctx.records(n, sorted=True)
            parts.append((r.lo, r.hi if r.hi is not None else np.zeros_like(r.lo), r.count))
        lo = np.concatenate([p[0] for p in parts])
        hi = np.concatenate([p[1] for p in parts])
        cnt = np.concatenate([p[2] for p in parts])
        order = np.lexsort((lo, hi))
        olo, ohi, ocnt = oracle.count([buf], k, x)
        assert np.array_equal(lo[order], olo) and np.array_equal(cnt[order], ocnt), k
        if k > 32:
            assert np.array_equal(hi[order], ohi)


def test_route_datasets_presence_union_equals_single(gpu_ctx, oracle):
    """fof mode of the multi-GPU plan on one GPU: every dataset split in
    three shares, each share routed to three destinations on its own; every
    destination counts, in presence mode, one input per dataset that sent it
    records; the union of the three results equals the oracle's presence
    count of the whole datasets, record for record."""
    from mczi_gb300 import exchange, gen
    from mczi_gb300.mc import CounterConfig
    datasets = gen.c3_datasets(n_datasets=6, genome_len=200_000, coverage=(2.0, 6.0))
    k, m, x, world = 31, 21, 2, 3
    cfg = CounterConfig(k, m, x)
    received = [[[] for _ in datasets] for _ in range(world)]  # [destination][dataset]
    for i, ds in enumerate(datasets):
        for share in exchange.split_records(ds, world):
            for d, g in enumerate(exchange.route_superkmers(gpu_ctx, [share], cfg, world)):
                if g.size:
                    received[d][i].append(g)
    los, cnts = [], []
    for d in range(world):
        inputs = [np.concatenate(p) for p in received[d] if p]
        assert len(inputs) == len(datasets), d  # every dataset reaches every destination here
        n = gpu_ctx.count(inputs, cfg, 1)
        r = gpu_ctx.records(n, sorted=True)
        los.append(r.lo)
        cnts.append(r.count)
    lo, cnt = np.concatenate(los), np.concatenate(cnts)
    order = np.argsort(lo, kind="stable")
    olo, _, ocnt = oracle.count(datasets, k, x, 1)
    assert olo.size > 0 and np.array_equal(lo[order], olo) and np.array_equal(cnt[order], ocnt)
