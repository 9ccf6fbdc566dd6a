"""ZI on the GPU against the oracle: absent canonical k-mer sets must be equal."""
import numpy as np
import pytest

from oracle_ref import encode, to_int

pytestmark = pytest.mark.gpu


def oracle_absent(oracle, index, queries, k):
    lo, hi = oracle.zi_absent(index, queries, k)
    return to_int(lo, hi)


def gpu_absent(ctx, index, queries, k, m):
    from mczi_gb300 import zi
    zi.build_dictionary(index, k, m, ctx=ctx)
    return zi.collect_query_kmers_absent_from_index(ctx, queries).encoded()


def rand_seq(rng, n):
    return rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=n).tobytes()


def mutate(rng, s, rate):
    a = np.frombuffer(s, dtype=np.uint8).copy()
    pos = rng.random(a.size) < rate
    a[pos] = rng.choice(np.frombuffer(b"ACGTN", dtype=np.uint8), size=int(pos.sum()))
    return a.tobytes()


def reads(rng, genome, n, L, rate):
    out = []
    for i in range(n):
        p = int(rng.integers(0, max(1, len(genome) - L)))
        out.append(b">q%d\n" % i + mutate(rng, genome[p:p + L], rate) + b"\n")
    return b"".join(out)


def test_golden_zi(gpu_ctx, golden):
    z = golden["zi"]
    got = gpu_absent(gpu_ctx, z["subtract"]["index"].encode(), [z["subtract"]["query"].encode()], 3, 1)
    assert sorted(got) == sorted(encode(s) for s in z["subtract"]["absent"])
    got = gpu_absent(gpu_ctx, z["dedup"]["index"].encode(), [z["dedup"]["query"].encode()], 3, 1)
    assert got == [encode("CCC")]


def test_zi_validation(gpu_ctx, golden):
    from mczi_gb300 import MCZIError, zi
    for k in golden["zi"]["validate_k"]["ok"]:
        zi.validate_k(k)
    for k in golden["zi"]["validate_k"]["err"]:
        with pytest.raises(MCZIError):
            zi.validate_k(k)
    for k, m in golden["zi"]["default_minimizer_size"]:
        assert zi.default_minimizer_size(k) == m
    with pytest.raises(MCZIError):
        zi.build_dictionary(b">i\nACGTACGT\n", 4, 2, ctx=gpu_ctx)


@pytest.mark.parametrize("k,m", [(3, 1), (5, 3), (11, 5), (21, 11), (31, 19), (33, 19), (45, 21), (63, 31)])
def test_zi_random_parity(gpu_ctx, oracle, k, m):
    rng = np.random.default_rng(k * 31 + m)
    g = rand_seq(rng, 20000)
    index = b">g\n" + g[:12000] + b"\n>h\n" + mutate(rng, g[12000:], 0.002) + b"\n"
    q1 = reads(rng, g, 300, 150, 0.01)
    q2 = reads(rng, rand_seq(rng, 5000), 100, 120, 0.0)
    q3 = b">n\nNNNNACGTNN\n>s\nAC\n"
    assert gpu_absent(gpu_ctx, index, [q1, q2, q3], k, m) == oracle_absent(oracle, index, [q1, q2, q3], k)


def test_zi_c4_shape(gpu_ctx, oracle):
    from mczi_gb300 import gen
    index, query = gen.c4_index_and_query(genome_len=400_000, query_bases=6_000_000, k=31)
    assert gpu_absent(gpu_ctx, index, [query], 31, 19) == oracle_absent(oracle, index, [query], 31)


def test_zi_per_input_equals_alone(gpu_ctx, oracle):
    """A request's result is the same alone and in a batch."""
    from mczi_gb300 import zi
    rng = np.random.default_rng(3)
    g = rand_seq(rng, 30000)
    zi.build_dictionary(b">g\n" + g + b"\n", 31, 19, ctx=gpu_ctx)
    reqs = [reads(rng, g if i % 2 else rand_seq(rng, 3000), int(rng.integers(1, 80)), 150, 0.01) for i in range(70)]
    alone = [zi.collect_query_kmers_absent_from_index(gpu_ctx, [r]).encoded() for r in reqs]
    zi.query_per_input(gpu_ctx, reqs)
    batch = zi.batch_results(gpu_ctx, len(reqs))
    for i, r in enumerate(reqs):
        assert zi.input_result(gpu_ctx, i) == alone[i], i
        assert sorted(int(v) for v in batch[i]) == alone[i], i
        assert alone[i] == oracle_absent(oracle, b">g\n" + g + b"\n", [r], 31)


@pytest.mark.parametrize("bucket", [0, 16, 1])
@pytest.mark.parametrize("k,m", [(31, 19), (31, 7), (33, 19), (63, 11)])
def test_zi_partition_paths(gpu_ctx, oracle, k, m, bucket):
    """Absent runs longer than a tile's per-run limit (low-complexity reads,
    where one minimizer value spans a whole scan tile), expand tiles that
    overflow (long superkmers: small m), and the two-level bucket split (small
    final buckets) all give the oracle's sets, for the union and per input."""
    from mczi_gb300 import zi
    rng = np.random.default_rng(k * 7 + m + bucket)
    g = rand_seq(rng, 30000)
    index = b">g\n" + g + b"\n"
    low = b">a\n" + b"A" * 3000 + b"\n>c\n" + b"AC" * 1500 + b"\n>t\n" + b"ACGTTGCA" * 300 + b"\n"
    qs = [reads(rng, g, 200, 150, 0.01), reads(rng, rand_seq(rng, 6000), 150, 150, 0.0), low,
          low + reads(rng, g, 50, 150, 0.02)]
    gpu_ctx.set_zi_bucket_records(bucket)
    try:
        zi.build_dictionary(index, k, m, ctx=gpu_ctx)
        assert zi.collect_query_kmers_absent_from_index(gpu_ctx, qs).encoded() == oracle_absent(oracle, index, qs, k)
        zi.query_per_input(gpu_ctx, qs)
        for i, q in enumerate(qs):
            assert zi.input_result(gpu_ctx, i) == oracle_absent(oracle, index, [q], k), i
    finally:
        gpu_ctx.set_zi_bucket_records(0)


@pytest.mark.parametrize("seg", [8192, 3 * 8192])
def test_zi_streamed_staging(gpu_ctx, oracle, seg):
    """Queries copied in segments while earlier segments are packed and
    scanned give the same absent sets, for the union and per input."""
    from mczi_gb300 import zi
    rng = np.random.default_rng(seg)
    g = rand_seq(rng, 40000)
    index = b">g\n" + g + b"\n"
    qs = [reads(rng, g, 300, 150, 0.01), reads(rng, rand_seq(rng, 20000), 400, 150, 0.01),
          b">n\nNNNNACGTNN\n>s\nAC\n", reads(rng, g, 200, 150, 0.02)]
    gpu_ctx.set_streamed_staging(True, seg)
    try:
        zi.build_dictionary(index, 31, 19, ctx=gpu_ctx)
        assert zi.collect_query_kmers_absent_from_index(gpu_ctx, qs).encoded() == oracle_absent(oracle, index, qs, 31)
        zi.query_per_input(gpu_ctx, qs)
        for i, q in enumerate(qs):
            assert zi.input_result(gpu_ctx, i) == oracle_absent(oracle, index, [q], 31), i
    finally:
        gpu_ctx.set_streamed_staging(True, 0)


def test_zi_widest_split(gpu_ctx, oracle):
    """2^17 final buckets (8 + 9 bits) from about 3 M absent windows."""
    from mczi_gb300 import zi
    rng = np.random.default_rng(77)
    g = rand_seq(rng, 50000)
    index = b">g\n" + g + b"\n"
    qs = [reads(rng, rand_seq(rng, 400000), 5000, 150, 0.01) for _ in range(4)] + [reads(rng, g, 500, 150, 0.01)]
    gpu_ctx.set_zi_bucket_records(16)
    try:
        zi.build_dictionary(index, 31, 19, ctx=gpu_ctx)
        assert zi.collect_query_kmers_absent_from_index(gpu_ctx, qs).encoded() == oracle_absent(oracle, index, qs, 31)
        zi.query_per_input(gpu_ctx, qs)
        for i, q in enumerate(qs):
            assert zi.input_result(gpu_ctx, i) == oracle_absent(oracle, index, [q], 31), i
    finally:
        gpu_ctx.set_zi_bucket_records(0)


def test_zi_fasta_output(gpu_ctx, oracle, tmp_path):
    from mczi_gb300 import zi
    rng = np.random.default_rng(9)
    g = rand_seq(rng, 8000)
    q = reads(rng, g, 200, 150, 0.02)
    zi.subtract(b">g\n" + g + b"\n", [q], 31, output=tmp_path / "z.fa", ctx=gpu_ctx)
    lo, hi = oracle.zi_absent(b">g\n" + g + b"\n", [q], 31)
    oracle.write_simplitigs(tmp_path / "o.fa", lo, hi, 31)
    assert (tmp_path / "z.fa").read_bytes() == (tmp_path / "o.fa").read_bytes()
    info = zi.info(gpu_ctx)
    assert info["built"] == 1 and info["mphf_levels"] >= 1


def test_serving_results_match_alone(gpu_ctx, oracle):
    """Continuous batching: requests submitted while others run are batched,
    and every request's result equals its result alone."""
    from mczi_gb300 import zi
    from mczi_gb300.serve import ZIServer
    rng = np.random.default_rng(21)
    g = rand_seq(rng, 40000)
    index = b">g\n" + g + b"\n"
    reqs = [reads(rng, g if i % 3 else rand_seq(rng, 4000), int(rng.integers(1, 200)), 150, 0.01) for i in range(60)]
    zi.build_dictionary(index, 31, 19, ctx=gpu_ctx)
    alone = [zi.collect_query_kmers_absent_from_index(gpu_ctx, [r]).encoded() for r in reqs]
    with ZIServer(index, 31, 19, workers=2, max_batch=16, hbm_budget=1 << 30) as srv:
        futs = [srv.submit(r) for r in reqs]
        got = [f.result(timeout=120) for f in futs]
        assert srv.batches < len(reqs)  # requests were batched
    for i in range(len(reqs)):
        assert sorted(int(v) for v in got[i]) == alone[i], i
        assert futs[i].latency_ms >= futs[i].queue_ms >= 0.0
    # a client that needs only the sizes releases requests without copying
    with ZIServer(index, 31, 19, workers=2, max_batch=16, keep_results=False) as srv:
        sizes = [f.result(timeout=120) for f in [srv.submit(r) for r in reqs]]
    assert sizes == [len(a) for a in alone]


def test_serving_wide_keys_and_empty_requests(gpu_ctx, oracle):
    """k > 32 results come back as (lo, hi) pairs; requests with no k-mer
    (empty, too short, not FASTX) get empty sets, not errors."""
    from mczi_gb300.serve import ZIServer
    rng = np.random.default_rng(33)
    g = rand_seq(rng, 20000)
    index = b">g\n" + g + b"\n"
    reqs = [reads(rng, g if i % 2 else rand_seq(rng, 3000), 30, 150, 0.01) for i in range(12)]
    reqs += [b"", b">s\nACGT\n", b"no record here\n"]
    with ZIServer(index, 45, 21, workers=1, max_batch=8) as srv:
        got = [f.result(timeout=120) for f in [srv.submit(r) for r in reqs]]
        assert srv.stats()["requests"] == len(reqs)
    for r, x in zip(reqs, got):
        want = oracle_absent(oracle, index, [r], 45) if r.startswith(b">") else []
        assert sorted((int(h) << 64) | int(l) for l, h in x) == want


def test_dictionary_from_count_result(gpu_ctx, oracle):
    """The MCZI index built on the device from a count's kept k-mers answers
    as ZI over those k-mers (each kept k-mer an index sequence), for k <= 32
    and k > 32."""
    from mczi_gb300 import zi
    from mczi_gb300.mc import CounterConfig, decode_kmer
    rng = np.random.default_rng(8)
    g = rand_seq(rng, 30000)
    idx_reads = reads(rng, g, 600, 150, 0.005)
    q = reads(rng, g, 200, 150, 0.01) + reads(rng, rand_seq(rng, 5000), 50, 150, 0.0)
    for k, m in ((31, 19), (45, 21)):
        n = gpu_ctx.count([idx_reads], CounterConfig(k, m, 1))
        r = gpu_ctx.records(n, sorted=True)
        hi = r.hi if r.hi is not None else np.zeros_like(r.lo)
        kept = b"".join(b">\n" + decode_kmer((int(h) << 64) | int(l), k) + b"\n" for l, h in zip(r.lo, hi))
        zi.build_dictionary_from_result(gpu_ctx, m)
        got = zi.collect_query_kmers_absent_from_index(gpu_ctx, [q]).encoded()
        assert got == oracle_absent(oracle, kept, [q], k), k
