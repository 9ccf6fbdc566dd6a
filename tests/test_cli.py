"""The MC / ZI command-line mirrors: flag validation on the CPU (no device
call happens before it), output parity on the GPU against the oracle."""
import numpy as np
import pytest

from oracle_ref import decode, encode, parse_kff, to_int


def run_cli(argv):
    from mczi_gb300 import cli
    return cli.main(argv)


def test_usage_and_flag_validation(tmp_path, capsys):
    assert run_cli([]) == 2
    fa = tmp_path / "a.fa"
    fa.write_bytes(b">r\nACGTACGT\n")
    out = tmp_path / "o.fa"
    # the reference's ensure! messages, before any device work
    assert run_cli(["mc", "-i", str(fa), "-k", "5", "-m", "3", "-o", str(out), "-t", "0"]) == 1
    assert "--threads must be greater than 0" in capsys.readouterr().err
    assert run_cli(["zi", "--index", str(fa), "-i", str(fa), "-k", "4", "-o", str(out)]) == 1
    assert "k must be odd for sshash-rs" in capsys.readouterr().err
    assert run_cli(["zi", "--index", str(fa), "-i", str(fa), "-k", "65", "-o", str(out)]) == 1
    assert "k must be in [3, 63] for sshash-rs" in capsys.readouterr().err
    assert run_cli(["zi", "--index", str(fa), "-i", str(fa), "-k", "5", "-m", "5", "-o", str(out)]) == 1
    assert "minimizer size must be > 0 and < k" in capsys.readouterr().err
    with pytest.raises(SystemExit):  # a required flag is missing: argparse's usage error
        run_cli(["mc", "-i", str(fa), "-k", "5", "-o", str(out)])
    with pytest.raises(SystemExit):
        run_cli(["mc", "-i", str(fa), "-k", "5", "-m", "3", "-o", str(out), "--format", "json"])


def _fasta_kmers(path, k):
    """k-mers of every record of a FASTA whose sequences wrap over lines."""
    out = set()
    for rec in path.read_bytes().split(b">")[1:]:
        s = b"".join(rec.split(b"\n")[1:]).decode()
        for i in range(len(s) - k + 1):
            out.add(encode(s[i:i + k]))
    return out


def _canon(v, k):
    s = decode(v, k)
    rc = s[::-1].translate(str.maketrans("ACGT", "TGCA"))
    return min(v, encode(rc))


@pytest.mark.gpu
def test_mc_cli_kff_and_fofn(oracle, tmp_path):
    from mczi_gb300 import gen
    data = gen.c1_reads(scale=0.002)
    a = tmp_path / "a.fa"
    a.write_bytes(data)
    out = tmp_path / "o.kff"
    assert run_cli(["mc", "-i", str(a), "-k", "31", "-m", "21", "-x", "2", "--format", "kff", "-o", str(out)]) == 0
    _, recs, ok = parse_kff(out.read_bytes())
    assert ok
    lo, hi, cnt = oracle.count([data], 31, 2)
    assert recs == {e: min(int(c), 3) for e, c in zip(to_int(lo, hi), cnt)}  # u8 counts saturate at x + 1
    # fof: two datasets listed in a FOFN, presence counts
    b = tmp_path / "b.fa"
    b.write_bytes(data[: len(data) // 2])
    fofn = tmp_path / "ds.fofn"
    fofn.write_text("a.fa\nb.fa\n")
    out2 = tmp_path / "p.kff"
    assert run_cli(["mc", "-i", str(fofn), "--fofn", "-k", "21", "-m", "11", "-x", "1", "--format", "kff",
                    "-o", str(out2)]) == 0
    _, recs2, ok2 = parse_kff(out2.read_bytes())
    lo2, hi2, cnt2 = oracle.count([data, data[: len(data) // 2]], 21, 1, 1)
    assert ok2 and recs2 == dict(zip(to_int(lo2, hi2), (int(c) for c in cnt2)))


@pytest.mark.gpu
def test_zi_cli_absent_set(oracle, tmp_path):
    rng = np.random.default_rng(3)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=4000).tobytes()
    other = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=3000).tobytes()
    index = b">g\n" + g + b"\n"
    query = b">q1\n" + g[500:1500] + b"\n>q2\n" + other + b"\n"
    ip, qp, out = tmp_path / "i.fa", tmp_path / "q.fa", tmp_path / "novel.fa"
    ip.write_bytes(index)
    qp.write_bytes(query)
    assert run_cli(["zi", "--index", str(ip), "-i", str(qp), "-k", "31", "-o", str(out)]) == 0
    got = {_canon(v, 31) for v in _fasta_kmers(out, 31)}
    assert got == set(oracle_absent_set(oracle, index, [query], 31))


def oracle_absent_set(oracle, index, queries, k):
    lo, hi = oracle.zi_absent(index, queries, k)
    return to_int(lo, hi)


def test_mczi_output_names_and_validation(tmp_path, capsys):
    from mczi_gb300 import mczi
    assert mczi.suffixed_query_file_name("reads.fq.gz", "filtered") == "reads.filtered.fq.gz"
    assert mczi.suffixed_query_file_name("a.FASTA", "x") == "a.x.FASTA"
    assert mczi.suffixed_query_file_name("noext", "f") == "noext.f"
    assert mczi.normalized_output_suffix(" .keep ") == "keep"
    fa = tmp_path / "i.fa"
    fa.write_bytes(b">r\nACGTACGTAC\n")
    assert run_cli(["mczi", "--index-input", str(fa), "--query-input", str(fa), "-k", "5", "-m", "3"]) == 1
    assert "--output is required unless --query-fofn or --output-mode no-output is set" in capsys.readouterr().err
    assert run_cli(["mczi", "--index-input", str(fa), "--query-input", str(fa), "-k", "5", "-m", "3",
                    "--output-mode", "no-output", "-o", str(tmp_path / "o.fa")]) == 1
    assert "--output is not used with --output-mode no-output" in capsys.readouterr().err
    assert run_cli(["mczi", "--index-input", str(fa), "--query-input", str(fa), "-k", "6", "-m", "3",
                    "-o", str(tmp_path / "o.fa")]) == 1
    assert "k must be odd for sshash-rs" in capsys.readouterr().err


@pytest.mark.gpu
def test_mczi_cli_absent_sets(oracle, tmp_path):
    rng = np.random.default_rng(9)
    g = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=5000).tobytes()
    other = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=2000).tobytes()
    # the index set: k-mers seen more than once (x = 1) in reads of g
    reads = b"".join(b">r%d\n%s\n" % (i, g[s:s + 300]) for i, s in enumerate(range(0, 4700, 150)))
    ip = tmp_path / "index.fa"
    ip.write_bytes(reads)
    q1 = tmp_path / "q1.fa"
    q1.write_bytes(b">a\n" + g[1000:1400] + b"\n>b\n" + other[:600] + b"\n")
    q2 = tmp_path / "q2.fasta"
    q2.write_bytes(b">c\n" + other[500:1500] + b"\n")
    lo, hi, _ = oracle.count([reads], 31, 1)
    idx_fa = tmp_path / "kept.fa"
    oracle.write_simplitigs(idx_fa, lo, hi, 31)
    fofn = tmp_path / "queries.fofn"
    fofn.write_text("q1.fa\nq2.fasta\n")
    outdir = tmp_path / "out"
    assert run_cli(["mczi", "--index-input", str(ip), "--query-input", str(fofn), "--query-fofn",
                    "-k", "31", "-m", "19", "-x", "1", "-o", str(outdir)]) == 0
    for q, name in ((q1, "q1.filtered.fa"), (q2, "q2.filtered.fasta")):
        got = {_canon(v, 31) for v in _fasta_kmers(outdir / name, 31)}
        assert got == set(oracle_absent_set(oracle, idx_fa.read_bytes(), [q.read_bytes()], 31))
    # one output for all queries
    single = tmp_path / "all.fa"
    assert run_cli(["mczi", "--index-input", str(ip), "--query-input", str(q1), str(q2),
                    "-k", "31", "-m", "19", "-o", str(single)]) == 0
    got = {_canon(v, 31) for v in _fasta_kmers(single, 31)}
    assert got == set(oracle_absent_set(oracle, idx_fa.read_bytes(), [q1.read_bytes(), q2.read_bytes()], 31))
