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
