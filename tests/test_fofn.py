"""File-of-filenames expansion (mczi_gb300.mc.expand_fofns) on the CPU,
with the reference's own cases (src/lib.rs:5993-6025)."""
import pytest


def test_relative_paths_resolve_and_comments_are_skipped(tmp_path):
    from mczi_gb300.mc import expand_fofns
    (tmp_path / "nested").mkdir()
    a, b = tmp_path / "nested" / "a.fa", tmp_path / "b.fa"
    a.write_bytes(b">a\nAAA\n")
    b.write_bytes(b">b\nCCC\n")
    fofn = tmp_path / "inputs.fofn"
    fofn.write_text(f"\n# comment\nnested/a.fa\n{b}\n")
    assert expand_fofns([fofn]) == [a, b]


def test_empty_fofn_is_rejected(tmp_path):
    from mczi_gb300 import _native as N
    from mczi_gb300.mc import expand_fofns
    fofn = tmp_path / "empty.fofn"
    fofn.write_text("\n# no inputs\n")
    with pytest.raises(N.MCZIError, match="no inputs found"):
        expand_fofns([fofn])
    with pytest.raises(N.MCZIError, match="failed to read FOFN"):
        expand_fofns([tmp_path / "missing.fofn"])
