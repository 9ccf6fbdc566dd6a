"""The packer's mask-based FASTA chunk classifier (the header the kernels
include, built for the host) against its byte-by-byte rule, on the CPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_fasta32_matches_byte_rule(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "pack_classify_fuzz"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "mczi_gb300" / "csrc"),
                    str(ROOT / "tests" / "pack_classify_fuzz.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "2000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert "0 mismatches" in r.stdout
