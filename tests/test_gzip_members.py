"""The host parser that finds gzip members carrying their sizes (BGZF), which
decides what is decoded on the device, on the CPU: every member's DEFLATE
span decodes (with zlib) to its part of the input and matches its CRC-32 and
ISIZE; buffers without sizes, truncated ones and trailing garbage are
refused; zero padding after the last member is allowed."""
import shutil
import struct
import subprocess
import zlib
import gzip
from pathlib import Path

import numpy as np
import pytest

from mczi_gb300 import bgzf

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path_factory.mktemp("gzm") / "gzip_members_check"
    csrc = ROOT / "mczi_gb300" / "csrc"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(csrc), str(ROOT / "tests" / "gzip_members_check.cpp"),
                    str(csrc / "decompress.cpp"), "-o", str(exe), "-ldl", "-lpthread"], check=True)
    return exe


def _run(exe, tmp_path, buf: bytes):
    p = tmp_path / "in.gz"
    p.write_bytes(buf)
    r = subprocess.run([str(exe), str(p)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    if lines[0] == "none":
        return None
    ms = [tuple(int(x) for x in ln.split()[1:]) for ln in lines[1:] if ln.startswith("m ")]
    return int(lines[0].split()[3]), ms


def test_bgzf_members_decode_to_the_input(checker, tmp_path):
    rng = np.random.default_rng(5)
    data = rng.choice(list(b"ACGT\n>"), 400_000).astype(np.uint8).tobytes()
    for level, block in ((6, bgzf.BLOCK), (0, 30_000), (1, 777)):
        z = bgzf.compress(data, level=level, block=block)
        total, ms = _run(checker, tmp_path, z)
        assert total == len(data)
        out = b""
        for in_off, in_len, out_len, crc in ms:
            part = zlib.decompress(z[in_off:in_off + in_len], -15)
            assert len(part) == out_len and zlib.crc32(part) == crc
            out += part
        assert out == data
    # zero padding after the end marker is allowed
    assert _run(checker, tmp_path, bgzf.compress(data[:1000]) + b"\0" * 64)[0] == 1000


def test_other_buffers_are_refused(checker, tmp_path):
    data = b">r\nACGT\n" * 10_000
    z = bgzf.compress(data)
    assert _run(checker, tmp_path, gzip.compress(data)) is None          # no size field
    assert _run(checker, tmp_path, z[:-30]) is None                       # truncated
    assert _run(checker, tmp_path, z + b"garbage") is None                # trailing bytes
    assert _run(checker, tmp_path, b"") is None
    assert _run(checker, tmp_path, data) is None                          # not gzip
    # an extra field without the size subfield
    m = bytearray(bgzf.member(data[:500]))
    m[12:14] = b"XY"
    assert _run(checker, tmp_path, bytes(m)) is None
    # a member whose size field runs past the buffer
    m = bytearray(bgzf.member(data[:500]))
    struct.pack_into("<H", m, 16, len(m) + 10)
    assert _run(checker, tmp_path, bytes(m)) is None
