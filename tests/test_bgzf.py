"""The BGZF writer (mczi_gb300.bgzf): standard gzip, every member carrying its
size, and the format's end marker; no GPU needed."""
import gzip
import struct
import zlib

import numpy as np

from mczi_gb300 import bgzf

# the 28-byte empty member BGZF files end with (BGZF format description)
EOF_MARKER = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")


def _members(z: bytes):
    out, p = [], 0
    while p < len(z):
        assert z[p:p + 4] == b"\x1f\x8b\x08\x04"
        xlen = struct.unpack_from("<H", z, p + 10)[0]
        assert z[p + 12:p + 16] == b"BC\x02\x00" and xlen == 6
        bsize = struct.unpack_from("<H", z, p + 16)[0]
        out.append(z[p:p + bsize + 1])
        p += bsize + 1
    return out


def test_bgzf_round_trip_and_layout():
    rng = np.random.default_rng(1)
    data = b"".join([b">r\n", rng.choice(list(b"ACGT"), 300_000).astype(np.uint8).tobytes(), b"\n"])
    for level in (0, 1, 6, 9):
        z = bgzf.compress(data, level=level)
        assert gzip.decompress(z) == data
        ms = _members(z)
        assert ms[-1] == EOF_MARKER
        assert sum(struct.unpack_from("<I", m, len(m) - 4)[0] for m in ms) == len(data)
        for m in ms[:-1]:
            assert len(m) <= 65536
    assert bgzf.compress(b"") == EOF_MARKER
    assert bgzf.member(b"") == EOF_MARKER
    # threads do not change the bytes
    assert bgzf.compress(data, threads=1) == bgzf.compress(data, threads=8)
    assert zlib.crc32(gzip.decompress(bgzf.compress(data, strategy=zlib.Z_FIXED))) == zlib.crc32(data)
