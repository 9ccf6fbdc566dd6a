"""BGZF writer: gzip members of at most 65,280 input bytes, each carrying its
size in the "BC" extra subfield (the BGZF layout), so that the library
decodes them on the device (mczi_inflate_gzip; the counting and ZI entry
points take such inputs compressed).  An empty member ends the file, as
BGZF files end.  Members are compressed on host threads (zlib releases the
interpreter lock while it compresses)."""
from __future__ import annotations

import os
import struct
import zlib
from concurrent.futures import ThreadPoolExecutor

BLOCK = 65280


def member(chunk: bytes, level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY) -> bytes:
    """One gzip member of `chunk` (at most 65,280 bytes, so that its size fits the field)."""
    c = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy)
    d = c.compress(chunk) + c.flush()
    bsize = 10 + 2 + 6 + len(d) + 8 - 1  # header, XLEN, the BC subfield, data, trailer; minus one
    if bsize > 0xFFFF:
        raise ValueError("member too large for its size field")
    head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, ord("B"), ord("C"), 2, bsize)
    return head + d + struct.pack("<II", zlib.crc32(chunk) & 0xFFFFFFFF, len(chunk) & 0xFFFFFFFF)


def compress(data, level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY, block: int = BLOCK,
             eof: bool = True, threads: int | None = None) -> bytes:
    """`data` (bytes-like) as BGZF members of `block` bytes, then the end marker."""
    mv = memoryview(data).cast("B")
    chunks = [bytes(mv[i:i + block]) for i in range(0, len(mv), block)]
    n = threads or min(32, os.cpu_count() or 1)
    if n > 1 and len(chunks) > 1:
        with ThreadPoolExecutor(n) as ex:
            parts = list(ex.map(lambda c: member(c, level, strategy), chunks))
    else:
        parts = [member(c, level, strategy) for c in chunks]
    if eof or not chunks:
        parts.append(member(b""))
    return b"".join(parts)
