"""BGZF writer for the tests: gzip members of at most 65,280 input bytes, each
carrying its size in the "BC" extra subfield (the layout of the BGZF format),
so that the library decodes them on the device.  An empty member ends the
file, as BGZF files end."""
import struct
import zlib

BLOCK = 65280


def member(chunk: bytes, level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY) -> bytes:
    c = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy)
    d = c.compress(chunk) + c.flush()
    bsize = 10 + 2 + 6 + len(d) + 8 - 1  # header, XLEN, the BC subfield, data, trailer; minus one
    head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, ord("B"), ord("C"), 2, bsize)
    return head + d + struct.pack("<II", zlib.crc32(chunk) & 0xFFFFFFFF, len(chunk) & 0xFFFFFFFF)


def compress(data: bytes, level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY, block: int = BLOCK,
             eof: bool = True) -> bytes:
    out = bytearray()
    for i in range(0, len(data), block):
        out += member(data[i:i + block], level, strategy)
    if eof or not data:
        out += member(b"")
    return bytes(out)
