"""Framebuffer output (sray_gb300/imageio.py): the PNG and PFM files decode
back to the framebuffer they were written from."""
import struct
import zlib

import numpy as np

from sray_gb300 import imageio


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks.setdefault(tag, b"")
        chunks[tag] += body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert depth == 8 and ctype == 6 and b"IEND" in chunks
    raw = zlib.decompress(chunks[b"IDAT"])
    rows = [raw[y * (4 * w + 1):(y + 1) * (4 * w + 1)] for y in range(h)]
    assert all(r[0] == 0 for r in rows)          # filter type none
    return np.frombuffer(b"".join(r[1:] for r in rows), np.uint8).reshape(h, w, 4)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.uniform(-0.2, 1.2, (7, 11, 4)).astype(np.float32)
    p = str(tmp_path / "f.png")
    imageio.write_png(p, img)
    back = _read_png(p)
    want = (np.clip(img, 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    assert np.array_equal(back, want)


def test_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    img = rng.normal(0, 3, (5, 9, 4)).astype(np.float32)
    p = str(tmp_path / "f.pfm")
    imageio.write_pfm(p, img)
    data = open(p, "rb").read()
    head, rest = data.split(b"\n", 3)[:3], data.split(b"\n", 3)[3]
    assert head[0] == b"PF" and head[1] == b"9 5" and float(head[2]) < 0
    back = np.frombuffer(rest, "<f4").reshape(5, 9, 3)[::-1]
    assert np.array_equal(back, img[..., :3])
