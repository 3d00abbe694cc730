"""Framebuffer output: PNG (8-bit sRGB-less clamp, as the reference's imago
save of an RGBA float image, src/img.cc:80-83) and PFM (lossless float)."""
import struct
import zlib

import numpy as np

__all__ = ["write_png", "write_pfm"]


def write_png(path, rgba):
    """rgba: float [h, w, 4] in [0, 1] (clamped); row 0 is the top row."""
    img = np.clip(np.asarray(rgba, dtype=np.float32), 0.0, 1.0)
    h, w = img.shape[:2]
    px = (img * 255.0 + 0.5).astype(np.uint8)
    raw = b"".join(b"\x00" + px[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def write_pfm(path, rgba):
    """Portable float map of the RGB channels (bottom-up rows, little endian)."""
    img = np.asarray(rgba, dtype=np.float32)[..., :3]
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())
