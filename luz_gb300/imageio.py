"""PNG output of composed frames (RGBA8), written with zlib: the headless stand-in
for the reference's swapchain present."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def write_png(path, rgba: np.ndarray) -> None:
    """rgba: (H, W, 4) or (H, W, 3) uint8."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w, c = img.shape
    ctype = {3: 2, 4: 6}[c]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(t: bytes, d: bytes) -> bytes:
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(data)
