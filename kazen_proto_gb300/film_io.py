"""Film output without OpenImageIO: PNG, PPM, PFM and OpenEXR writers for
(H, W, 3) float images (row 0 at the top).

Replaces Film::write / write_tiles (src/core/film.cpp:57-96 in kazen_proto,
OIIO). The 8-bit formats store the values the way the reference's OIIO
output does for a FLOAT -> UINT8 write: clamped to [0, 1] and scaled by 255,
no transfer curve. PFM and EXR keep 32-bit floats; the EXR file is a
scanline image, no compression, channels B, G, R (the order the format
requires), written from the OpenEXR file-layout specification.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def _as_image(img) -> np.ndarray:
    a = np.asarray(img, np.float32)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError(f"expected an (H, W, 3) image, got {a.shape}")
    return a


def to_8bit(img) -> np.ndarray:
    return np.round(np.clip(_as_image(img), 0.0, 1.0) * 255.0).astype(np.uint8)


def write_ppm(path: str, img) -> None:
    a = to_8bit(img)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(a.tobytes())


def write_pfm(path: str, img) -> None:
    a = _as_image(img)
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (a.shape[1], a.shape[0]))  # negative scale: little-endian
        f.write(np.ascontiguousarray(a[::-1]).astype("<f4").tobytes())  # PFM stores the bottom row first


def write_png(path: str, img) -> None:
    a = to_8bit(img)
    h, w = a.shape[:2]

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))  # filter type 0 per row
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))  # 8-bit RGB
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def write_exr(path: str, img) -> None:
    a = _as_image(img)
    h, w = a.shape[:2]

    def attr(name: str, kind: str, data: bytes) -> bytes:
        return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(data)) + data

    chlist = b"".join(c.encode() + b"\0" + struct.pack("<iBBBBii", 2, 0, 0, 0, 0, 1, 1) for c in "BGR") + b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (struct.pack("<ii", 20000630, 2)
              + attr("channels", "chlist", chlist)
              + attr("compression", "compression", b"\0")
              + attr("dataWindow", "box2i", box)
              + attr("displayWindow", "box2i", box)
              + attr("lineOrder", "lineOrder", b"\0")
              + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
              + attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
              + b"\0")
    line_bytes = 3 * 4 * w
    first = len(header) + 8 * h
    offsets = struct.pack("<%dQ" % h, *[first + y * (8 + line_bytes) for y in range(h)])
    planes = [np.ascontiguousarray(a[:, :, c]).astype("<f4") for c in (2, 1, 0)]  # B, G, R
    with open(path, "wb") as f:
        f.write(header)
        f.write(offsets)
        for y in range(h):
            f.write(struct.pack("<ii", y, line_bytes))
            for p in planes:
                f.write(p[y].tobytes())


WRITERS = {".png": write_png, ".ppm": write_ppm, ".pfm": write_pfm, ".exr": write_exr}


def write_image(path: str, img) -> None:
    """Write by extension: .png, .ppm, .pfm or .exr."""
    ext = os.path.splitext(path)[1].lower()
    if ext not in WRITERS:
        raise ValueError(f"unsupported image format {ext!r} (supported: {', '.join(sorted(WRITERS))})")
    WRITERS[ext](path, img)
