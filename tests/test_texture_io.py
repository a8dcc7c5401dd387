"""Texture image input (kazen_proto_gb300.texture_io): TIFF with every
compression and predictor it reads, PNG with all five filter types, and
round trips through the film writers."""
import struct
import zlib

import numpy as np
import pytest

from kazen_proto_gb300 import film_io
from kazen_proto_gb300 import texture_io as T


def test_lzw_round_trip():
    rng = np.random.default_rng(0)
    for n, k in ((0, 2), (1, 2), (300, 2), (20000, 4), (100000, 256), (70000, 16)):
        d = bytes(rng.integers(0, k, n, dtype=np.uint8))
        assert T.lzw_decode(T.lzw_encode(d)) == d


def write_tiff(path, a, compression=1, predictor=1, rows_per_strip=3):
    """Little-endian chunky TIFF of an (H, W, C) uint8/uint16/float32 array."""
    H, W, C = a.shape
    bps = a.dtype.itemsize * 8
    fmt = 3 if a.dtype == np.float32 else 1
    strips = []
    for y in range(0, H, rows_per_strip):
        s = a[y:y + rows_per_strip].astype(a.dtype.newbyteorder("<"))
        if predictor == 2:
            s = np.diff(s, axis=1, prepend=np.zeros_like(s[:, :1]))
        raw = s.tobytes()
        strips.append({1: raw, 5: T.lzw_encode(raw) if compression == 5 else b"", 8: zlib.compress(raw)}[compression])
    data_off = 8
    offs = []
    blob = b""
    for st in strips:
        offs.append(data_off + len(blob))
        blob += st
    ifd_off = data_off + len(blob)
    extra_off = ifd_off + 2 + 12 * 11 + 4
    extra = struct.pack("<%dI" % len(offs), *offs) + struct.pack("<%dI" % len(strips), *[len(x) for x in strips]) \
        + struct.pack("<%dH" % C, *([bps] * C))
    tags = [(256, 4, 1, W), (257, 4, 1, H), (258, 3, C, extra_off + 8 * len(strips) if C > 2 else bps),
            (259, 3, 1, compression), (262, 3, 1, 2 if C >= 3 else 1), (273, 4, len(strips), extra_off),
            (277, 3, 1, C), (278, 4, 1, rows_per_strip), (279, 4, len(strips), extra_off + 4 * len(strips)),
            (317, 3, 1, predictor), (339, 3, 1, fmt)]
    ifd = struct.pack("<H", len(tags))
    for tag, typ, cnt, val in tags:
        if cnt == 1 or (typ == 3 and cnt == 2):
            v = struct.pack("<H", val) + b"\0\0" if typ == 3 else struct.pack("<I", val)
        else:
            v = struct.pack("<I", val)
        ifd += struct.pack("<HHI", tag, typ, cnt) + v
    ifd += b"\0\0\0\0"
    with open(path, "wb") as f:
        f.write(b"II*\0" + struct.pack("<I", ifd_off) + blob + ifd + extra)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32])
@pytest.mark.parametrize("compression,predictor", [(1, 1), (5, 1), (5, 2), (8, 2)])
@pytest.mark.parametrize("channels", [1, 3, 4])
def test_tiff(tmp_path, dtype, compression, predictor, channels):
    if dtype == np.float32 and predictor == 2:
        pytest.skip("the horizontal predictor is defined for integer samples")
    rng = np.random.default_rng(channels)
    if dtype == np.float32:
        a = rng.random((7, 11, channels)).astype(np.float32)
    else:
        a = rng.integers(0, np.iinfo(dtype).max, (7, 11, channels)).astype(dtype)
    write_tiff(tmp_path / "t.tif", a, compression, predictor)
    got = T.read_image(str(tmp_path / "t.tif"))
    scale = 1.0 if dtype == np.float32 else float(np.iinfo(dtype).max)
    want = a.astype(np.float32) / scale
    want = np.repeat(want[:, :, :1], 3, 2) if channels == 1 else want[:, :, :3]
    assert got.shape == (7, 11, 3) and np.allclose(got, want, atol=1e-7)


def _png(path, rows, W, H, ctype, depth=8):
    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(rows)) + chunk(b"IEND", b""))


def test_png_filters(tmp_path):
    rng = np.random.default_rng(1)
    H, W, C = 6, 9, 4
    a = rng.integers(0, 256, (H, W * C)).astype(np.int32)
    raw = b""
    prev = np.zeros(W * C, np.int32)
    for y in range(H):
        f = y % 5
        line = a[y]
        left = np.concatenate([np.zeros(C, np.int32), line[:-C]])
        ul = np.concatenate([np.zeros(C, np.int32), prev[:-C]])
        if f == 0:
            p = np.zeros_like(line)
        elif f == 1:
            p = left
        elif f == 2:
            p = prev
        elif f == 3:
            p = (left + prev) >> 1
        else:
            pa, pb, pc = np.abs(prev - ul), np.abs(left - ul), np.abs(left + prev - 2 * ul)
            p = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, ul))
        raw += bytes([f]) + ((line - p) & 0xFF).astype(np.uint8).tobytes()
        prev = line
    _png(tmp_path / "f.png", raw, W, H, 6)
    got = T.read_image(str(tmp_path / "f.png"))
    assert np.allclose(got, a.reshape(H, W, C)[:, :, :3] / 255.0, atol=1e-7)


@pytest.mark.parametrize("ext", ["png", "ppm", "pfm", "exr"])
def test_round_trip_with_film_writers(tmp_path, ext):
    rng = np.random.default_rng(2)
    img = rng.random((5, 8, 3)).astype(np.float32)
    p = str(tmp_path / ("x." + ext))
    film_io.write_image(p, img)
    got = T.read_image(p)
    tol = 0.5 / 255 + 1e-6 if ext in ("png", "ppm") else 0.0
    assert got.shape == img.shape and np.abs(got - img).max() <= tol


def test_unsupported(tmp_path):
    with pytest.raises(ValueError):
        T.read_image(str(tmp_path / "x.jpg"))
    (tmp_path / "x.png").write_bytes(b"not a png")
    with pytest.raises(ValueError):
        T.read_image(str(tmp_path / "x.png"))
