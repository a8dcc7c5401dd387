"""Image input for textures, without OpenImageIO: TIFF, PNG, PPM, PFM and
uncompressed scanline OpenEXR -> (H, W, 3) float32, row 0 at the top.

Replaces the OIIO texture reads behind the reference's OSL texture() and
environment() calls (src/shading/renderservices.cpp in kazen_proto). As OIIO
returns them for a float lookup: 8- and 16-bit integers are scaled to [0, 1]
(no transfer curve), floats are kept, a grey image is spread to RGB, alpha
is dropped.

TIFF follows the TIFF 6.0 specification: chunky (PlanarConfiguration 1)
strips or tiles, 8/16-bit unsigned or 32-bit float samples, compression
none (1), LZW (5, section 13: MSB-first codes of 9-12 bits, Clear 256,
EndOfInformation 257, the code width grows one code early) or Deflate
(8, 32946), with the horizontal-differencing predictor (2, section 14).
PNG follows the PNG specification: 8/16-bit grey, grey+alpha, RGB and RGBA,
no interlace, filter types 0-4.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def _to_rgb(a: np.ndarray) -> np.ndarray:
    if a.ndim == 2:
        a = a[:, :, None]
    c = a.shape[2]
    if c in (1, 2):
        a = np.repeat(a[:, :, :1], 3, axis=2)
    elif c >= 3:
        a = a[:, :, :3]
    return np.ascontiguousarray(a, np.float32)


def _scale(a: np.ndarray) -> np.ndarray:
    if a.dtype == np.uint8:
        return a.astype(np.float32) / 255.0
    if a.dtype == np.uint16:
        return a.astype(np.float32) / 65535.0
    return a.astype(np.float32)


# ---------------------------------------------------------------- TIFF
def lzw_decode(data: bytes) -> bytes:
    """TIFF LZW (TIFF 6.0 section 13)."""
    out = bytearray()
    table = [bytes([i]) for i in range(256)] + [b"", b""]
    width, bitpos, nbits = 9, 0, len(data) * 8
    prev = None
    while bitpos + width <= nbits:
        byte, off = bitpos >> 3, bitpos & 7
        chunk = int.from_bytes(data[byte:byte + 3].ljust(3, b"\0"), "big")
        code = (chunk >> (24 - off - width)) & ((1 << width) - 1)
        bitpos += width
        if code == 257:
            break
        if code == 256:
            table = table[:258]
            width, prev = 9, None
            continue
        if prev is None:
            entry = table[code]
        elif code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        elif code == len(table):
            entry = prev + prev[:1]
            table.append(entry)
        else:
            raise ValueError("corrupt LZW stream")
        out += entry
        prev = entry
        if len(table) + 1 >= (1 << width) and width < 12:
            width += 1
    return bytes(out)


def lzw_encode(data: bytes) -> bytes:
    """TIFF LZW encoder (the inverse of lzw_decode; used to make test images)."""
    table = {bytes([i]): i for i in range(256)}
    nxt, width = 258, 9
    bits, nb = 0, 0
    out = bytearray()

    def emit(code):
        nonlocal bits, nb
        bits = (bits << width) | code
        nb += width
        while nb >= 8:
            nb -= 8
            out.append((bits >> nb) & 0xFF)

    emit(256)
    w = b""
    for ch in data:
        wc = w + bytes([ch])
        if wc in table:
            w = wc
            continue
        emit(table[w])
        table[wc] = nxt
        nxt += 1
        # the decoder adds each entry one code later, so it widens after the
        # code that brings its table to 2^width - 1 entries
        if nxt >= (1 << width) and width < 12:
            width += 1
        if nxt >= 4093:
            emit(256)
            table = {bytes([i]): i for i in range(256)}
            nxt, width = 258, 9
        w = bytes([ch])
    if w:
        emit(table[w])
    emit(257)
    if nb:
        out.append((bits << (8 - nb)) & 0xFF)
    return bytes(out)


_TIFF_TYPES = {1: "B", 2: "c", 3: "H", 4: "I", 5: "II", 6: "b", 7: "B", 8: "h", 9: "i", 10: "ii", 11: "f", 12: "d",
               16: "Q"}


def _tiff_tags(b: bytes, end: str, off: int):
    n = struct.unpack(end + "H", b[off:off + 2])[0]
    tags = {}
    for i in range(n):
        e = off + 2 + 12 * i
        tag, typ, cnt = struct.unpack(end + "HHI", b[e:e + 8])
        fmt = _TIFF_TYPES.get(typ)
        if fmt is None:
            continue
        size = struct.calcsize(end + fmt) * cnt
        raw = b[e + 8:e + 12] if size <= 4 else b[struct.unpack(end + "I", b[e + 8:e + 12])[0]:][:size]
        vals = struct.unpack(end + fmt * cnt, raw[:size]) if fmt != "c" else (raw[:size],)
        tags[tag] = vals
    return tags


def read_tiff(path: str) -> np.ndarray:
    b = open(path, "rb").read()
    if b[:4] not in (b"II*\0", b"MM\0*"):
        raise ValueError(f"{path}: not a TIFF file")
    end = "<" if b[:2] == b"II" else ">"
    t = _tiff_tags(b, end, struct.unpack(end + "I", b[4:8])[0])
    W, H = t[256][0], t[257][0]
    spp = t.get(277, (1,))[0]
    bps = t.get(258, (1,))[0]
    comp = t.get(259, (1,))[0]
    pred = t.get(317, (1,))[0]
    fmt = t.get(339, (1,))[0]
    if t.get(284, (1,))[0] != 1:
        raise ValueError(f"{path}: planar TIFF is not supported")
    if comp not in (1, 5, 8, 32946):
        raise ValueError(f"{path}: TIFF compression {comp} is not supported")
    if (bps, fmt) not in ((8, 1), (16, 1), (32, 3)):
        raise ValueError(f"{path}: {bps}-bit samples (format {fmt}) are not supported")
    dt = np.dtype({8: "u1", 16: "u2", 32: "f4"}[bps]).newbyteorder(end)

    def decode(chunk: bytes) -> bytes:
        if comp == 5:
            return lzw_decode(chunk)
        if comp in (8, 32946):
            return zlib.decompress(chunk)
        return chunk

    def unpredict(a: np.ndarray) -> np.ndarray:  # (rows, cols, spp) integer samples
        if pred == 2:
            a = np.cumsum(a, axis=1, dtype=a.dtype)
        elif pred != 1:
            raise ValueError(f"{path}: TIFF predictor {pred} is not supported")
        return a

    img = np.zeros((H, W, spp), dt.newbyteorder("="))
    if 322 in t:  # tiles
        tw, th = t[322][0], t[323][0]
        offs, cnts = t[324], t[325]
        across = (W + tw - 1) // tw
        for k, (o, c) in enumerate(zip(offs, cnts)):
            a = np.frombuffer(decode(b[o:o + c]), dt)[:tw * th * spp].reshape(th, tw, spp)
            a = unpredict(a.astype(dt.newbyteorder("=")))
            y0, x0 = (k // across) * th, (k % across) * tw
            img[y0:y0 + th, x0:x0 + tw] = a[:min(th, H - y0), :min(tw, W - x0)]
    else:
        rps = t.get(278, (H,))[0]
        y = 0
        for o, c in zip(t[273], t[279]):
            rows = min(rps, H - y)
            a = np.frombuffer(decode(b[o:o + c]), dt)[:rows * W * spp].reshape(rows, W, spp)
            img[y:y + rows] = unpredict(a.astype(dt.newbyteorder("=")))
            y += rows
    return _to_rgb(_scale(img))


# ---------------------------------------------------------------- PNG
def read_png(path: str) -> np.ndarray:
    b = open(path, "rb").read()
    if b[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, b"", None
    while pos < len(b):
        n = struct.unpack(">I", b[pos:pos + 4])[0]
        kind, data = b[pos + 4:pos + 8], b[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", data)
        elif kind == b"IDAT":
            idat += data
        elif kind == b"IEND":
            break
    W, H, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if chans is None or depth not in (8, 16) or interlace:
        raise ValueError(f"{path}: PNG colour type {ctype}, depth {depth}, interlace {interlace} not supported")
    bpp = chans * depth // 8
    raw = zlib.decompress(idat)
    stride = W * bpp
    out = np.zeros((H, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(H):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 1:  # Sub: a running sum per byte of the pixel
            cur = (np.cumsum(line.reshape(-1, bpp), axis=0) & 0xFF).reshape(-1)
        elif f == 2:  # Up
            cur = (line + prev) & 0xFF
        elif f in (3, 4):  # Average, Paeth: sequential along the row, a pixel at a time
            ln = line.reshape(-1, bpp)
            up = prev.reshape(-1, bpp)
            cur2 = np.zeros_like(ln)
            a = np.zeros(bpp, np.int32)
            c = np.zeros(bpp, np.int32)
            for x in range(ln.shape[0]):
                b = up[x]
                if f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = np.abs(b - c), np.abs(a - c), np.abs(a + b - 2 * c)
                    p = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
                a = (ln[x] + p) & 0xFF
                cur2[x] = a
                c = b
            cur = cur2.reshape(-1)
        else:
            raise ValueError(f"{path}: PNG filter {f}")
        out[y] = cur
        prev = cur
    a = out.view(">u2").astype(np.uint16) if depth == 16 else out
    return _to_rgb(_scale(a.reshape(H, W, chans)))


# ---------------------------------------------------------------- PPM / PFM / EXR
def _tokens(b: bytes, n: int):
    toks, pos = [], 0
    while len(toks) < n:
        while b[pos:pos + 1].isspace():
            pos += 1
        if b[pos:pos + 1] == b"#":
            pos = b.index(b"\n", pos) + 1
            continue
        s = pos
        while not b[pos:pos + 1].isspace():
            pos += 1
        toks.append(b[s:pos])
    return toks, pos + 1


def read_ppm(path: str) -> np.ndarray:
    b = open(path, "rb").read()
    (magic, w, h, mx), pos = _tokens(b, 4)
    if magic != b"P6":
        raise ValueError(f"{path}: only binary PPM (P6) is supported")
    W, H, M = int(w), int(h), int(mx)
    a = np.frombuffer(b, ">u2" if M > 255 else np.uint8, W * H * 3, pos).reshape(H, W, 3)
    return np.ascontiguousarray(a.astype(np.float32) / M)


def read_pfm(path: str) -> np.ndarray:
    b = open(path, "rb").read()
    (magic, w, h, sc), pos = _tokens(b, 4)
    if magic not in (b"PF", b"Pf"):
        raise ValueError(f"{path}: not a PFM file")
    c = 3 if magic == b"PF" else 1
    W, H, scale = int(w), int(h), float(sc)
    a = np.frombuffer(b, "<f4" if scale < 0 else ">f4", W * H * c, pos).reshape(H, W, c)
    return _to_rgb(a[::-1])  # PFM stores the bottom row first


def read_exr(path: str) -> np.ndarray:
    """Uncompressed scanline OpenEXR with half or float R, G, B channels."""
    b = open(path, "rb").read()
    if struct.unpack("<I", b[:4])[0] != 20000630:
        raise ValueError(f"{path}: not an OpenEXR file")
    pos, attrs = 8, {}
    while b[pos] != 0:
        e = b.index(b"\0", pos)
        name = b[pos:e].decode()
        e2 = b.index(b"\0", e + 1)
        size = struct.unpack("<i", b[e2 + 1:e2 + 5])[0]
        attrs[name] = b[e2 + 5:e2 + 5 + size]
        pos = e2 + 5 + size
    pos += 1
    if attrs.get("compression", b"\0") != b"\0":
        raise ValueError(f"{path}: compressed OpenEXR is not supported")
    chans, cl = [], attrs["channels"]
    p = 0
    while cl[p] != 0:
        e = cl.index(b"\0", p)
        chans.append((cl[p:e].decode(), struct.unpack("<i", cl[e + 1:e + 5])[0]))
        p = e + 17
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"])
    W, H = x1 - x0 + 1, y1 - y0 + 1
    dts = {1: "<f2", 2: "<f4"}
    pos += 8 * H
    planes = {name: np.zeros((H, W), np.float32) for name, _ in chans}
    for y in range(H):
        pos += 8
        for name, typ in chans:
            if typ not in dts:
                raise ValueError(f"{path}: channel type {typ} is not supported")
            n = W * (2 if typ == 1 else 4)
            planes[name][y] = np.frombuffer(b, dts[typ], W, pos)
            pos += n
    get = lambda k: planes.get(k, planes.get("Y", np.zeros((H, W), np.float32)))  # noqa: E731
    return np.ascontiguousarray(np.stack([get("R"), get("G"), get("B")], -1), np.float32)


READERS = {".tif": read_tiff, ".tiff": read_tiff, ".png": read_png, ".ppm": read_ppm, ".pfm": read_pfm,
           ".exr": read_exr}


def read_image(path: str) -> np.ndarray:
    ext = os.path.splitext(path)[1].lower()
    if ext not in READERS:
        raise ValueError(f"unsupported texture format {ext!r} (supported: {', '.join(sorted(READERS))})")
    return READERS[ext](path)
