"""Image-file decoding restated from the format specifications — TEST INFRASTRUCTURE ONLY.

Upstream reads image files with ``fluidimage.util.imread`` (util/util.py:46-59), a
wrapper of ``fluiddyn.io.image.imread``, which hands them to PIL / imageio.  None of
those is installed here, so this oracle restates the published formats for the
kinds found in upstream's image samples: TIFF 6.0 baseline (uncompressed, grayscale,
strips joined by their StripByteCounts), Windows BMP (BITMAPINFOHEADER, 8-bit
palette), PNG (RFC 2083: zlib stream, filters 0-4 reconstructed byte by byte in
plain Python).  Parity with PIL is unpinned (no PIL output exists here to record);
the tests pin the oracle with files of known content written by their own encoder
and, where upstream's image_samples are present, with their headers' sizes.
"""

from __future__ import annotations

import zlib

import numpy as np


def _u(data, pos, n, little):
    return int.from_bytes(data[pos:pos + n], "little" if little else "big")


def decode_tiff(data: bytes) -> np.ndarray:
    little = data[:2] == b"II"
    assert data[:2] in (b"II", b"MM") and _u(data, 2, 2, little) == 42
    ifd = _u(data, 4, 4, little)
    sizes = {1: 1, 3: 2, 4: 4}
    tags = {}
    for k in range(_u(data, ifd, 2, little)):
        e = ifd + 2 + 12 * k
        tag, typ, count = _u(data, e, 2, little), _u(data, e + 2, 2, little), _u(data, e + 4, 4, little)
        if typ not in sizes:  # RATIONAL, ASCII and the like: no tag read here needs them
            continue
        size = sizes[typ]
        pos = e + 8 if size * count <= 4 else _u(data, e + 8, 4, little)
        tags[tag] = [_u(data, pos + size * i, size, little) for i in range(count)]
    width, height, bits = tags[256][0], tags[257][0], tags[258][0]
    assert tags.get(259, [1])[0] == 1 and tags.get(277, [1])[0] == 1
    body = b"".join(data[o:o + c] for o, c in zip(tags[273], tags[279]))
    dt = np.dtype(np.uint8) if bits == 8 else np.dtype("<u2" if little else ">u2")
    img = np.frombuffer(body, dt, count=width * height).reshape(height, width)
    img = img.astype(np.uint8 if bits == 8 else np.uint16)
    if tags.get(262, [1])[0] == 0:  # WhiteIsZero
        img = np.iinfo(img.dtype).max - img
    return img


def decode_bmp(data: bytes) -> np.ndarray:
    assert data[:2] == b"BM"
    off = _u(data, 10, 4, True)
    hsize = _u(data, 14, 4, True)
    width = int.from_bytes(data[18:22], "little", signed=True)
    height = int.from_bytes(data[22:26], "little", signed=True)
    assert _u(data, 28, 2, True) == 8 and _u(data, 30, 4, True) == 0
    ncolors = _u(data, 46, 4, True) or 256
    gray = [data[14 + hsize + 4 * i + 2] for i in range(ncolors)]
    stride = ((width * 8 + 31) // 32) * 4
    rows = [data[off + r * stride:off + r * stride + width] for r in range(abs(height))]
    idx = np.array([list(r) for r in rows], dtype=np.uint8)
    if height > 0:  # bottom-up
        idx = idx[::-1]
    lut = np.zeros(256, np.uint8)
    lut[:ncolors] = gray[:256]
    return lut[idx]


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def decode_png(data: bytes) -> np.ndarray:
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n = _u(data, pos, 4, False)
        kind = data[pos + 4:pos + 8]
        if kind == b"IHDR":
            width, height = _u(data, pos + 8, 4, False), _u(data, pos + 12, 4, False)
            depth, color, interlace = data[pos + 16], data[pos + 17], data[pos + 20]
        elif kind == b"IDAT":
            idat += data[pos + 8:pos + 8 + n]
        pos += 12 + n
    assert color == 0 and depth in (8, 16) and interlace == 0
    bpp = depth // 8
    stride = width * bpp
    raw = zlib.decompress(idat)
    prev = [0] * stride
    out = []
    for r in range(height):
        ftype = raw[r * (stride + 1)]
        line = list(raw[r * (stride + 1) + 1:(r + 1) * (stride + 1)])
        cur = [0] * stride
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[ftype]
            cur[i] = (line[i] + pred) & 0xFF
        out.append(cur)
        prev = cur
    buf = np.array(out, dtype=np.uint8)
    if depth == 8:
        return buf
    return buf.reshape(height, width, 2).astype(np.uint16) @ np.array([256, 1], np.uint16)


def decode(path) -> np.ndarray:
    data = open(path, "rb").read()
    if data[:2] in (b"II", b"MM"):
        return decode_tiff(data)
    if data[:2] == b"BM":
        return decode_bmp(data)
    return decode_png(data)
