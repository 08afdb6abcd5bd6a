"""Writers of small TIFF, BMP and PNG files of known content for the image decode
tests (written from the format specifications; TIFF 6.0, BMP BITMAPINFOHEADER,
PNG RFC 2083)."""

from __future__ import annotations

import struct
import zlib

import numpy as np


def tiff_bytes(img, big_endian=False, rows_per_strip=None, white_is_zero=False):
    """Uncompressed grayscale TIFF of a uint8 / uint16 image (strips after the IFD)."""
    e = ">" if big_endian else "<"
    h, w = img.shape
    bits = 8 * img.dtype.itemsize
    stored = (np.iinfo(img.dtype).max - img) if white_is_zero else img
    body = stored.astype(stored.dtype.newbyteorder(e)).tobytes()
    rps = rows_per_strip or h
    nstrips = -(-h // rps)
    row_bytes = w * img.dtype.itemsize
    counts = [min(rps, h - s * rps) * row_bytes for s in range(nstrips)]
    entries = 10
    ifd = 8
    extra = ifd + 2 + 12 * entries + 4  # strip offset / count arrays after the IFD
    arrays = extra
    data0 = arrays + (8 * nstrips if nstrips > 1 else 0)
    offsets = [data0 + sum(counts[:s]) for s in range(nstrips)]

    def entry(tag, typ, vals):
        fmt = {3: "H", 4: "I"}[typ]
        size = {3: 2, 4: 4}[typ]
        if len(vals) * size <= 4:
            v = struct.pack(e + fmt * len(vals), *vals).ljust(4, b"\0")
            return struct.pack(e + "HHI", tag, typ, len(vals)) + v
        return struct.pack(e + "HHII", tag, typ, len(vals), vals[0])

    ents = [entry(256, 4, [w]), entry(257, 4, [h]), entry(258, 3, [bits]),
            entry(259, 3, [1]), entry(262, 3, [0 if white_is_zero else 1])]
    if nstrips > 1:
        ents.append(struct.pack(e + "HHII", 273, 4, nstrips, arrays))
    else:
        ents.append(entry(273, 4, offsets))
    ents += [entry(277, 3, [1]), entry(278, 4, [rps])]
    if nstrips > 1:
        ents.append(struct.pack(e + "HHII", 279, 4, nstrips, arrays + 4 * nstrips))
    else:
        ents.append(entry(279, 4, counts))
    ents.append(entry(284, 3, [1]))
    assert len(ents) == entries
    out = (b"II" if not big_endian else b"MM") + struct.pack(e + "HI", 42, ifd)
    out += struct.pack(e + "H", entries) + b"".join(ents) + struct.pack(e + "I", 0)
    if nstrips > 1:
        out += struct.pack(e + "I" * nstrips, *offsets) + struct.pack(e + "I" * nstrips, *counts)
    assert len(out) == data0
    return out + body


def bmp_bytes(img, top_down=False, palette=None):
    """8-bit BMP of the palette indices ``img`` with a gray palette (default identity)."""
    h, w = img.shape
    pal = np.arange(256, dtype=np.uint8) if palette is None else np.asarray(palette, np.uint8)
    stride = (w + 3) // 4 * 4
    rows = img if top_down else img[::-1]
    pix = b"".join(r.tobytes().ljust(stride, b"\0") for r in rows)
    paletted = b"".join(bytes((v, v, v, 0)) for v in pal)
    off = 14 + 40 + len(paletted)
    head = b"BM" + struct.pack("<IHHI", off + len(pix), 0, 0, off)
    info = struct.pack("<IiiHHIIiiII", 40, w, -h if top_down else h, 1, 8, 0, len(pix),
                       2835, 2835, len(pal), 0)
    return head + info + paletted + pix


def _chunk(kind, body):
    return (struct.pack(">I", len(body)) + kind + body +
            struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF))


def png_bytes(img, filters=(0, 1, 2, 3, 4), color=0):
    """Grayscale PNG of a uint8 / uint16 image, row r filtered with filters[r % len]."""
    h, w = img.shape
    bpp = img.dtype.itemsize
    data = img.astype(img.dtype.newbyteorder(">")).tobytes()
    stride = w * bpp
    out = bytearray()
    prev = bytes(stride)
    for r in range(h):
        cur = data[r * stride:(r + 1) * stride]
        ft = filters[r % len(filters)]
        out.append(ft)
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 0:
                pred = 0
            elif ft == 1:
                pred = a
            elif ft == 2:
                pred = b
            elif ft == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out.append((cur[i] - pred) & 0xFF)
        prev = cur
    ihdr = struct.pack(">IIBBBBB", w, h, 8 * bpp, color, 0, 0, 0)
    z = zlib.compress(bytes(out), 6)
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", z[:len(z) // 2]) +
            _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b""))


def cases(seed=5):
    """(name, file bytes, expected image) for the decode tests."""
    rng = np.random.default_rng(seed)
    u8 = rng.integers(0, 256, (37, 45), dtype=np.uint8)
    u16 = rng.integers(0, 65536, (29, 51), dtype=np.uint16)
    pal = (255 - np.arange(256)).astype(np.uint8)
    return [
        ("tiff_u8_le", tiff_bytes(u8), u8),
        ("tiff_u16_le_strips", tiff_bytes(u16, rows_per_strip=4), u16),
        ("tiff_u16_be_strips", tiff_bytes(u16, big_endian=True, rows_per_strip=7), u16),
        ("tiff_u8_be_white_is_zero", tiff_bytes(u8, big_endian=True, white_is_zero=True), u8),
        ("bmp_bottom_up", bmp_bytes(u8), u8),
        ("bmp_top_down_palette", bmp_bytes(u8, top_down=True, palette=pal), pal[u8]),
        ("png_u8", png_bytes(u8), u8),
        ("png_u16", png_bytes(u16, filters=(4, 3, 2, 1, 0)), u16),
    ]
