"""Image files of PIV series: ``imread`` (drop-in for ``fluidimage.util.imread``,
util/util.py:46-59) and ``imread_device``, the decode into HBM.

Formats are those of upstream's image samples and cameras: uncompressed grayscale
TIFF (8 or 16 bits, one or many strips, either byte order, BlackIsZero or
WhiteIsZero; the first page), 8-bit BMP with a gray palette (bottom-up or top-down
rows), grayscale PNG of 8 or 16 bits (the five row filters, not interlaced).  Other
kinds (colour, compressed TIFF, tiles, interlaced PNG) raise ``NotImplementedError``.
Images come back as uint8 or uint16 of shape (height, width).

The host parses the container (``read_payload``); the pixel payload crosses to the
device in one copy and ``fi_image_unpack`` writes the image there (strips, row
order, padding, byte order and palette are resolved in the kernel).  A PNG's DEFLATE
stream is inflated with zlib and its scanlines are reconstructed by the library's
native ``fi_png_unfilter`` before the copy: both steps are sequential by
construction.
"""

from __future__ import annotations

import ctypes as C
import struct
import zlib
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib as L

__all__ = ["Payload", "read_payload", "imread", "imread_device"]


@dataclass
class Payload:
    """Pixel payload of an image file: row ``r`` of the image is ``width *
    bytes_per_sample`` bytes of ``raw`` from ``row_offsets[r]``."""

    fmt: str
    height: int
    width: int
    bytes_per_sample: int
    big_endian: bool
    raw: np.ndarray  # uint8
    row_offsets: np.ndarray  # int64, one per row
    lut: np.ndarray | None = None  # uint8[256] for 1-byte samples
    invert: bool = False

    @property
    def dtype(self):
        return np.uint8 if self.bytes_per_sample == 1 else np.uint16

    def check(self):
        row_bytes = self.width * self.bytes_per_sample
        off = self.row_offsets
        if off.size != self.height or (off.size and (off.min() < 0 or
                                                      off.max() + row_bytes > self.raw.size)):
            raise ValueError(f"{self.fmt} file truncated: its rows run past the data")
        return self


# ---------------------------------------------------------------------------- TIFF
_TIFF_TYPES = {1: ("B", 1), 3: ("H", 2), 4: ("I", 4), 16: ("Q", 8)}


def _tiff_payload(data: bytes) -> Payload:
    """TIFF 6.0 baseline, uncompressed grayscale (first image file directory)."""
    if data[:2] == b"II":
        e = "<"
    elif data[:2] == b"MM":
        e = ">"
    else:
        raise ValueError("not a TIFF file")
    (magic,) = struct.unpack(e + "H", data[2:4])
    if magic != 42:
        raise NotImplementedError(f"TIFF variant {magic} (BigTIFF) is not supported")
    (ifd,) = struct.unpack(e + "I", data[4:8])
    (nent,) = struct.unpack(e + "H", data[ifd:ifd + 2])
    tags = {}
    for k in range(nent):
        tag, typ, count, raw = struct.unpack(e + "HHI4s", data[ifd + 2 + 12 * k:ifd + 14 + 12 * k])
        if typ not in _TIFF_TYPES:
            continue
        fmt, size = _TIFF_TYPES[typ]
        if size * count <= 4:
            vals = struct.unpack(e + fmt * count, raw[:size * count])
        else:
            (off,) = struct.unpack(e + "I", raw)
            vals = struct.unpack(e + fmt * count, data[off:off + size * count])
        tags[tag] = vals
    width, height = tags[256][0], tags[257][0]
    bits = tags.get(258, (1,))
    spp = tags.get(277, (1,))[0]
    compression = tags.get(259, (1,))[0]
    photometric = tags.get(262, (1,))[0]
    sample_format = tags.get(339, (1,))[0]
    if 322 in tags or 324 in tags:
        raise NotImplementedError("tiled TIFF is not supported")
    if compression != 1:
        raise NotImplementedError(f"TIFF compression {compression} is not supported")
    if spp != 1 or photometric not in (0, 1):
        raise NotImplementedError("colour TIFF is not supported (grayscale only)")
    if bits[0] not in (8, 16) or sample_format != 1:
        raise NotImplementedError(f"TIFF samples of {bits[0]} bits (format {sample_format}) "
                                  "are not supported (8 or 16-bit unsigned)")
    bps = bits[0] // 8
    rps = min(tags.get(278, (height,))[0], height)
    strips = np.asarray(tags[273], dtype=np.int64)
    rows = np.arange(height, dtype=np.int64)
    strip = rows // rps
    if strip.max() >= strips.size:
        raise ValueError("TIFF file truncated: fewer strips than rows need")
    offsets = strips[strip] + (rows - strip * rps) * (width * bps)
    return Payload("tiff", height, width, bps, e == ">", np.frombuffer(data, np.uint8),
                   offsets, None, photometric == 0)


# ----------------------------------------------------------------------------- BMP
def _bmp_payload(data: bytes) -> Payload:
    """Windows bitmap, uncompressed 8-bit with a gray palette."""
    if data[:2] != b"BM":
        raise ValueError("not a BMP file")
    (pix,) = struct.unpack("<I", data[10:14])
    (hsize,) = struct.unpack("<I", data[14:18])
    if hsize < 40:
        raise NotImplementedError("OS/2 bitmaps are not supported")
    width, height, _planes, bitcount, compression = struct.unpack("<iiHHI", data[18:34])
    (ncolors,) = struct.unpack("<I", data[46:50])
    if compression != 0:
        raise NotImplementedError(f"BMP compression {compression} is not supported")
    if bitcount != 8:
        raise NotImplementedError(f"BMP of {bitcount} bits per pixel is not supported "
                                  "(8-bit gray palette only)")
    ncolors = ncolors or 256
    pal = np.frombuffer(data, np.uint8, count=4 * ncolors, offset=14 + hsize).reshape(-1, 4)
    if not (np.array_equal(pal[:, 0], pal[:, 1]) and np.array_equal(pal[:, 1], pal[:, 2])):
        raise NotImplementedError("BMP with a colour palette is not supported")
    lut = np.zeros(256, np.uint8)
    lut[:ncolors] = pal[:256, 2]
    top_down = height < 0
    height = abs(height)
    stride = (width * bitcount + 31) // 32 * 4
    rows = np.arange(height, dtype=np.int64)
    offsets = pix + (rows if top_down else height - 1 - rows) * stride
    return Payload("bmp", height, width, 1, False, np.frombuffer(data, np.uint8), offsets, lut)


# ----------------------------------------------------------------------------- PNG
_PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"


def _png_payload(data: bytes) -> Payload:
    """PNG (RFC 2083), grayscale of 8 or 16 bits, not interlaced."""
    if data[:8] != _PNG_SIGNATURE:
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos + 8 <= len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        (crc,) = struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])
        if zlib.crc32(ctype + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"PNG chunk {ctype!r}: CRC mismatch")
        if ctype == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
        pos += 12 + length
    if hdr is None:
        raise ValueError("PNG file without IHDR")
    width, height, depth, color, _comp, _filt, interlace = hdr
    if color != 0:
        raise NotImplementedError(f"PNG colour type {color} is not supported (grayscale only)")
    if depth not in (8, 16):
        raise NotImplementedError(f"PNG bit depth {depth} is not supported (8 or 16)")
    if interlace != 0:
        raise NotImplementedError("interlaced PNG is not supported")
    bps = depth // 8
    row_bytes = width * bps
    filtered = zlib.decompress(b"".join(idat))
    if len(filtered) < height * (row_bytes + 1):
        raise ValueError("PNG file truncated: fewer scanlines than rows")
    out = np.empty(height * row_bytes, np.uint8)
    src = np.frombuffer(filtered, np.uint8)
    L.check(L.load().fi_png_unfilter(src.ctypes.data_as(C.c_void_p), height, row_bytes, bps,
                                     out.ctypes.data_as(C.c_void_p)), "fi_png_unfilter")
    offsets = np.arange(height, dtype=np.int64) * row_bytes
    return Payload("png", height, width, bps, True, out, offsets)


_READERS = {b"II": _tiff_payload, b"MM": _tiff_payload, b"BM": _bmp_payload,
            _PNG_SIGNATURE[:2]: _png_payload}


def read_payload(path) -> Payload:
    """Parse the image file ``path`` into its pixel payload (host)."""
    path = str(path) if isinstance(path, Path) else path
    try:
        with open(path, "rb") as f:
            data = f.read()
    except OSError as error:  # upstream re-raises with the path as the message
        raise type(error)(path) from error
    reader = _READERS.get(data[:2])
    if reader is None:
        raise NotImplementedError(f"{path}: image format not supported (TIFF, BMP, PNG)")
    try:
        return reader(data).check()
    except (KeyError, IndexError, struct.error, zlib.error) as error:
        raise ValueError(f"{path}: malformed or truncated image file ({error!r})") from error


def imread(path) -> np.ndarray:
    """The image of ``path`` as a (height, width) uint8 or uint16 numpy array (host)."""
    p = read_payload(path)
    row_bytes = p.width * p.bytes_per_sample
    idx = p.row_offsets[:, None] + np.arange(row_bytes, dtype=np.int64)[None, :]
    rows = p.raw[idx]
    if p.bytes_per_sample == 1:
        img = p.lut[rows] if p.lut is not None else rows
        return (255 - img) if p.invert else np.ascontiguousarray(img)
    img = rows.view(">u2" if p.big_endian else "<u2").astype(np.uint16)
    return (65535 - img) if p.invert else img


def imread_device(path, device="cuda", stream=None):
    """The image of ``path`` decoded into a (height, width) torch tensor on ``device``:
    one host-to-device copy of the pixel payload (with the row offsets and the
    palette), then ``fi_image_unpack`` on the stream.  8-bit images are uint8; 16-bit
    images are uint16 values kept bit for bit in an int16 tensor, the device image
    type of ``WorkPIV.calcul_device`` (``.view(torch.uint16)`` reads them as such)."""
    import torch

    p = read_payload(path)
    lib = L.load()
    nraw = -(-p.raw.size // 16) * 16
    nlut = 256 if p.lut is not None else 0
    host = torch.empty(nraw + 8 * p.height + nlut, dtype=torch.uint8, pin_memory=True)
    h = host.numpy()
    h[:p.raw.size] = p.raw
    h[nraw:nraw + 8 * p.height] = p.row_offsets.view(np.uint8)
    if nlut:
        h[nraw + 8 * p.height:] = p.lut
    dev = torch.device(device)
    strm = stream if stream is not None else torch.cuda.current_stream(dev)
    out = torch.empty((p.height, p.width),
                      dtype=torch.uint8 if p.bytes_per_sample == 1 else torch.int16, device=dev)
    with torch.cuda.stream(strm):
        buf = torch.empty_like(host, device=dev)
        buf.copy_(host, non_blocking=True)
        base = buf.data_ptr()
        L.check(lib.fi_image_unpack(base, p.raw.size, base + nraw, p.height, p.width,
                                    p.bytes_per_sample, int(p.big_endian),
                                    base + nraw + 8 * p.height if nlut else None,
                                    int(p.invert), out.data_ptr(), None, strm.cuda_stream),
                "fi_image_unpack")
    # like upstream's imread, the call returns with the image ready (the pinned staging
    # buffer and the device payload are released after the kernel)
    strm.synchronize()
    return out
