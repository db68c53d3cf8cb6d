"""PNG texture ingest for Texture::from_png_file (src/texture.rs:26-45).

The reference decodes with the `png` crate (0.16.8, default options) and then treats the
buffer as tightly packed 8-bit RGBA rows, top row first (`texel_width: 4`); it only
debug-asserts that the file is non-interlaced RGBA8. This reader follows the PNG
specification (ISO/IEC 15948) for exactly that case: chunk walk with CRC-32 checks, IHDR,
concatenated IDAT inflated with zlib, and the five per-row filters (None, Sub, Up, Average,
Paeth). Any other colour type, bit depth or an interlaced file raises ValueError instead of
producing the reference's release-mode garbage.
"""
import struct
import zlib

import numpy as np

_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_BPP = 4  # bytes per pixel of 8-bit RGBA


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter_row(ftype, row, prev):
    """Reconstruct one scanline in place (row and prev are bytearrays of equal length)."""
    n = len(row)
    if ftype == 0:
        return
    if ftype == 1:  # Sub
        for i in range(_BPP, n):
            row[i] = (row[i] + row[i - _BPP]) & 0xFF
    elif ftype == 2:  # Up
        r = (np.frombuffer(bytes(row), np.uint8) + np.frombuffer(bytes(prev), np.uint8)).astype(np.uint8)
        row[:] = r.tobytes()
    elif ftype == 3:  # Average
        for i in range(n):
            left = row[i - _BPP] if i >= _BPP else 0
            row[i] = (row[i] + ((left + prev[i]) >> 1)) & 0xFF
    elif ftype == 4:  # Paeth
        for i in range(n):
            if i >= _BPP:
                row[i] = (row[i] + _paeth(row[i - _BPP], prev[i], prev[i - _BPP])) & 0xFF
            else:
                row[i] = (row[i] + prev[i]) & 0xFF
    else:
        raise ValueError(f"PNG: unknown filter type {ftype}")


def decode_png_rgba8(data: bytes) -> np.ndarray:
    """Decode an 8-bit RGBA, non-interlaced PNG to a (height, width, 4) uint8 array."""
    if data[:8] != _SIGNATURE:
        raise ValueError("PNG: bad signature")
    pos, ihdr, idat, seen_end = 8, None, [], False
    while pos + 12 <= len(data):
        length, ctype = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        (crc,) = struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])
        if len(body) != length or zlib.crc32(ctype + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"PNG: corrupt {ctype!r} chunk")
        pos += 12 + length
        if ctype == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            seen_end = True
            break
    if ihdr is None or not idat or not seen_end:
        raise ValueError("PNG: missing IHDR, IDAT or IEND")
    w, h, depth, color, comp, filt, interlace = ihdr
    if depth != 8 or color != 6:
        raise ValueError(f"PNG: only 8-bit RGBA is supported (bit depth {depth}, colour type {color})")
    if interlace != 0:
        raise ValueError("PNG: interlaced images are not supported")
    if comp != 0 or filt != 0 or w == 0 or h == 0:
        raise ValueError("PNG: unsupported compression/filter method or empty image")
    raw = zlib.decompress(b"".join(idat))
    stride = w * _BPP
    if len(raw) != h * (stride + 1):
        raise ValueError("PNG: image data has the wrong length")
    out = bytearray(h * stride)
    prev = bytearray(stride)
    for y in range(h):
        base = y * (stride + 1)
        row = bytearray(raw[base + 1:base + 1 + stride])
        _unfilter_row(raw[base], row, prev)
        out[y * stride:(y + 1) * stride] = row
        prev = row
    return np.frombuffer(bytes(out), np.uint8).reshape(h, w, 4).copy()


def read_png_rgba8(path) -> np.ndarray:
    """Texture::from_png_file's decode step: the file at `path` as (height, width, 4) RGBA8."""
    with open(path, "rb") as f:
        return decode_png_rgba8(f.read())


def encode_png_rgba8(img: np.ndarray, filters=(0,), level=6) -> bytes:
    """Write (height, width, 4) uint8 RGBA as a PNG; row y uses filter filters[y % len(filters)].

    Used to store rendered frames and to exercise every filter type of the decoder.
    """
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w, ch = img.shape
    if ch != 4:
        raise ValueError("encode_png_rgba8 expects (height, width, 4)")
    stride = w * _BPP
    rows = img.reshape(h, stride).astype(np.int32)
    raw = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ftype = filters[y % len(filters)]
        cur = rows[y]
        left = np.concatenate([np.zeros(_BPP, np.int32), cur[:-_BPP]])
        upleft = np.concatenate([np.zeros(_BPP, np.int32), prev[:-_BPP]])
        if ftype == 0:
            f = cur
        elif ftype == 1:
            f = cur - left
        elif ftype == 2:
            f = cur - prev
        elif ftype == 3:
            f = cur - ((left + prev) >> 1)
        elif ftype == 4:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            f = cur - pred
        else:
            raise ValueError(f"unknown filter {ftype}")
        raw.append(ftype)
        raw += (f & 0xFF).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    return (_SIGNATURE + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(raw), level)) + chunk(b"IEND", b""))


def argb_to_rgba8(argb: np.ndarray) -> np.ndarray:
    """Resolved ARGB u32 frame (Color::to_argb layout, src/color.rs:15-20) → (H, W, 4) RGBA8."""
    a = np.asarray(argb, dtype=np.uint32)
    return np.stack([(a >> 16) & 0xFF, (a >> 8) & 0xFF, a & 0xFF, a >> 24], axis=-1).astype(np.uint8)
