"""PNG reading for wave initialisation images (the reference's init-textures).

A small non-interlaced PNG decoder (bit depth 8; grey, grey+alpha, RGB,
RGBA and palette images) built on zlib.  It exists so a host program can
hand the reference's InitFromImage textures to cwa_wave_init_from_image
without an imaging library.

The reference's loader (CoupledWaterAnimation/LoadTexture.cpp:5-32) reads the
bitmap bottom-up, so texture row 0 is the image's bottom row; `gl_rows`
makes the same flip.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), np.uint8)
    prev = bytearray(stride)
    pos = 0
    for y in range(h):
        ftype = raw[pos]
        line = bytearray(raw[pos + 1:pos + 1 + stride])
        pos += 1 + stride
        if ftype == 1:
            for i in range(bpp, stride):
                line[i] = (line[i] + line[i - bpp]) & 0xFF
        elif ftype == 2:
            for i in range(stride):
                line[i] = (line[i] + prev[i]) & 0xFF
        elif ftype == 3:
            for i in range(stride):
                left = line[i - bpp] if i >= bpp else 0
                line[i] = (line[i] + ((left + prev[i]) >> 1)) & 0xFF
        elif ftype == 4:
            for i in range(stride):
                left = line[i - bpp] if i >= bpp else 0
                up_left = prev[i - bpp] if i >= bpp else 0
                line[i] = (line[i] + _paeth(left, prev[i], up_left)) & 0xFF
        elif ftype != 0:
            raise ValueError(f"bad PNG filter type {ftype}")
        out[y] = np.frombuffer(bytes(line), np.uint8)
        prev = line
    return out


def decode_png(data: bytes) -> np.ndarray:
    """PNG bytes -> (h, w, 4) uint8 RGBA, row 0 = the image's top row."""
    if data[:8] != _SIG:
        raise ValueError("not a PNG file")
    pos, idat, palette, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if w is None or depth != 8 or interlace != 0 or ctype not in _CHANNELS:
        raise ValueError("only non-interlaced 8-bit grey/RGB/RGBA/palette PNGs are supported")
    ch = _CHANNELS[ctype]
    px = _unfilter(zlib.decompress(b"".join(idat)), h, w * ch, ch).reshape(h, w, ch)
    out = np.empty((h, w, 4), np.uint8)
    if ctype == 0:
        out[..., :3] = px[..., :1]
        out[..., 3] = 255
    elif ctype == 4:
        out[..., :3] = px[..., :1]
        out[..., 3] = px[..., 1]
    elif ctype == 2:
        out[..., :3] = px
        out[..., 3] = 255
    elif ctype == 6:
        out[:] = px
    else:  # palette
        if palette is None:
            raise ValueError("palette PNG without PLTE")
        idx = px[..., 0]
        out[..., :3] = palette[idx]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        out[..., 3] = alpha[idx]
    return out


def read_png(path) -> np.ndarray:
    with open(path, "rb") as f:
        return decode_png(f.read())


def gl_rows(img: np.ndarray) -> np.ndarray:
    """Bottom row first, as the reference's bitmap loader uploads textures."""
    return np.ascontiguousarray(img[::-1])


def encode_png(rgba: np.ndarray, filter_type: int = 0) -> bytes:
    """(h, w, 4) uint8 -> PNG bytes, every row with one filter type (0-4)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    rows = img.reshape(h, w * 4).astype(np.int32)
    raw = bytearray()
    prev = np.zeros(w * 4, np.int32)
    for y in range(h):
        line = rows[y]
        left = np.concatenate([np.zeros(4, np.int32), line[:-4]])
        up_left = np.concatenate([np.zeros(4, np.int32), prev[:-4]])
        if filter_type == 0:
            f = line
        elif filter_type == 1:
            f = line - left
        elif filter_type == 2:
            f = line - prev
        elif filter_type == 3:
            f = line - ((left + prev) >> 1)
        elif filter_type == 4:
            pred = np.array([_paeth(int(a), int(b), int(c)) for a, b, c in zip(left, prev, up_left)], np.int32)
            f = line - pred
        else:
            raise ValueError("filter type must be 0-4")
        raw.append(filter_type)
        raw += (f & 0xFF).astype(np.uint8).tobytes()
        prev = line

    def chunk(kind: bytes, body: bytes) -> bytes:
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b""))
