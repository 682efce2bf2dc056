"""PNG decoding for the init-from-image path (coupledwateranimation_gb300/images.py)
and the oracle's InitFromImage restatement, on CPU."""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from coupledwateranimation_gb300 import images

GOLDEN = Path(__file__).resolve().parent / "golden" / "init_textures.npz"


def _png(w, h, ctype, rows: list[bytes], plte: bytes | None = None, trns: bytes | None = None) -> bytes:
    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    raw = b"".join(b"\x00" + r for r in rows)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if plte is not None:
        out += chunk(b"PLTE", plte)
    if trns is not None:
        out += chunk(b"tRNS", trns)
    return out + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b"")


@pytest.mark.parametrize("ftype", [0, 1, 2, 3, 4])
def test_png_roundtrip_every_filter(ftype):
    rng = np.random.default_rng(ftype)
    img = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    assert np.array_equal(images.decode_png(images.encode_png(img, ftype)), img)


def test_png_grey_rgb_palette():
    g = images.decode_png(_png(3, 2, 0, [bytes([0, 128, 255]), bytes([1, 2, 3])]))
    assert g.shape == (2, 3, 4) and g[0, 1].tolist() == [128, 128, 128, 255]
    rgb = images.decode_png(_png(2, 1, 2, [bytes([10, 20, 30, 40, 50, 60])]))
    assert rgb[0, 1].tolist() == [40, 50, 60, 255]
    pal = images.decode_png(_png(2, 1, 3, [bytes([1, 0])], plte=bytes([9, 8, 7, 6, 5, 4]), trns=bytes([17])))
    assert pal[0, 0].tolist() == [6, 5, 4, 255] and pal[0, 1].tolist() == [9, 8, 7, 17]


def test_png_rejects_unsupported():
    with pytest.raises(ValueError):
        images.decode_png(b"not a png")


def test_gl_rows_flips():
    img = np.arange(2 * 3 * 4, dtype=np.uint8).reshape(2, 3, 4)
    assert np.array_equal(images.gl_rows(img)[0], img[1])


def test_init_texture_fixtures():
    d = np.load(GOLDEN)
    assert set(d.files) == {"splash", "wake", "breaking_wave"}
    for k in d.files:
        a = d[k]
        assert a.shape == (64, 64, 4) and a.dtype == np.uint8
        assert np.array_equal(images.decode_png(images.encode_png(a, 4)), a)


def test_oracle_from_image_restatement(orc):
    img = images.gl_rows(np.load(GOLDEN)["breaking_wave"])
    for nx, nz in [(64, 64), (16, 8), (100, 70)]:
        got = orc.wave_from_image_f32(nx, nz, img)
        want = np.zeros((nz, nx), np.float32)
        h, w = img.shape[:2]
        for y in range(min(nz, h)):
            for x in range(nx):
                if 2 * x < w:
                    want[y, x] = np.float32(img[y, 2 * x, 0]) / np.float32(255.0)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
