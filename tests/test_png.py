"""CPU tests of the PNG heightmap decoder (wave_tool_gb300.png), the stb
replacement for src/render-engine.cpp:1308-1322: images written here with
every colour type, bit depth, scanline filter and both interlace modes decode
to the 8-bit samples stb_image would give; the reference's own heightmap
asset decodes like an independent decoder (when the reference checkout is on
this machine)."""
from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np
import pytest

ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_rows(samples, depth):
    """(h, w, c) integer samples -> (h, row_bytes) uint8 scanline bytes."""
    h, w, c = samples.shape
    if depth == 8:
        return samples.reshape(h, w * c).astype(np.uint8)
    if depth == 16:
        s = samples.reshape(h, w * c).astype(np.uint16)
        return np.stack([s >> 8, s & 255], axis=2).reshape(h, 2 * w * c).astype(np.uint8)
    bits = ((samples.reshape(h, w * c, 1) >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8)
    return np.packbits(bits.reshape(h, w * c * depth), axis=1)


def _filter_rows(rows, bpp, rng):
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for r in range(rows.shape[0]):
        x = rows[r].astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), x[:-bpp]]) if len(x) > bpp else np.zeros_like(x)
        a = a[:len(x)]
        b = prev
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])[:len(x)]
        f = int(rng.integers(0, 5))
        if f == 0:
            y = x
        elif f == 1:
            y = x - a
        elif f == 2:
            y = x - b
        elif f == 3:
            y = x - (a + b) // 2
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            y = x - np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        out += bytes([f]) + (y & 255).astype(np.uint8).tobytes()
        prev = x
    return bytes(out)


def encode(samples, depth, ctype, rng, interlace=0, palette=None, trns=None):
    h, w, c = samples.shape
    bpp = max(1, depth * c // 8)
    if interlace:
        raw = b""
        for x0, y0, dx, dy in ADAM7:
            sub = samples[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += _filter_rows(_pack_rows(sub, depth), bpp, rng)
    else:
        raw = _filter_rows(_pack_rows(samples, depth), bpp, rng)
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if palette is not None:
        out += _chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        out += _chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    z = zlib.compress(raw)
    out += _chunk(b"IDAT", z[:len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:])  # split across two IDATs
    return out + _chunk(b"IEND", b"")


def stb_8bit(samples, depth, ctype):
    """What stb_image hands back, per channel, for these stored samples."""
    if depth == 16:
        return (samples >> 8).astype(np.uint8)
    if depth < 8 and ctype == 0:
        return (samples * (255 // ((1 << depth) - 1))).astype(np.uint8)
    return samples.astype(np.uint8)


@pytest.mark.parametrize("interlace", [0, 1])
def test_decode_every_format(wt, interlace):
    from wave_tool_gb300 import png
    rng = np.random.default_rng(5 + interlace)
    cases = [(0, d) for d in (1, 2, 4, 8, 16)] + [(2, 8), (2, 16), (4, 8), (4, 16), (6, 8), (6, 16)] + \
            [(3, d) for d in (1, 2, 4, 8)]
    for ctype, depth in cases:
        for (h, w) in ((1, 1), (7, 13), (33, 17)):
            c = CHANNELS[ctype]
            if ctype == 3:
                n_pal = min(1 << depth, 40)
                pal = rng.integers(0, 256, (n_pal, 3))
                idx = rng.integers(0, n_pal, (h, w, 1))
                trns = rng.integers(0, 256, n_pal // 2) if depth >= 2 else None
                data = encode(idx, depth, ctype, rng, interlace, palette=pal, trns=trns)
                want = pal[idx[..., 0]].astype(np.uint8)
                if trns is not None:
                    alpha = np.full(n_pal, 255)
                    alpha[:len(trns)] = trns
                    want = np.concatenate([want, alpha[idx[..., 0]][..., None].astype(np.uint8)], axis=2)
            else:
                s = rng.integers(0, 1 << depth, (h, w, c))
                data = encode(s, depth, ctype, rng, interlace)
                want = stb_8bit(s, depth, ctype)
            got = png.decode(data)
            assert got.dtype == np.uint8 and got.shape == want.shape, (ctype, depth, h, w)
            assert np.array_equal(got, want), (ctype, depth, h, w, interlace)


def test_decode_rejects_corrupt_files(wt):
    from wave_tool_gb300 import png
    rng = np.random.default_rng(9)
    good = encode(rng.integers(0, 256, (4, 4, 1)), 8, 0, rng)
    with pytest.raises(png.PngError):
        png.decode(b"GIF89a" + good[6:])
    bad_crc = bytearray(good)
    bad_crc[30] ^= 0xFF  # inside IHDR's body
    with pytest.raises(png.PngError):
        png.decode(bytes(bad_crc))
    with pytest.raises(png.PngError):  # palette image without PLTE
        png.decode(encode(rng.integers(0, 4, (4, 4, 1)), 2, 3, rng))


def test_reference_asset_decodes_like_an_independent_decoder(wt):
    from wave_tool_gb300 import png
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_oracle import REF_ASSET, decode_grey_png
    if not REF_ASSET.exists():
        pytest.skip("reference checkout not on this machine")
    img = png.decode(REF_ASSET.read_bytes())
    assert img.shape[2] == 1
    assert np.array_equal(img[..., 0].astype(np.int32), decode_grey_png(REF_ASSET))
