"""Headless image output (yh_write_png, yh_write_hdr): the files are read back here and
checked against the conversion RendererCore::saveImage gets from GL and stb
(src/RendererCore.cpp:608-646): rows flipped (the file's first row is the frame's last),
8-bit channels round(clamp(c, 0, 1) * 255), RGBE within its 8-bit mantissa."""
import struct
import zlib

import numpy as np

from yune_gb300.core import write_hdr, write_png


def _frame(h=37, w=53, seed=2):
    rng = np.random.default_rng(seed)
    f = rng.uniform(-0.2, 1.3, (h, w, 4)).astype(np.float32)
    f[0, 0, 0] = np.nan
    f[1, 1, :3] = [0.5 / 255, 1.5 / 255, 254.5 / 255]   # halfway values
    return f


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc, typ
        chunks.setdefault(typ, b"")
        chunks[typ] += body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (depth, ctype) == (8, 2) and b"IEND" in chunks
    raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(h, w * 3 + 1)
    assert (raw[:, 0] == 0).all()   # filter type None
    return raw[:, 1:].reshape(h, w, 3)


def test_png_pixels(tmp_path):
    f = _frame()
    p = tmp_path / "f.png"
    write_png(p, f)
    got = _read_png(p)
    c = np.nan_to_num(f[::-1, :, :3], nan=0.0)
    want = np.floor(np.clip(c, 0.0, 1.0).astype(np.float32) * np.float32(255.0) + np.float32(0.5))
    # round half away from zero on exact halves, as lround does
    assert np.array_equal(got, want.astype(np.uint8))


def test_png_large_frame_spans_several_deflate_blocks(tmp_path):
    f = np.zeros((300, 400, 4), np.float32)
    f[..., 0] = np.linspace(0, 1, 400)[None, :]
    p = tmp_path / "big.png"
    write_png(p, f)
    got = _read_png(p)
    assert got.shape == (300, 400, 3) and got[0, -1, 0] == 255 and got[0, 0, 0] == 0


def test_hdr_pixels(tmp_path):
    f = np.abs(_frame()) * np.float32(40.0)
    f[2, 3, :3] = 0.0
    p = tmp_path / "f.hdr"
    write_hdr(p, f)
    data = open(p, "rb").read()
    head, body = data.split(b"\n\n", 1)
    assert head.startswith(b"#?RADIANCE") and b"FORMAT=32-bit_rle_rgbe" in head
    res, px = body.split(b"\n", 1)
    h, w = f.shape[:2]
    assert res == b"-Y %d +X %d" % (h, w)
    rgbe = np.frombuffer(px, np.uint8).reshape(h, w, 4).astype(np.float64)
    dec = np.where(rgbe[..., 3:] > 0, rgbe[..., :3] * np.ldexp(1.0, (rgbe[..., 3:] - 136).astype(int)), 0.0)
    want = np.nan_to_num(f[::-1, :, :3].astype(np.float64), nan=0.0)
    peak = want.max(axis=-1, keepdims=True)
    assert (np.abs(dec - want) <= peak * 2.0 ** -7 + 1e-30).all()
    assert (rgbe[h - 1 - 2, 3] == 0).all()   # an all-zero pixel stays zero
