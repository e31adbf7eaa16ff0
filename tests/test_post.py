"""The output path without a GPU: the oracle's restatement of the
post-processors against the reference's own (compiled from its sources),
and the PNG / HDR writers of the C ABI read back with a project-written
decoder (zlib for the PNG stream)."""
import struct
import zlib

import numpy as np
import pytest

import oracle
from tracer_gb300.native import write_hdr, write_png


def _image(seed, h=9, w=13):
    rng = np.random.default_rng(seed)
    img = np.abs(rng.normal(0, 2, (h, w, 3))).astype(np.float32)
    img[0, 0] = [0.0, 1e-40, 3e38]
    img[0, 1] = [np.inf, np.nan, -1.0]
    return img


@pytest.mark.skipif(not oracle.ref_available(), reason="the reference build (oracle/_ref) is not present")
@pytest.mark.parametrize("which,param", [("aces", 1.0), ("aces", 2.7), ("aces", -1.0), ("gamma", 1 / 2.2),
                                         ("gamma", 2.2), ("gamma", 0.0)])
def test_post_processors_restatement_equals_the_reference(which, param):
    img = _image(1)
    a = oracle.post_process("port", img, which, param)
    r = oracle.post_process("reference", img, which, param)
    assert np.array_equal(a.view(np.uint32), r.view(np.uint32))


def test_rgb8_rule():
    img = np.array([[[0.0, 1.0, 0.5], [2.0, -1.0, np.nan], [1e-9, 0.999, 3e38]]], np.float32)
    got = oracle.post_rgb8(img)
    want = [[int(min(255, max(0, np.trunc(np.float32(np.power(np.float32(c), np.float32(1 / 2.2))) * 255))))
             if np.isfinite(c) and c >= 0 else 0 for c in px] for px in img[0]]
    assert got[0].tolist() == want


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        chunks.append((typ, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 2, 0, 0, 0)
    raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 3)


def _read_hdr(path):
    data = open(path, "rb").read()
    head, rest = data.split(b"\n\n", 1)
    assert head.startswith(b"#?RADIANCE") and b"FORMAT=32-bit_rle_rgbe" in head
    dims, body = rest.split(b"\n", 1)
    _, h, _, w = dims.split()
    h, w = int(h), int(w)
    out = np.zeros((h, w, 4), np.uint8)
    pos = 0
    for y in range(h):
        if 8 <= w <= 32767:
            assert body[pos:pos + 2] == b"\x02\x02" and (body[pos + 2] << 8 | body[pos + 3]) == w
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = body[pos]
                    pos += 1
                    assert 0 < n <= 128  # literal runs only
                    out[y, x:x + n, c] = np.frombuffer(body[pos:pos + n], np.uint8)
                    pos += n
                    x += n
        else:
            out[y] = np.frombuffer(body[pos:pos + 4 * w], np.uint8).reshape(w, 4)
            pos += 4 * w
    assert pos == len(body)
    return out


@pytest.mark.parametrize("h,w", [(1, 1), (7, 13), (300, 400)])
def test_png_writer(tmp_path, h, w):
    rgb8 = np.random.default_rng(h * w).integers(0, 256, (h, w, 3), dtype=np.uint8)
    p = tmp_path / "img.png"
    write_png(str(p), rgb8)
    assert np.array_equal(_read_png(str(p)), rgb8)


@pytest.mark.parametrize("h,w", [(3, 5), (6, 8), (5, 300)])
def test_hdr_writer(tmp_path, h, w):
    img = np.abs(np.random.default_rng(w).normal(0, 3, (h, w, 3))).astype(np.float32)
    rgbe = oracle.post_rgbe(img)
    p = tmp_path / "img.hdr"
    write_hdr(str(p), rgbe)
    got = _read_hdr(str(p))
    assert np.array_equal(got, rgbe)
    # RGBE keeps 8 significant bits of the largest channel
    m = img.max(-1)
    dec = got[..., :3].astype(np.float64) * np.ldexp(1.0, got[..., 3].astype(np.int64) - 136)[..., None]
    assert np.all(np.abs(dec.max(-1) - m) <= m * 2 ** -7)
