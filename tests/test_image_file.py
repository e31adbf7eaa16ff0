"""The reference's image-file helpers (src/utility/image_file.cpp) through the
C++ host API: the Radiance HDR reader on files written here (flat and
run-length scanlines), write/read round trips, create_texture2d_from_file's
format rules and create_texture_from_file on MTL materials."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from tracer_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "image_file.cpp")
TR_ERR_ARG = 1
TR_ERR_UNSUPPORTED = 8


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    so = build.build()
    out = str(tmp_path_factory.mktemp("img") / "image_file")
    libdir = os.path.dirname(so)
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", SRC, f"-L{libdir}",
                    "-ltracer_gb300", f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def _decode(rgbe):
    """RGBE to float per the format's definition: byte * 2^(e - 136), 0 for e = 0."""
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(np.float32(1), e - 136), 0).astype(np.float32)
    return rgbe[..., :3].astype(np.float32) * f[..., None]


def _hdr_bytes(rgbe, rle):
    h, w = rgbe.shape[:2]
    out = bytearray(f"#?RADIANCE\n# test\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n-Y {h} +X {w}\n".encode())
    for y in range(h):
        if not rle:
            out += rgbe[y].tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            comp, x = rgbe[y, :, c], 0
            while x < w:  # runs of equal bytes (>= 3) as runs, the rest as literals
                run = 1
                while x + run < w and run < 127 and comp[x + run] == comp[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, comp[x]])
                    x += run
                    continue
                n = 1
                while x + n < w and n < 128 and not (x + n + 2 < w and comp[x + n] == comp[x + n + 1] == comp[x + n + 2]):
                    n += 1
                out += bytes([n]) + comp[x:x + n].tobytes()
                x += n
    return bytes(out)


def _load(program, path):
    r = subprocess.run([program, "load", str(path)], capture_output=True, text=True)
    lines = r.stdout.splitlines()
    if r.returncode != 0:
        return None, lines
    w, h = (int(v) for v in lines[0].split()[1:])
    px = np.array([[float(v) for v in ln.split()] for ln in lines[1:]], np.float32).reshape(h, w, 3)
    return px, lines


@pytest.mark.parametrize("rle,w,h", [(False, 5, 3), (True, 40, 6), (True, 300, 2)])
def test_load_hdr(program, tmp_path, rle, w, h):
    rng = np.random.default_rng(w)
    rgbe = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    rgbe[..., 3] = rng.integers(100, 160, (h, w))
    rgbe[0, : w // 2] = rgbe[0, 0]  # a run
    rgbe[-1, -1, 3] = 0             # exponent 0: black
    p = tmp_path / "a.hdr"
    p.write_bytes(_hdr_bytes(rgbe, rle))
    px, _ = _load(program, p)
    assert px is not None
    assert np.array_equal(px, _decode(rgbe))


def test_write_then_load_round_trip(program, tmp_path):
    p = tmp_path / "b.hdr"
    subprocess.run([program, "write", str(p), "17", "9"], check=True)
    px, _ = _load(program, p)
    y, x = np.mgrid[0:9, 0:17].astype(np.float32)
    want = np.stack([np.float32(0.01) * x + np.float32(0.5) * y, 3 + x, np.where(x == y, 0, 120.5)], -1)
    # RGBE keeps 8 mantissa bits of the largest channel
    assert np.allclose(px, want, rtol=0, atol=want.max(-1, keepdims=True) / 128)


@pytest.mark.parametrize("name,status", [("missing.png", TR_ERR_ARG), ("missing.jpg", TR_ERR_ARG),
                                         ("x.tga", TR_ERR_ARG), ("x.bmp", TR_ERR_ARG), ("noext", TR_ERR_ARG),
                                         ("missing.hdr", TR_ERR_ARG)])
def test_texture_file_rules(program, tmp_path, name, status):
    """create_texture2d_from_file: .hdr, .png and .jpg/.jpeg read (a missing
    file is an argument error); other extensions -- .tga and .bmp too, which
    the reference's is_float_image rejects -- refused as the reference refuses
    them."""
    r = subprocess.run([program, "tex", str(tmp_path / name)], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith(f"error {status}"), r.stdout


def test_hdr_texture_and_bad_header(program, tmp_path):
    rgbe = np.full((2, 2, 4), 128, np.uint8)
    rgbe[..., 3] = 130  # 0.5 * 4 = 2.0
    (tmp_path / "c.hdr").write_bytes(_hdr_bytes(rgbe, False))
    r = subprocess.run([program, "tex", str(tmp_path / "c.hdr")], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split()[1:] == ["2", "2", "2"]
    (tmp_path / "t.hdr").write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n\0\0\0\0")
    r = subprocess.run([program, "load", str(tmp_path / "t.hdr")], capture_output=True, text=True)
    assert r.returncode == 1 and "xyze" in r.stdout


def test_material_textures(program, tmp_path):
    sky = np.zeros((2, 3, 4), np.uint8)
    sky[..., :3], sky[..., 3] = 128, 129  # 0.5 * 2 = 1.0 everywhere
    (tmp_path / "sky.hdr").write_bytes(_hdr_bytes(sky, False))
    (tmp_path / "s.obj").write_text("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n")
    (tmp_path / "s.mtl").write_text(
        "newmtl wall\nKd 0.7 0.6 0.5\nKs 0.1 0.1 0.1\nNs 20\n"
        "newmtl lamp\nKe 17 12 4\n"
        "newmtl glassy\nKd 0 0 0\nNi 1.5\n"
        "newmtl mapped\nKd 0.5 0.5 0.5\nmap_Kd " + str(tmp_path / "sky.hdr") + "\n")
    r = subprocess.run([program, "mtl", str(tmp_path / "s.obj")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    got = {ln.split()[1]: ln.split() for ln in r.stdout.splitlines()}
    w = got["wall"]
    assert w[3:6] == ["0.7", "0.6", "0.5"] and w[7:10] == ["0.1", "0.1", "0.1"] and w[11] == "20"
    assert w[w.index("emission") + 1] == "0" and w[w.index("glass") + 1] == "0"
    lamp = got["lamp"]
    assert lamp[13:16] == ["17", "12", "4"] and lamp[lamp.index("emission") + 1] == "1"
    g = got["glassy"]
    # ior > 1 makes glass; a black ks becomes 1 and is the transmission colour
    assert g[g.index("glass") + 1] == "1" and g[g.index("kt") + 1] == "1" and g[g.index("ior") + 1] == "1.5"
    m = got["mapped"]
    assert m[3:6] == ["0.5", "0.5", "0.5"]  # the map (1.0) scaled by Kd


def _png(rows, ctype, palette=None, filters=None, level=9):
    """A PNG of 8-bit rows (list of byte arrays, top first), zlib-compressed,
    each row encoded with the given filter type (0-4) as ISO/IEC 15948 defines."""
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    h, w = len(rows), len(rows[0]) // ch
    raw, prev = bytearray(), bytes(len(rows[0]))
    for y, row in enumerate(rows):
        ft = (filters or [0])[y % len(filters or [0])]
        out = bytearray()
        for i, v in enumerate(row):
            a = row[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            if ft == 0:
                pr = 0
            elif ft == 1:
                pr = a
            elif ft == 2:
                pr = b
            elif ft == 3:
                pr = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            out.append((v - pr) & 255)
        raw += bytes([ft]) + out
        prev = bytes(row)

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if palette is not None:
        png += chunk(b"PLTE", bytes(palette))
    # two IDAT chunks, the second one empty-ish: the stream spans chunks
    if level == "fixed":  # fixed Huffman codes only
        c = zlib.compressobj(9, zlib.DEFLATED, 15, 9, zlib.Z_FIXED)
        z = c.compress(bytes(raw)) + c.flush()
    else:
        z = zlib.compress(bytes(raw), level)
    return png + chunk(b"IDAT", z[:len(z) // 2]) + chunk(b"IDAT", z[len(z) // 2:]) + chunk(b"IEND", b"")


def _load_png(program, path):
    r = subprocess.run([program, "png", str(path)], capture_output=True, text=True)
    lines = r.stdout.splitlines()
    if r.returncode != 0:
        return None, lines
    w, h = (int(v) for v in lines[0].split()[1:])
    return np.array([[int(v) for v in ln.split()] for ln in lines[1:]], np.uint8).reshape(h, w, 3), lines


@pytest.mark.parametrize("level", [0, "fixed", 9])
@pytest.mark.parametrize("ctype", [0, 2, 3, 6])
def test_load_png(program, tmp_path, ctype, level):
    """Grey, RGB, palette and RGBA PNGs with every filter type, as stored,
    fixed- and dynamic-Huffman zlib streams; rows come back
    flipped (the file's last row is row 0), grey expanded to RGB, alpha dropped."""
    rng = np.random.default_rng(ctype)
    h, w = 7, 23
    ch = {0: 1, 2: 3, 3: 1, 6: 4}[ctype]
    smooth = (np.add.outer(np.arange(h) * 9, np.arange(w * ch) * 3) % 256).astype(np.uint8)
    data = np.where(rng.random((h, w * ch)) < 0.3, rng.integers(0, 256, (h, w * ch)), smooth).astype(np.uint8)
    palette = rng.integers(0, 256, 3 * 256).astype(np.uint8) if ctype == 3 else None
    p = tmp_path / "a.png"
    p.write_bytes(_png([bytes(r) for r in data], ctype, palette, filters=[0, 1, 2, 3, 4], level=level))
    got, lines = _load_png(program, p)
    assert got is not None, lines
    px = data.reshape(h, w, ch)
    if ctype == 0:
        want = np.repeat(px, 3, axis=2)
    elif ctype == 3:
        want = palette.reshape(256, 3)[px[..., 0]]
    else:
        want = px[..., :3]
    assert np.array_equal(got, want[::-1])


def test_png_refusals(program, tmp_path):
    p = tmp_path / "ga.png"
    p.write_bytes(_png([bytes(8)] * 2, 4))
    r = subprocess.run([program, "png", str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "component" in r.stdout  # grey+alpha, as the reference refuses it
    good = _png([bytes(range(12))] * 3, 2)
    for cut in (30, 2, 3):  # truncated inside the data, and with only part of the last chunk header left
        p = tmp_path / f"bad{cut}.png"
        p.write_bytes(good[:-cut] if cut == 30 else good[:-12] + good[-12:-12 + 8 + cut])
        r = subprocess.run([program, "png", str(p)], capture_output=True, text=True)
        assert r.returncode in (0, 1) and ("error" in r.stdout or r.stdout.startswith("size")), r.stdout
    # image data that inflates past the image's size is refused
    big = bytearray(_png([bytes(12)] * 3, 2))
    z = zlib.compress(bytes(100000))
    idat = struct.pack(">I", len(z)) + b"IDAT" + z + struct.pack(">I", zlib.crc32(b"IDAT" + z) & 0xffffffff)
    at = big.index(b"IDAT") - 4
    p = tmp_path / "bomb.png"
    p.write_bytes(bytes(big[:at]) + idat + b"\0\0\0\0IEND\xaeB`\x82")
    r = subprocess.run([program, "png", str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "longer than the image" in r.stdout, r.stdout


def _lerp8(img, u, v):
    """ImageTexture2D's byte lookup: each weighted texel truncated to a byte, / 255."""
    h, w = img.shape[:2]
    u = min(max(np.float32(u) - np.floor(np.float32(u)), 0), 1) * (w - 1)
    v = min(max(np.float32(v) - np.floor(np.float32(v)), 0), 1) * (h - 1)
    u0, v0 = int(u), int(v)
    u1, v1 = min(u0 + 1, w - 1), min(v0 + 1, h - 1)
    du, dv = u - u0, v - v0
    t = lambda x, f: (np.floor(f * x.astype(np.float64))).astype(np.int64) & 255
    top = (t(img[v0, u0], 1 - du) + t(img[v0, u1], du)) & 255
    bot = (t(img[v1, u0], 1 - du) + t(img[v1, u1], du)) & 255
    return (((t(top, 1 - dv) + t(bot, dv)) & 255).astype(np.float32) / np.float32(255)).astype(np.float32)


def test_png_texture_lookup(program, tmp_path):
    img = np.random.default_rng(3).integers(0, 256, (5, 9, 3), dtype=np.uint8)
    p = tmp_path / "t.png"
    p.write_bytes(_png([bytes(r) for r in img.reshape(5, 27)], 2))
    r = subprocess.run([program, "tex", str(p)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    got = np.array([float(v) for v in r.stdout.split()[1:]], np.float32)
    assert np.array_equal(got, _lerp8(img[::-1], 0.25, 0.5))


def test_material_with_png_map(program, tmp_path):
    """An 8-bit map of an MTL material: bytes / 255 raised to 2.2, back to
    bytes, times Kd, each step truncating to a byte."""
    p = tmp_path / "wall.png"
    p.write_bytes(_png([bytes([200, 100, 50] * 4)] * 3, 2))
    (tmp_path / "s.obj").write_text("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n")
    (tmp_path / "s.mtl").write_text(f"newmtl wall\nKd 0.5 0.5 0.5\nmap_Kd {p}\n")
    r = subprocess.run([program, "mtl", str(tmp_path / "s.obj")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    kd = np.array([float(v) for v in r.stdout.split()[3:6]], np.float32)
    texel = []
    for b in (200, 100, 50):
        g = int(np.float32(np.float32(b) / np.float32(255)) ** np.float32(2.2) * np.float32(255))
        texel.append(int(g * np.float32(0.5)))
    # the program looks the texture up at (0.5, 0.5): halfway between texels,
    # where the byte arithmetic can lose one level
    want = _lerp8(np.tile(np.array(texel, np.uint8), (3, 4, 1)), 0.5, 0.5)
    assert np.allclose(kd, want, rtol=0, atol=1e-6), (kd, want)
