"""The reference's image-file helpers (src/utility/image_file.cpp) through the
C++ host API: the Radiance HDR reader on files written here (flat and
run-length scanlines), write/read round trips, create_texture2d_from_file's
format rules and create_texture_from_file on MTL materials."""
import os
import subprocess

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


@pytest.mark.parametrize("name,status", [("x.png", TR_ERR_UNSUPPORTED), ("x.jpg", TR_ERR_UNSUPPORTED),
                                         ("x.tga", TR_ERR_ARG), ("noext", TR_ERR_ARG), ("missing.hdr", TR_ERR_ARG)])
def test_texture_file_rules(program, tmp_path, name, status):
    """create_texture2d_from_file: .hdr read, 8-bit formats unsupported here,
    other extensions rejected as the reference rejects them."""
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


def test_material_with_png_map_is_unsupported(program, tmp_path):
    (tmp_path / "s.obj").write_text("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n")
    (tmp_path / "s.mtl").write_text("newmtl wall\nKd 0.7 0.6 0.5\nmap_Kd wall.png\n")
    r = subprocess.run([program, "mtl", str(tmp_path / "s.obj")], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith(f"error {TR_ERR_UNSUPPORTED}")
