"""The 8-bit image reader behind load_image_from_file: baseline JPEG, TGA and
BMP (and PNG, tests/test_image_file.py), found from the file's bytes, rows
flipped and 1/4 channels turned into RGB as the reference's reader does
(src/utility/image_file.cpp:26-58 over its vendored stb_image v2.26).

The decoded bytes are the reference's, bit for bit: against a fixture made by
the reference's own reader (tests/golden/make_golden.py), and -- where the
reference build exists -- live on fresh files from the reference's own
encoders and from tests/jpeg_writer.py."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from tracer_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "image_file.cpp")
FIXTURE = os.path.join(ROOT, "tests", "golden", "image_files.npz")
TR_ERR_ARG = 1
TR_ERR_UNSUPPORTED = 8


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    so = build.build()
    out = str(tmp_path_factory.mktemp("fmt") / "image_file")
    libdir = os.path.dirname(so)
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", SRC, f"-L{libdir}",
                    "-ltracer_gb300", f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def _read(program, path):
    r = subprocess.run([program, "png", str(path)], capture_output=True, text=True)
    lines = r.stdout.splitlines()
    if r.returncode != 0:
        return None, lines[0] if lines else ""
    w, h = (int(v) for v in lines[0].split()[1:])
    return np.array([[int(v) for v in ln.split()] for ln in lines[1:]], np.uint8).reshape(h, w, 3), ""


def _cases():
    g = np.load(FIXTURE)
    k = 0
    while f"name{k}" in g:
        yield str(g[f"name{k}"]), g[f"file{k}"].tobytes(), g[f"rgb{k}"]
        k += 1


@pytest.mark.parametrize("case", range(18))
def test_reader_against_the_reference_fixture(program, tmp_path, case):
    name, data, want = list(_cases())[case]
    p = tmp_path / name
    p.write_bytes(data)
    got, err = _read(program, p)
    assert got is not None, err
    print(name, got.shape)
    assert np.array_equal(got, want)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", range(4))
def test_reader_against_the_reference_live(program, tmp_path, seed):
    """Random images, sizes and settings: the reference's encoders (JPEG at a
    random quality, TGA raw or run-length, BMP; 1, 3 or 4 channels) and the
    test JPEG writer (random sampling factors, restart interval, scans), read
    by this reader and by the reference's."""
    import ctypes as C
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from jpeg_writer import write_jpeg
    lib = C.CDLL(oracle.REF_SO)
    rng = np.random.default_rng(seed)

    def ref_read(path):
        w, h = C.c_int(), C.c_int()
        assert lib.ref_load_image(str(path).encode(), C.byref(w), C.byref(h), None) == 0
        px = np.zeros((h.value, w.value, 3), np.uint8)
        lib.ref_load_image(str(path).encode(), C.byref(w), C.byref(h), px.ctypes.data_as(C.c_void_p))
        return px

    for k in range(6):
        h, w = int(rng.integers(1, 70)), int(rng.integers(1, 70))
        yy, xx = np.mgrid[0:h, 0:w]
        img = np.stack([xx * rng.integers(1, 9), yy * rng.integers(1, 9), (xx + yy) * 3], -1).clip(0, 255)
        img = (img * 0.7 + rng.random((h, w, 3)) * 76).astype(np.uint8)
        kind = k % 4
        if kind < 3:
            c = int(rng.choice([1, 3, 4]))
            src = np.ascontiguousarray(np.dstack([img, img[..., :1]])[..., :c])
            p = tmp_path / (f"s{seed}_{k}." + ["jpg", "tga", "bmp"][kind])
            q = int(rng.integers(20, 100)) if kind == 0 else int(rng.integers(0, 2))
            assert lib.ref_write_image(str(p).encode(), kind, w, h, c, src.ctypes.data_as(C.c_void_p), q) == 1
        else:
            hs = [tuple(int(v) for v in rng.choice([1, 2], 2)) for _ in range(3)]
            p = tmp_path / f"w{seed}_{k}.jpg"
            p.write_bytes(write_jpeg(img, sampling=hs, quant=int(rng.integers(1, 20)),
                                     restart=int(rng.integers(0, 4)), interleaved=bool(rng.integers(0, 2))))
        got, err = _read(program, p)
        assert got is not None, (p, err)
        assert np.array_equal(got, ref_read(p)), p


def test_refusals(program, tmp_path):
    """Formats outside the reader (progressive and arithmetic-coded JPEG,
    four-component JPEG, compressed BMP) are TR_ERR_UNSUPPORTED; truncated
    or unknown files TR_ERR_ARG."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from jpeg_writer import write_jpeg
    img = (np.arange(16 * 16 * 3) % 251).astype(np.uint8).reshape(16, 16, 3)
    good = bytearray(write_jpeg(img))
    sof = good.index(b"\xFF\xC0")
    for marker, status in ((0xC2, TR_ERR_UNSUPPORTED), (0xC9, TR_ERR_UNSUPPORTED)):
        bad = bytearray(good)
        bad[sof + 1] = marker
        (tmp_path / "p.jpg").write_bytes(bytes(bad))
        got, err = _read(program, tmp_path / "p.jpg")
        assert got is None and err.startswith(f"error {status}"), err
    for cut in (40, len(good) // 2):
        (tmp_path / "t.jpg").write_bytes(bytes(good[:cut]))
        got, err = _read(program, tmp_path / "t.jpg")
        # a cut inside the scan's data decodes what is there (the missing
        # bits read as zeros, as the reference does); inside a header it fails
        assert got is not None or err.startswith(f"error {TR_ERR_ARG}"), err
    (tmp_path / "u.img").write_bytes(b"not an image at all" * 4)
    got, err = _read(program, tmp_path / "u.img")
    assert got is None and err.startswith(f"error {TR_ERR_ARG}"), err
    # BMP with BI_RLE8 compression
    bmp = bytearray(b"BM" + (70).to_bytes(4, "little") + bytes(4) + (54 + 8).to_bytes(4, "little") +
                    (40).to_bytes(4, "little") + (2).to_bytes(4, "little") + (2).to_bytes(4, "little") +
                    (1).to_bytes(2, "little") + (8).to_bytes(2, "little") + (1).to_bytes(4, "little") + bytes(20) +
                    bytes(16))
    (tmp_path / "r.bmp").write_bytes(bytes(bmp))
    got, err = _read(program, tmp_path / "r.bmp")
    assert got is None and err.startswith(f"error {TR_ERR_UNSUPPORTED}"), err
