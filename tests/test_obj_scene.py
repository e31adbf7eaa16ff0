"""The reference's OBJ scene flow (src/main.cpp:215-275) through the C++
host API, on the CPU: an OBJ/MTL pair whose walls use a PNG map, a glass
block (Ni > 1) and an emissive quad becomes a scene description by
load_model_from_file, create_texture_from_file, create_phong_material /
create_glass and create_triangle_mesh; the oracle and the reference build
render that description bit for bit alike."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from tracer_gb300 import build
from tracer_gb300.abi import make_filter, make_params

from test_host_api import _read_desc
from test_image_file import _png

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "obj_scene.cpp")


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    so = build.build()
    out = str(tmp_path_factory.mktemp("objscene") / "obj_scene")
    libdir = os.path.dirname(so)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}", SRC,
                    f"-L{libdir}", "-ltracer_gb300", f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def _box_obj():
    """An open box (floor, back, left, right walls with uvs), a glass block and a lamp."""
    v, vt, f = [], [], []

    def quad(p, mat):
        base = len(v)
        v.extend(p)
        vt.extend([(0, 0), (1, 0), (1, 1), (0, 1)])
        f.append((mat, [base + 1, base + 2, base + 3, base + 4]))
    quad([(-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)], "floor")
    quad([(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)], "wall")
    quad([(-1, -1, 1), (-1, -1, -1), (-1, 1, -1), (-1, 1, 1)], "wall")
    quad([(1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)], "wall")
    quad([(-0.3, 0.99, -0.3), (0.3, 0.99, -0.3), (0.3, 0.99, 0.3), (-0.3, 0.99, 0.3)], "lamp")
    g = [(-0.5, -1, -0.2), (0.0, -1, -0.2), (0.0, -0.3, -0.2), (-0.5, -0.3, -0.2)]
    quad(g, "glass")
    lines = ["mtllib scene.mtl"] + [f"v {x} {y} {z}" for x, y, z in v] + [f"vt {a} {b}" for a, b in vt]
    lines += ["vn 0 1 0", "vn 0 0 1", "vn 1 0 0", "vn -1 0 0", "vn 0 -1 0"]
    normals = {"floor": 1, "lamp": 5, "glass": 2}
    cur = None
    for k, (mat, idx) in enumerate(f):
        if mat != cur:
            lines += [f"o part{k}", f"usemtl {mat}"]
            cur = mat
        n = normals.get(mat, [2, 3, 4][min(k - 1, 2)])
        lines.append("f " + " ".join(f"{i}/{i}/{n}" for i in idx))
    return "\n".join(lines) + "\n"


def test_obj_scene_renders_like_the_reference(program, tmp_path):
    board = np.zeros((8, 8, 3), np.uint8)
    board[...] = np.where(((np.add.outer(np.arange(8), np.arange(8)) // 2) % 2 == 1)[..., None],
                          np.array([40, 90, 200], np.uint8), np.array([220, 200, 180], np.uint8))
    (tmp_path / "wall.png").write_bytes(_png([bytes(r) for r in board.reshape(8, 24)], 2))
    (tmp_path / "scene.obj").write_text(_box_obj())
    (tmp_path / "scene.mtl").write_text(
        "newmtl floor\nKd 0.7 0.7 0.7\n"
        "newmtl wall\nKd 0.9 0.9 0.9\nKs 0.05 0.05 0.05\nNs 30\nmap_Kd wall.png\n"
        "newmtl lamp\nKd 0 0 0\nKe 15 12 8\n"
        "newmtl glass\nKs 0 0 0\nNi 1.5\n")
    cwd = os.getcwd()
    os.chdir(tmp_path)  # MTL map names are relative, as the reference reads them
    try:
        r = subprocess.run([program, str(tmp_path / "scene.obj"), str(tmp_path / "s")], capture_output=True,
                           text=True)
    finally:
        os.chdir(cwd)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "1 textures" in r.stdout and "2 lights" in r.stdout, r.stdout
    sb, cam = _read_desc(str(tmp_path / "s.desc"))
    from tracer_gb300.abi import TR_MAT_GLASS, TR_MAT_PHONG
    kinds = sorted(m.rec.kind for m in sb.materials)
    assert kinds.count(TR_MAT_GLASS) == 1 and kinds.count(TR_MAT_PHONG) == 3
    if not oracle.ref_available():
        pytest.skip("reference build not available")
    par = make_params(24, 24, 4, 2, 6)
    port, ref = oracle.Oracle(sb, "port"), oracle.Oracle(sb, "reference")
    for o in (port, ref):
        o.set_camera(cam, make_filter(0.5, 0.6))
    a, b = port.render(par), ref.render(par)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a[..., :3] / a[..., 3:]).mean() > 0
