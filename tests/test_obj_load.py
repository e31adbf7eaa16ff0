"""load_model_from_file (the reference's src/utility/mesh_load.cpp:25-113)
through the C++ host API: a program reads OBJ/MTL files written here and
prints the model; faces with negative indices, polygons, two shapes,
vertex deduplication, normal normalisation, materials and errors."""
import os
import subprocess

import numpy as np
import pytest

from tracer_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "obj_load.cpp")

OBJ = """# two shapes
mtllib scene.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 2
o quad
usemtl white
f 1/1/1 2/2/1 3/3/1 4/4/1
g tri
usemtl lamp
f -4//-1 -3//-1 -2//-1
f 1/1/1 2/2/1 3/3/1
"""
MTL = """newmtl white
Kd 0.73 0.73 0.73
Ni 1.5
Pr 0.25
map_Kd wall.png
newmtl lamp
Kd 0 0 0
Ke 17 12 4
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    so = build.build()
    out = str(tmp_path_factory.mktemp("obj") / "obj_load")
    libdir = os.path.dirname(so)
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", SRC, f"-L{libdir}",
                    "-ltracer_gb300", f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def _run(program, tmp_path, obj, mtl=MTL):
    (tmp_path / "scene.obj").write_text(obj)
    (tmp_path / "scene.mtl").write_text(mtl)
    r = subprocess.run([program, str(tmp_path / "scene.obj")], capture_output=True, text=True)
    return r.returncode, r.stdout.splitlines()


def test_obj_model(program, tmp_path):
    rc, lines = _run(program, tmp_path, OBJ)
    assert rc == 0, lines
    assert lines[0] == "name /scene.obj"
    assert lines[1] == "materials 2"
    assert lines[2].split() == ["material", "white", "0.73", "0.73", "0.73", "1.5", "0.25", "0", "wall.png"]
    assert lines[3].split()[:2] == ["material", "lamp"] and lines[3].split()[7] == "17"
    assert lines[4] == "meshes 2"
    # the quad: four vertices (normal (0,0,2) normalised), fan-triangulated
    assert lines[5] == "mesh quad 4 2"
    v = np.array([[float(x) for x in l.split()[1:]] for l in lines[6:10]], np.float32)
    assert np.array_equal(v[:, 0:3], np.float32([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]))
    assert np.array_equal(v[:, 3:6], np.tile(np.float32([0, 0, 1]), (4, 1)))
    assert np.array_equal(v[:, 6:8], np.float32([[0, 0], [1, 0], [1, 1], [0, 1]]))
    assert lines[10:12] == ["t 0 1 2 0", "t 0 2 3 0"]
    # the triangle group: negative indices and no uv (0, 0); the second face
    # reuses the first vertex (uv (0, 0) too) and adds two (deduplication by
    # position, normal and uv)
    assert lines[12] == "mesh tri 5 2"
    assert lines[18:20] == ["t 0 1 2 1", "t 0 3 4 1"]


@pytest.mark.parametrize("bad,what", [("f 1 2 3\n", "without a normal"), ("f 1//1 2//1 9//1\n", "out of range"),
                                      ("v 1 2\n", "three numbers"), ("f 1//1 2//1\n", "fewer than three")])
def test_obj_errors(program, tmp_path, bad, what):
    rc, lines = _run(program, tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\n" + bad)
    assert rc == 1 and lines[0].startswith("error") and what in lines[0]


def test_missing_file(program, tmp_path):
    r = subprocess.run([program, str(tmp_path / "none.obj")], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stdout
