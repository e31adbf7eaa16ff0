"""The C ABI library builds, loads and exports every entry point that
include/*.h declares (no compute: this runs without a GPU)."""
import ctypes
import os
import re

import numpy as np

from tracer_gb300 import build
from tracer_gb300.abi import NODE_DTYPE, RAY_DTYPE, TrCamera, TrMaterial, TrRay, TrRenderParams, TrSceneDesc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(tr_[a-z0-9_]+)\s*\(", src, re.M):
                names.add(m.group(1))
    return names


def test_exports_every_declared_symbol():
    lib = ctypes.CDLL(build.build())
    names = declared_functions()
    assert {"tr_ctx_create", "tr_scene_upload", "tr_trace_closest", "tr_trace_any", "tr_render"} <= names
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_struct_layouts():
    assert ctypes.sizeof(TrRay) == 32 and RAY_DTYPE.itemsize == 32
    assert NODE_DTYPE.itemsize == 32
    assert ctypes.sizeof(TrCamera) == 4 * 13
    assert ctypes.sizeof(TrRenderParams) == 4 * 8
    assert ctypes.sizeof(TrMaterial) == 4 * 62  # + glass kr, kt, ior; metal color, eta, k; Disney 2015; maps


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirror against the C compiler's layout of include/tracer_gpu.h:
    sizes and the offsets of the fields added last."""
    import subprocess
    from tracer_gb300.abi import TrFilter, TrTexture
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "layout.c"
    fields = {"tr_scene_desc": ["env_width", "env_texels", "env_to_world", "env_texels8", "num_textures",
                                "textures", "max_leaf_prims"],
              "tr_material": ["k", "transmission", "specular_scale", "tex_ka", "tex_ns"],
              "tr_texture": ["texels", "texels8"], "tr_camera": ["focal_dist"], "tr_filter": ["alpha"],
              "tr_render_params": ["flags"]}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "tracer_gpu.h"', "int main(void) {"]
    for t, fs in fields.items():
        lines.append(f'  printf("{t} %zu\\n", sizeof({t}));')
        for f in fs:
            lines.append(f'  printf("{t}.{f} %zu\\n", offsetof({t}, {f}));')
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", f"-I{os.path.join(root, 'include')}", str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                    check=True).stdout.splitlines())
    py = {"tr_scene_desc": TrSceneDesc, "tr_material": TrMaterial, "tr_texture": TrTexture, "tr_camera": TrCamera,
          "tr_filter": TrFilter, "tr_render_params": TrRenderParams}
    for t, fs in fields.items():
        assert int(got[t]) == ctypes.sizeof(py[t]), t
        for f in fs:
            assert int(got[f"{t}.{f}"]) == getattr(py[t], f).offset, (t, f)


def test_make_ray_matches_reference_semantics():
    from tracer_gb300 import scenes
    from tracer_gb300.native import make_ray
    rng = np.random.default_rng(4)
    d = rng.normal(size=(200, 3)).astype(np.float32)
    want = scenes.ref_normalize(d)
    for i in range(200):
        r = make_ray((0, 0, 0), tuple(float(x) for x in d[i]))
        assert np.array_equal(np.array(r.d, np.float32).view(np.uint32), want[i].view(np.uint32))


def test_status_strings():
    from tracer_gb300.native import lib
    L = lib()
    for s in range(9):
        assert L.tr_status_string(s)


def test_tuning_struct_layout():
    from tracer_gb300.abi import TrTuning
    assert ctypes.sizeof(TrTuning) == 40


def test_guide_kappa_range_matches_header():
    import re
    from pathlib import Path

    from tracer_gb300.native import GpuContext
    h = (Path(__file__).resolve().parents[1] / "include" / "tracer_gpu.h").read_text()
    lo = float(re.search(r"#define TR_GUIDE_LOG_KAPPA_MIN \(([-0-9.]+)f\)", h).group(1))
    hi = float(re.search(r"#define TR_GUIDE_LOG_KAPPA_MAX \(([-0-9.]+)f\)", h).group(1))
    assert GpuContext.GUIDE_LOG_KAPPA == (lo, hi)
