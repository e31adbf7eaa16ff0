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
    assert ctypes.sizeof(TrMaterial) == 4 * 49  # + glass kr, kt, ior; metal color, eta, k; Disney 2015; maps


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
    assert ctypes.sizeof(TrTuning) == 20


def test_guide_kappa_range_matches_header():
    import re
    from pathlib import Path

    from tracer_gb300.native import GpuContext
    h = (Path(__file__).resolve().parents[1] / "include" / "tracer_gpu.h").read_text()
    lo = float(re.search(r"#define TR_GUIDE_LOG_KAPPA_MIN \(([-0-9.]+)f\)", h).group(1))
    hi = float(re.search(r"#define TR_GUIDE_LOG_KAPPA_MAX \(([-0-9.]+)f\)", h).group(1))
    assert GpuContext.GUIDE_LOG_KAPPA == (lo, hi)
