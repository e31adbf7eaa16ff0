"""Parity oracle -- TEST INFRASTRUCTURE ONLY.

Two CPU implementations of Tracer's path-tracing hot path behind the same
Python interface:

* ``Oracle("port")``: oracle/tracer_oracle.cpp, a restatement of the
  reference's algorithm (builds anywhere; used beside the GPU).
* ``Oracle("reference")``: the reference's own sources compiled here by
  ``make -C oracle ref`` (only where the reference checkout exists).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only to check the GPU path's results or as the timed CPU
baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from tracer_gb300.abi import (NODE_DTYPE, RAY_DTYPE, TrCamera, TrFilter, TrRay, TrRenderParams,
                              TrSceneDesc, TrBvhNode32)

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libtracer_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtracer_ref.so")
REF_SO_O0 = os.path.join(HERE, "_ref", "O0", "libtracer_ref.so")  # the as-shipped -O0 build (CPU-baseline record)
# the reference checkout: a sibling of this repository unless TRACER_REF_ROOT says otherwise
REF_ROOT = os.environ.get("TRACER_REF_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_ref() -> str | None:
    """Compiles the reference oracle when the reference checkout is present."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True)
    return REF_SO


def ref_available() -> bool:
    if not os.path.exists(REF_SO):
        return False
    try:
        C.CDLL(REF_SO)
        return True
    except OSError:
        return False


_libs: dict[str, C.CDLL] = {}


def _load(kind: str) -> C.CDLL:
    if kind in _libs:
        return _libs[kind]
    if kind == "port":
        if not os.path.exists(PORT_SO):
            build_port()
        lib = C.CDLL(PORT_SO)
        pre = "orc_"
    else:
        lib = C.CDLL(REF_SO_O0 if kind == "reference-O0" else REF_SO)
        pre = "ref_"
    vp, sz = C.c_void_p, C.c_size_t
    f32p, i32p, u32p, u8p = (C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                             C.POINTER(C.c_uint8))
    getattr(lib, pre + "scene_create").restype = vp
    getattr(lib, pre + "scene_create").argtypes = [C.POINTER(TrSceneDesc)]
    getattr(lib, pre + "scene_destroy").argtypes = [vp]
    getattr(lib, pre + "set_camera").argtypes = [vp, C.POINTER(TrCamera), C.POINTER(TrFilter)]
    getattr(lib, pre + "make_ray").argtypes = [f32p, f32p, C.c_float, C.c_float, C.POINTER(TrRay)]
    getattr(lib, pre + "cross").argtypes = [f32p, f32p, f32p, sz]
    getattr(lib, pre + "normalize").argtypes = [f32p, f32p, sz]
    getattr(lib, pre + "pcg_uniform").argtypes = [C.c_int, f32p, sz]
    if kind == "port":
        lib.orc_trace_closest.argtypes = [vp, C.POINTER(TrRay), sz, i32p, f32p, u32p, u32p, C.c_int]
        lib.orc_trace_any.argtypes = [vp, C.POINTER(TrRay), sz, u8p, u32p, u32p, C.c_int]
        lib.orc_render.restype = C.c_uint64
        lib.orc_render.argtypes = [vp, C.POINTER(TrRenderParams), C.c_int, C.c_int, f32p,
                                   C.POINTER(C.c_double), C.c_int]
        lib.orc_render_rows.restype = C.c_uint64
        lib.orc_render_rows.argtypes = [vp, C.POINTER(TrRenderParams), i32p, C.c_int, f32p, C.c_int]
        lib.orc_render_log.restype = sz
        lib.orc_render_log.argtypes = [vp, C.POINTER(TrRenderParams), C.c_int, C.c_int, C.POINTER(sz)]
        lib.orc_log_fetch.argtypes = [C.POINTER(TrRay), i32p, f32p, C.POINTER(TrRay), u8p]
        lib.orc_bvh_num_nodes.restype = sz
        lib.orc_bvh_num_nodes.argtypes = [vp]
        lib.orc_bvh_export.argtypes = [vp, C.POINTER(TrBvhNode32), u32p]
        lib.orc_slab_scale.argtypes = [f32p, f32p, sz]
    else:
        lib.ref_trace_closest.argtypes = [vp, C.POINTER(TrRay), sz, i32p, f32p, C.c_int]
        lib.ref_trace_any.argtypes = [vp, C.POINTER(TrRay), sz, u8p, C.c_int]
        lib.ref_render.argtypes = [vp, C.POINTER(TrRenderParams), f32p, C.c_int]
        lib.ref_render_stock.restype = C.c_double
        lib.ref_render_stock.argtypes = [vp, C.POINTER(TrRenderParams), C.c_int, f32p]
        lib.ref_bvh_export.restype = sz
        lib.ref_bvh_export.argtypes = [vp, C.POINTER(TrBvhNode32), u32p]
    _libs[kind] = lib
    return lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """One CPU scene in the port or the reference build."""

    def __init__(self, scene_buffers, kind: str = "port", threads: int | None = None):
        self.kind = kind
        self.lib = _load(kind)
        self.pre = "orc_" if kind == "port" else "ref_"
        self.threads = threads or os.cpu_count() or 1
        self._desc = scene_buffers.desc()
        self._scene = scene_buffers
        self.h = getattr(self.lib, self.pre + "scene_create")(C.byref(self._desc))
        if not self.h:
            raise ValueError("oracle rejected the scene")

    def close(self):
        if self.h:
            getattr(self.lib, self.pre + "scene_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_camera(self, cam: TrCamera, filt: TrFilter):
        self._cam, self._filt = cam, filt
        getattr(self.lib, self.pre + "set_camera")(self.h, C.byref(cam), C.byref(filt))

    def trace_closest(self, rays: np.ndarray, counts: bool = False):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        n = len(rays)
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        if self.kind == "port":
            nodes = np.empty(n, np.uint32) if counts else None
            prims = np.empty(n, np.uint32) if counts else None
            self.lib.orc_trace_closest(self.h, _p(rays, TrRay), n, _p(prim, C.c_int32), _p(t, C.c_float),
                                       _p(nodes, C.c_uint32) if counts else None,
                                       _p(prims, C.c_uint32) if counts else None, self.threads)
            if counts:
                return prim, t, nodes, prims
        else:
            self.lib.ref_trace_closest(self.h, _p(rays, TrRay), n, _p(prim, C.c_int32), _p(t, C.c_float),
                                       self.threads)
        return prim, t

    def trace_any(self, rays: np.ndarray, counts: bool = False):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        n = len(rays)
        hit = np.empty(n, np.uint8)
        if self.kind == "port":
            nodes = np.empty(n, np.uint32) if counts else None
            prims = np.empty(n, np.uint32) if counts else None
            self.lib.orc_trace_any(self.h, _p(rays, TrRay), n, _p(hit, C.c_uint8),
                                   _p(nodes, C.c_uint32) if counts else None,
                                   _p(prims, C.c_uint32) if counts else None, self.threads)
            if counts:
                return hit, nodes, prims
        else:
            self.lib.ref_trace_any(self.h, _p(rays, TrRay), n, _p(hit, C.c_uint8), self.threads)
        return hit

    def render(self, params: TrRenderParams, fp64: bool = False, rows: tuple[int, int] | None = None):
        """Per-pixel-seeded render; returns (H, W, 4) sums + weight."""
        W, H = params.width, params.height
        if self.kind == "port":
            r0, r1 = rows if rows else (0, 0)
            if fp64:
                out = np.zeros((H, W, 4), np.float64)
                self.lib.orc_render(self.h, C.byref(params), r0, r1, None, _p(out, C.c_double), self.threads)
            else:
                out = np.zeros((H, W, 4), np.float32)
                self.lib.orc_render(self.h, C.byref(params), r0, r1, _p(out, C.c_float), None, self.threads)
            return out
        out = np.zeros((H, W, 4), np.float32)
        self.lib.ref_render(self.h, C.byref(params), _p(out, C.c_float), self.threads)
        return out

    def render_rows(self, params: TrRenderParams, rows):
        """Port only: the given rows of the per-pixel-seeded render, in parallel."""
        rows = np.ascontiguousarray(rows, np.int32)
        out = np.zeros((len(rows), params.width, 4), np.float32)
        n = self.lib.orc_render_rows(self.h, C.byref(params), _p(rows, C.c_int32), len(rows),
                                     _p(out, C.c_float), self.threads)
        return out, int(n)

    def render_stock_seconds(self, params: TrRenderParams, workers: int = 0):
        """Reference build only: time of the stock create_pt_renderer render()."""
        assert self.kind.startswith("reference")
        return self.lib.ref_render_stock(self.h, C.byref(params), workers, None)

    def render_log(self, params: TrRenderParams, pix0: int, pix1: int):
        """Port only: every closest/any query of pixels [pix0, pix1) with results."""
        n_any = C.c_size_t()
        n = self.lib.orc_render_log(self.h, C.byref(params), pix0, pix1, C.byref(n_any))
        cr = np.zeros(n, RAY_DTYPE)
        cp = np.zeros(n, np.int32)
        ct = np.zeros(n, np.float32)
        ar = np.zeros(n_any.value, RAY_DTYPE)
        ah = np.zeros(n_any.value, np.uint8)
        self.lib.orc_log_fetch(_p(cr, TrRay), _p(cp, C.c_int32), _p(ct, C.c_float), _p(ar, TrRay),
                               _p(ah, C.c_uint8))
        return cr, cp, ct, ar, ah

    def bvh(self):
        if self.kind == "port":
            n = self.lib.orc_bvh_num_nodes(self.h)
            nodes = np.zeros(n, NODE_DTYPE)
            order = np.zeros(len(self._scene.prim_shape), np.uint32)
            self.lib.orc_bvh_export(self.h, _p(nodes, TrBvhNode32), _p(order, C.c_uint32))
        else:
            n = self.lib.ref_bvh_export(self.h, None, None)
            nodes = np.zeros(n, NODE_DTYPE)
            order = np.zeros(len(self._scene.prim_shape), np.uint32)
            self.lib.ref_bvh_export(self.h, _p(nodes, TrBvhNode32), _p(order, C.c_uint32))
        return nodes, order


def make_ray(kind, o, d, t_min, t_max):
    lib = _load(kind)
    pre = "orc_" if kind == "port" else "ref_"
    r = TrRay()
    oa = (C.c_float * 3)(*o)
    da = (C.c_float * 3)(*d)
    getattr(lib, pre + "make_ray")(oa, da, t_min, t_max, C.byref(r))
    return r


def unit(kind, name, *arrays, out_shape, n):
    lib = _load(kind)
    pre = "orc_" if kind == "port" else "ref_"
    out = np.zeros(out_shape, np.float32)
    args = [_p(np.ascontiguousarray(a, np.float32), C.c_float) for a in arrays]
    getattr(lib, pre + name)(*args, _p(out, C.c_float), n)
    return out


def pcg_uniform(kind, seed, n):
    lib = _load(kind)
    pre = "orc_" if kind == "port" else "ref_"
    out = np.zeros(n, np.float32)
    getattr(lib, pre + "pcg_uniform")(seed, _p(out, C.c_float), n)
    return out


# ---- output path: film resolve, post-processors, 8-bit and RGBE encodings
def _post_lib(kind):
    lib = _load(kind)
    f32p, u8p, sz = C.POINTER(C.c_float), C.POINTER(C.c_uint8), C.c_size_t
    if kind == "port":
        lib.orc_post_resolve.argtypes = [f32p, sz, f32p]
        lib.orc_post_aces.argtypes = [f32p, sz, C.c_float]
        lib.orc_post_gamma.argtypes = [f32p, sz, C.c_float]
        lib.orc_post_rgb8.argtypes = [f32p, sz, C.c_float, u8p]
        lib.orc_post_rgbe.argtypes = [f32p, sz, u8p]
    else:
        lib.ref_post_process.argtypes = [f32p, C.c_int, C.c_int, C.c_int, C.c_float]
    return lib


def post_resolve(film: np.ndarray) -> np.ndarray:
    """(H, W, 4) float32 film sums -> (H, W, 3) image (Film::write_render_target)."""
    film = np.ascontiguousarray(film, np.float32)
    out = np.zeros(film.shape[:-1] + (3,), np.float32)
    _post_lib("port").orc_post_resolve(_p(film, C.c_float), film.size // 4, _p(out, C.c_float))
    return out


def post_process(kind: str, rgb: np.ndarray, which: str, param: float) -> np.ndarray:
    """ACES tone mapper ("aces", exposure) or gamma corrector ("gamma", gamma)
    on an (H, W, 3) image: the restatement ("port") or the reference's own
    post-processors ("reference")."""
    img = np.array(rgb, np.float32, copy=True, order="C")
    lib = _post_lib(kind)
    if kind == "port":
        fn = lib.orc_post_aces if which == "aces" else lib.orc_post_gamma
        fn(_p(img, C.c_float), img.size, param)
    else:
        h, w = img.shape[:2]
        lib.ref_post_process(_p(img, C.c_float), w, h, 0 if which == "aces" else 1, param)
    return img


def post_rgb8(rgb: np.ndarray, inv_gamma: float = 1.0 / 2.2) -> np.ndarray:
    img = np.ascontiguousarray(rgb, np.float32)
    out = np.zeros(img.shape, np.uint8)
    _post_lib("port").orc_post_rgb8(_p(img, C.c_float), img.size, inv_gamma, _p(out, C.c_uint8))
    return out


def post_rgbe(rgb: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(rgb, np.float32)
    out = np.zeros(img.shape[:-1] + (4,), np.uint8)
    _post_lib("port").orc_post_rgbe(_p(img, C.c_float), img.size // 3, _p(out, C.c_uint8))
    return out
