"""ctypes binding of libtracer_gb300.so (the C ABI in include/tracer_gpu.h).

Loading fails loudly: there is no CPU fallback. `GpuContext` owns one
`tr_ctx` (one CUDA device, one stream).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .abi import (NODE_DTYPE, RAY_DTYPE, TR_OK, TrBvhNode32, TrCamera, TrFilter, TrRay, TrRenderParams, TrTuning, TrGuideParams, TrBatchJob,
                  TrSceneDesc, TrStats)

_lib = None


class TracerError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"tracer_gb300 status {status}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Loads the native library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    L = C.CDLL(path)
    vp, sz = C.c_void_p, C.c_size_t
    st = C.c_int
    L.tr_status_string.restype = C.c_char_p
    L.tr_status_string.argtypes = [st]
    L.tr_make_ray.restype = st
    L.tr_make_ray.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_float, C.POINTER(TrRay)]
    L.tr_ctx_create.restype = st
    L.tr_ctx_create.argtypes = [C.POINTER(vp), C.c_int]
    L.tr_ctx_destroy.restype = None
    L.tr_ctx_destroy.argtypes = [vp]
    L.tr_ctx_last_error.restype = C.c_char_p
    L.tr_ctx_last_error.argtypes = [vp]
    L.tr_ctx_stream.restype = vp
    L.tr_ctx_stream.argtypes = [vp]
    L.tr_synchronize.restype = st
    L.tr_synchronize.argtypes = [vp]
    L.tr_scene_upload.restype = st
    L.tr_scene_upload.argtypes = [vp, C.POINTER(TrSceneDesc)]
    L.tr_bvh_info.restype = st
    L.tr_bvh_info.argtypes = [vp, C.POINTER(sz), C.POINTER(sz)]
    L.tr_bvh_export.restype = st
    L.tr_bvh_export.argtypes = [vp, C.POINTER(TrBvhNode32), C.POINTER(C.c_uint32)]
    L.tr_bvh_upload.restype = st
    L.tr_bvh_upload.argtypes = [vp, C.POINTER(TrBvhNode32), sz, C.POINTER(C.c_uint32), sz]
    L.tr_trace_closest.restype = st
    L.tr_trace_closest.argtypes = [vp, C.POINTER(TrRay), sz, C.POINTER(C.c_int32), C.POINTER(C.c_float)]
    L.tr_trace_any.restype = st
    L.tr_trace_any.argtypes = [vp, C.POINTER(TrRay), sz, C.POINTER(C.c_uint8)]
    L.tr_trace_closest_dev.restype = st
    L.tr_trace_closest_dev.argtypes = [vp, vp, sz, vp, vp]
    L.tr_trace_any_dev.restype = st
    L.tr_trace_any_dev.argtypes = [vp, vp, sz, vp]
    L.tr_render.restype = st
    L.tr_render.argtypes = [vp, C.POINTER(TrCamera), C.POINTER(TrFilter), C.POINTER(TrRenderParams),
                            C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(TrStats)]
    L.tr_ctx_set_bvh_builder.restype = st
    L.tr_ctx_set_bvh_builder.argtypes = [vp, C.c_int32]
    L.tr_bvh_stats.restype = st
    L.tr_bvh_stats.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    for name, args in (("tr_film_resolve_dev", [vp, vp, vp, sz, vp]), ("tr_aces_tone_map_dev", [vp, vp, sz, C.c_float]),
                       ("tr_gamma_correct_dev", [vp, vp, sz, C.c_float]),
                       ("tr_to_rgb8_dev", [vp, vp, sz, C.c_float, vp]), ("tr_to_rgbe_dev", [vp, vp, sz, vp]),
                       ("tr_write_png", [C.c_char_p, vp, C.c_uint32, C.c_uint32]),
                       ("tr_write_hdr", [C.c_char_p, vp, C.c_uint32, C.c_uint32])):
        getattr(L, name).restype = st
        getattr(L, name).argtypes = args
    L.tr_any_tree_info.restype = st
    L.tr_any_tree_info.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_int32)]
    L.tr_ctx_set_tuning.restype = st
    L.tr_ctx_set_tuning.argtypes = [vp, C.POINTER(TrTuning)]
    L.tr_ctx_get_tuning.restype = st
    L.tr_ctx_get_tuning.argtypes = [vp, C.POINTER(TrTuning)]
    L.tr_guide_init.restype = st
    L.tr_guide_init.argtypes = [vp, C.c_uint64]
    L.tr_guide_set_params.restype = st
    L.tr_guide_set_params.argtypes = [vp, C.POINTER(C.c_float), C.c_size_t]
    L.tr_guide_get_params.restype = st
    L.tr_guide_get_params.argtypes = [vp, C.POINTER(C.c_float), C.c_size_t]
    L.tr_guide_forward_dev.restype = st
    L.tr_guide_forward_dev.argtypes = [vp, C.c_void_p, C.c_size_t, C.c_void_p]
    L.tr_guide_backward_dev.restype = st
    L.tr_guide_backward_dev.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    L.tr_guide_loss_dev.restype = st
    L.tr_guide_loss_dev.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                    C.POINTER(C.c_float)]
    L.tr_guide_train_step_dev.restype = st
    L.tr_guide_train_step_dev.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_float,
                                          C.POINTER(C.c_float)]
    L.tr_render_guided_dev.restype = st
    L.tr_render_guided_dev.argtypes = [vp, C.POINTER(TrCamera), C.POINTER(TrFilter), C.POINTER(TrRenderParams),
                                       C.POINTER(TrGuideParams), C.c_void_p, C.c_void_p, C.POINTER(TrStats)]
    L.tr_guide_train_on_records.restype = st
    L.tr_guide_train_on_records.argtypes = [vp, C.c_int32, C.c_uint32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]
    L.tr_guide_light_init.restype = st
    L.tr_guide_light_init.argtypes = [vp, C.POINTER(C.c_int32), C.c_int32]
    L.tr_guide_light_update.restype = st
    L.tr_guide_light_update.argtypes = [vp, C.c_float]
    L.tr_scene_set_upload.restype = st
    L.tr_scene_set_upload.argtypes = [vp, C.POINTER(TrSceneDesc), C.c_uint32]
    L.tr_render_batch_dev.restype = st
    L.tr_render_batch_dev.argtypes = [vp, C.POINTER(TrBatchJob), C.c_uint32, C.POINTER(TrStats)]
    L.tr_autotune.restype = st
    L.tr_autotune.argtypes = [vp, C.POINTER(TrBatchJob), C.c_uint32, C.c_int32, C.POINTER(TrTuning),
                              C.POINTER(C.c_double)]
    L.tr_trace_count_dev.restype = st
    L.tr_trace_count_dev.argtypes = [vp, C.c_void_p, C.c_size_t, C.c_int32, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint64)]
    L.tr_render_dev.restype = st
    L.tr_render_dev.argtypes = [vp, C.POINTER(TrCamera), C.POINTER(TrFilter), C.POINTER(TrRenderParams),
                                vp, vp, C.POINTER(TrStats)]
    L.tr_cancel.restype = st
    L.tr_cancel.argtypes = [vp]
    L.tr_selftest.restype = st
    L.tr_selftest.argtypes = [vp, C.c_int, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]
    _lib = L
    return L


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class GpuContext:
    """One tr_ctx on a CUDA device."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = C.c_void_p()
        s = self.L.tr_ctx_create(C.byref(h), device)
        if s != TR_OK:
            raise TracerError(s, "tr_ctx_create failed (no usable CUDA device?)")
        self.h = h
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            self.L.tr_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s):
        if s != TR_OK:
            raise TracerError(s, self.L.tr_ctx_last_error(self.h).decode())

    @property
    def stream(self) -> int:
        return self.L.tr_ctx_stream(self.h)

    def synchronize(self):
        self._check(self.L.tr_synchronize(self.h))

    def upload(self, scene_buffers):
        d = scene_buffers.desc()
        self._keep = (scene_buffers, d)
        self._check(self.L.tr_scene_upload(self.h, C.byref(d)))

    def bvh(self):
        nn, npr = C.c_size_t(), C.c_size_t()
        self._check(self.L.tr_bvh_info(self.h, C.byref(nn), C.byref(npr)))
        nodes = np.zeros(nn.value, NODE_DTYPE)
        order = np.zeros(npr.value, np.uint32)
        self._check(self.L.tr_bvh_export(self.h, _p(nodes, TrBvhNode32), _p(order, C.c_uint32)))
        return nodes, order

    def upload_bvh(self, nodes, order):
        nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
        order = np.ascontiguousarray(order, np.uint32)
        self._check(self.L.tr_bvh_upload(self.h, _p(nodes, TrBvhNode32), len(nodes), _p(order, C.c_uint32),
                                         len(order)))

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        prim = np.empty(len(rays), np.int32)
        t = np.empty(len(rays), np.float32)
        self._check(self.L.tr_trace_closest(self.h, _p(rays, TrRay), len(rays), _p(prim, C.c_int32),
                                            _p(t, C.c_float)))
        return prim, t

    def trace_any(self, rays):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hit = np.empty(len(rays), np.uint8)
        self._check(self.L.tr_trace_any(self.h, _p(rays, TrRay), len(rays), _p(hit, C.c_uint8)))
        return hit

    def trace_closest_dev(self, d_rays: int, n: int, d_prim: int, d_t: int):
        self._check(self.L.tr_trace_closest_dev(self.h, d_rays, n, d_prim, d_t))

    def trace_any_dev(self, d_rays: int, n: int, d_hit: int):
        self._check(self.L.tr_trace_any_dev(self.h, d_rays, n, d_hit))

    def render(self, cam: TrCamera, filt: TrFilter, params: TrRenderParams, fp64: bool = False):
        """Film sums (H, W, 4): r, g, b, weight; plus the run statistics."""
        W, H = params.width, params.height
        stats = TrStats()
        if fp64:
            out = np.zeros((H, W, 4), np.float64)
            s = self.L.tr_render(self.h, C.byref(cam), C.byref(filt), C.byref(params), None,
                                 _p(out, C.c_double), C.byref(stats))
        else:
            out = np.zeros((H, W, 4), np.float32)
            s = self.L.tr_render(self.h, C.byref(cam), C.byref(filt), C.byref(params), _p(out, C.c_float),
                                 None, C.byref(stats))
        self._check(s)
        return out, stats

    def tuning(self) -> TrTuning:
        t = TrTuning()
        self._check(self.L.tr_ctx_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, refill: int | None = None, trav_blocks_per_sm: int | None = None,
                   shade_blocks_per_sm: int | None = None, graph_iterations: int | None = None,
                   any_node_width: int | None = None, ray_bin_bits: int | None = None,
                   treelet_nodes: int | None = None, occluder_cache: int | None = None,
                   render_mode: int | None = None, any_hit_order: int | None = None) -> None:
        t = self.tuning()
        if any_hit_order is not None:
            t.any_hit_order = any_hit_order
        if render_mode is not None:
            t.render_mode = render_mode
        if occluder_cache is not None:
            t.occluder_cache = occluder_cache
        if ray_bin_bits is not None:
            t.ray_bin_bits = ray_bin_bits
        if treelet_nodes is not None:
            t.treelet_nodes = treelet_nodes
        if any_node_width is not None:
            t.any_node_width = any_node_width
        if graph_iterations is not None:
            t.graph_iterations = graph_iterations
        if refill is not None:
            t.trav_refill_lanes = refill
        if trav_blocks_per_sm is not None:
            t.trav_blocks_per_sm = trav_blocks_per_sm
        if shade_blocks_per_sm is not None:
            t.shade_blocks_per_sm = shade_blocks_per_sm
        self._check(self.L.tr_ctx_set_tuning(self.h, C.byref(t)))

    def set_bvh_builder(self, device: bool) -> None:
        """Builder of later uploads: the reference's host tree (False) or the device tree (True)."""
        self._check(self.L.tr_ctx_set_bvh_builder(self.h, 1 if device else 0))

    def bvh_stats(self) -> tuple[int, int]:
        """(builder of the uploaded tree: 0 reference, 1 device; its depth)."""
        b, d = C.c_int32(), C.c_int32()
        self._check(self.L.tr_bvh_stats(self.h, C.byref(b), C.byref(d)))
        return b.value, d.value

    # ---- output path (device buffers, ordered on the context's stream)
    def film_resolve_dev(self, d_film: int, pixels: int, d_rgb: int, fp64: bool = False) -> None:
        self._check(self.L.tr_film_resolve_dev(self.h, None if fp64 else d_film, d_film if fp64 else None, pixels, d_rgb))

    def aces_tone_map_dev(self, d_rgb: int, pixels: int, exposure: float) -> None:
        self._check(self.L.tr_aces_tone_map_dev(self.h, d_rgb, pixels, exposure))

    def gamma_correct_dev(self, d_rgb: int, pixels: int, gamma: float) -> None:
        self._check(self.L.tr_gamma_correct_dev(self.h, d_rgb, pixels, gamma))

    def to_rgb8_dev(self, d_rgb: int, pixels: int, d_out: int, inv_gamma: float = 1.0 / 2.2) -> None:
        self._check(self.L.tr_to_rgb8_dev(self.h, d_rgb, pixels, inv_gamma, d_out))

    def to_rgbe_dev(self, d_rgb: int, pixels: int, d_out: int) -> None:
        self._check(self.L.tr_to_rgbe_dev(self.h, d_rgb, pixels, d_out))

    def any_tree_info(self) -> tuple[int, int]:
        """(four-wide any-hit tree nodes, its traversal stack bound)."""
        n, b = C.c_uint64(), C.c_int32()
        self._check(self.L.tr_any_tree_info(self.h, C.byref(n), C.byref(b)))
        return n.value, b.value

    # ---- path-guiding model
    GUIDE_PARAMS = 15592
    GUIDE_LOG_KAPPA = (-4.0, 7.0)  # TR_GUIDE_LOG_KAPPA_MIN / _MAX

    def guide_init(self, seed: int = 0) -> None:
        self._check(self.L.tr_guide_init(self.h, seed))

    def guide_set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        self._check(self.L.tr_guide_set_params(self.h, _p(p, C.c_float), p.size))

    def guide_params(self) -> np.ndarray:
        p = np.zeros(self.GUIDE_PARAMS, np.float32)
        self._check(self.L.tr_guide_get_params(self.h, _p(p, C.c_float), p.size))
        return p

    def guide_forward_dev(self, d_in: int, n: int, d_out: int) -> None:
        self._check(self.L.tr_guide_forward_dev(self.h, d_in, n, d_out))

    def guide_backward_dev(self, d_in: int, d_dout: int, n: int, d_grads: int) -> None:
        self._check(self.L.tr_guide_backward_dev(self.h, d_in, d_dout, n, d_grads))

    def guide_loss_dev(self, d_in: int, d_dir: int, d_w: int, n: int, d_dout: int) -> float:
        loss = C.c_float()
        self._check(self.L.tr_guide_loss_dev(self.h, d_in, d_dir, d_w, n, d_dout, C.byref(loss)))
        return loss.value

    def guide_train_step_dev(self, d_in: int, d_dir: int, d_w: int, n: int, lr: float = 1e-3) -> float:
        loss = C.c_float()
        self._check(self.L.tr_guide_train_step_dev(self.h, d_in, d_dir, d_w, n, lr, C.byref(loss)))
        return loss.value

    def render_guided_dev(self, cam: TrCamera, filt: TrFilter, params: TrRenderParams, guide: TrGuideParams,
                          d_out: int, fp64: bool = False) -> TrStats:
        stats = TrStats()
        self._check(self.L.tr_render_guided_dev(self.h, C.byref(cam), C.byref(filt), C.byref(params), C.byref(guide),
                                                None if fp64 else d_out, d_out if fp64 else None, C.byref(stats)))
        return stats

    def guide_train_on_records(self, steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_float()
        self._check(self.L.tr_guide_train_on_records(self.h, steps, batch, lr, seed, C.byref(loss)))
        return loss.value

    def guide_light_init(self, grid=(32, 16, 24), bins: int = 8) -> None:
        """Light table of learned light sampling (statistics zero, distributions uniform)."""
        g = (C.c_int32 * 3)(*grid)
        self._check(self.L.tr_guide_light_init(self.h, g, bins))

    def guide_light_update(self, uniform_share: float = 0.2) -> None:
        """Recorded light-sample statistics -> the table's sampling distributions."""
        self._check(self.L.tr_guide_light_update(self.h, uniform_share))

    def upload_set(self, scenes) -> None:
        """Uploads a scene set (list of SceneBuffers) for batched rendering."""
        descs = (TrSceneDesc * len(scenes))(*[sb.desc() for sb in scenes])
        self._keep_set = (scenes, descs)
        self._check(self.L.tr_scene_set_upload(self.h, descs, len(scenes)))

    def render_batch_dev(self, jobs) -> TrStats:
        """jobs: list of (scene index, camera, filter, params, device film pointer)."""
        arr = self._jobs(jobs)
        stats = TrStats()
        self._check(self.L.tr_render_batch_dev(self.h, arr, len(jobs), C.byref(stats)))
        return stats

    @staticmethod
    def _jobs(jobs):
        arr = (TrBatchJob * len(jobs))()
        for k, (scene, cam, filt, par, film) in enumerate(jobs):
            arr[k].scene = scene
            arr[k].camera = cam
            arr[k].filter = filt
            arr[k].params = par
            arr[k].d_rgbw = film
        return arr

    def autotune(self, jobs, probe_spp: int = 2):
        """Tunes the launch settings on (a short version of) a batch; returns (tuning, ms)."""
        best, ms = TrTuning(), C.c_double()
        self._check(self.L.tr_autotune(self.h, self._jobs(jobs), len(jobs), probe_spp, C.byref(best), C.byref(ms)))
        return best, ms.value

    def trace_count_dev(self, d_rays: int, n: int, any_hit: bool):
        """(boxes, primitives) tested by the traversal of n device rays."""
        b, p = C.c_uint64(), C.c_uint64()
        self._check(self.L.tr_trace_count_dev(self.h, d_rays, n, 1 if any_hit else 0, C.byref(b), C.byref(p)))
        return b.value, p.value

    def render_dev(self, cam: TrCamera, filt: TrFilter, params: TrRenderParams, d_out: int, fp64: bool = False):
        stats = TrStats()
        s = self.L.tr_render_dev(self.h, C.byref(cam), C.byref(filt), C.byref(params),
                                 None if fp64 else d_out, d_out if fp64 else None, C.byref(stats))
        self._check(s)
        return stats


def selftest(ctx: "GpuContext", which: int, n: int, seed: int = 1) -> int:
    bad = C.c_uint64()
    ctx._check(ctx.L.tr_selftest(ctx.h, which, n, seed, C.byref(bad)))
    return bad.value


def make_ray(o, d, t_min=0.0, t_max=3.4028234663852886e38) -> TrRay:
    r = TrRay()
    oa = (C.c_float * 3)(*o)
    da = (C.c_float * 3)(*d)
    s = lib().tr_make_ray(oa, da, t_min, t_max, C.byref(r))
    if s != TR_OK:
        raise TracerError(s, "tr_make_ray")
    return r


def write_png(path: str, rgb8: np.ndarray) -> None:
    """(H, W, 3) uint8 image to an 8-bit RGB PNG (tr_write_png; host only)."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    s = lib().tr_write_png(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0])
    if s != TR_OK:
        raise TracerError(s, f"tr_write_png failed for {path}")


def write_hdr(path: str, rgbe: np.ndarray) -> None:
    """(H, W, 4) uint8 RGBE image to a Radiance HDR file (tr_write_hdr; host only)."""
    a = np.ascontiguousarray(rgbe, np.uint8)
    s = lib().tr_write_hdr(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0])
    if s != TR_OK:
        raise TracerError(s, f"tr_write_hdr failed for {path}")
