"""ctypes mirror of include/tracer_gpu.h (the C ABI of the GPU path).

The structures here are byte-for-byte the C structs; `SceneBuffers` keeps the
numpy arrays a `tr_scene_desc` points into alive for as long as it is used.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

TR_OK = 0
TR_ERR_ARG = 1
TR_ERR_OOM = 2
TR_ERR_QUEUE_OVERFLOW = 3
TR_ERR_TIMEOUT = 4
TR_ERR_CUDA = 5
TR_ERR_STATE = 6
TR_ERR_CANCELLED = 7
TR_ERR_UNSUPPORTED = 8

TR_MAT_PHONG = 0
TR_MAT_DISNEY12 = 1
TR_MAT_GLASS = 2
TR_MAT_METAL = 3
TR_MAT_DISNEY15 = 4

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)
u8p = C.POINTER(C.c_uint8)


class TrRay(C.Structure):
    _fields_ = [("o", C.c_float * 3), ("d", C.c_float * 3), ("t_min", C.c_float), ("t_max", C.c_float)]


RAY_DTYPE = np.dtype([("o", "<f4", 3), ("d", "<f4", 3), ("t_min", "<f4"), ("t_max", "<f4")])
assert RAY_DTYPE.itemsize == C.sizeof(TrRay) == 32


class TrBvhNode32(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("offset", C.c_int32),
                ("count", C.c_uint16), ("axis", C.c_uint8), ("pad", C.c_uint8)]


NODE_DTYPE = np.dtype([("lo", "<f4", 3), ("hi", "<f4", 3), ("offset", "<i4"), ("count", "<u2"),
                       ("axis", "u1"), ("pad", "u1")])
assert NODE_DTYPE.itemsize == C.sizeof(TrBvhNode32) == 32


class TrMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ka", C.c_float * 3), ("kd", C.c_float * 3), ("ks", C.c_float * 3),
                ("ns", C.c_float), ("base_color", C.c_float * 3),
                ("subsurface", C.c_float), ("metallic", C.c_float), ("specular", C.c_float),
                ("specular_tint", C.c_float), ("roughness", C.c_float), ("anisotropic", C.c_float),
                ("sheen", C.c_float), ("sheen_tint", C.c_float), ("clearcoat", C.c_float),
                ("clearcoat_gloss", C.c_float), ("kr", C.c_float * 3), ("kt", C.c_float * 3), ("ior", C.c_float),
                ("color", C.c_float * 3), ("eta", C.c_float * 3), ("k", C.c_float * 3),
                ("transmission", C.c_float), ("transmission_roughness", C.c_float),
                ("specular_scale", C.c_float * 3),
                ("tex_ka", C.c_uint32), ("tex_kd", C.c_uint32), ("tex_ks", C.c_uint32), ("tex_ns", C.c_uint32),
                ("tex_param", C.c_uint32 * 13)]


class TrTexture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("texels", f32p),
                ("texels8", C.POINTER(C.c_uint8))]


class TrSceneDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", f32p), ("normals", f32p), ("uvs", f32p),
                ("num_triangles", C.c_uint32), ("indices", i32p),
                ("num_spheres", C.c_uint32), ("sphere_radius", f32p), ("sphere_to_world", f32p),
                ("sphere_to_local", f32p),
                ("num_materials", C.c_uint32), ("materials", C.POINTER(TrMaterial)),
                ("num_prims", C.c_uint32), ("prim_shape", i32p), ("prim_material", i32p),
                ("prim_emission", f32p),
                ("num_lights", C.c_uint32), ("light_prims", i32p),
                ("max_leaf_prims", C.c_int32),
                ("env_width", C.c_uint32), ("env_height", C.c_uint32), ("env_texels", f32p),
                ("env_to_light", f32p), ("env_to_world", f32p), ("env_texels8", C.POINTER(C.c_uint8)),
                ("num_textures", C.c_uint32), ("textures", C.POINTER(TrTexture))]


class TrCamera(C.Structure):
    _fields_ = [("film_aspect", C.c_float), ("pos", C.c_float * 3), ("target", C.c_float * 3),
                ("up", C.c_float * 3), ("fov", C.c_float), ("lens_radius", C.c_float),
                ("focal_dist", C.c_float)]


class TrFilter(C.Structure):
    _fields_ = [("radius", C.c_float), ("alpha", C.c_float)]


class TrRenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("min_depth", C.c_int32), ("max_depth", C.c_int32),
                ("direct_light_sample_num", C.c_int32), ("seed_base", C.c_uint32), ("flags", C.c_uint32)]


TR_RENDER_TIME_STAGES = 1
TR_RENDER_COUNT_VISITS = 2
STAGE_NAMES = ["extend", "logic", "material_phong", "material_disney", "nee_phong", "nee_disney", "shadow",
               "reset", "bin"]


class TrStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("shade_items", C.c_uint64), ("iterations", C.c_uint64), ("device_ms", C.c_double),
                ("stage_ms", C.c_double * 9), ("closest_boxes", C.c_uint64), ("closest_prims", C.c_uint64),
                ("any_boxes", C.c_uint64), ("any_prims", C.c_uint64), ("guide_records", C.c_uint64),
                ("occluder_hits", C.c_uint64)]


class TrGuideParams(C.Structure):
    _fields_ = [("alpha", C.c_float), ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("record", C.c_int32),
                ("max_records", C.c_uint32), ("light_guide", C.c_int32), ("light_record", C.c_int32),
                ("max_depth", C.c_int32)]


TR_RENDER_MODE_AUTO, TR_RENDER_MODE_WAVEFRONT, TR_RENDER_MODE_PERSISTENT = 0, 1, 2


class TrTuning(C.Structure):
    _fields_ = [("trav_refill_lanes", C.c_int32), ("trav_blocks_per_sm", C.c_int32),
                ("shade_blocks_per_sm", C.c_int32), ("graph_iterations", C.c_int32),
                ("any_node_width", C.c_int32), ("ray_bin_bits", C.c_int32), ("treelet_nodes", C.c_int32),
                ("occluder_cache", C.c_int32), ("render_mode", C.c_int32), ("any_hit_order", C.c_int32)]


class TrBatchJob(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("camera", TrCamera), ("filter", TrFilter), ("params", TrRenderParams),
                ("d_rgbw", C.c_void_p)]


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Material:
    """One tr_material. kind=TR_MAT_PHONG uses ka/kd/ks/ns; Disney12 base_color .. clearcoat_gloss;
    TR_MAT_GLASS kr/kt/ior; TR_MAT_METAL color/eta/k with roughness/anisotropic; TR_MAT_DISNEY15
    base_color, metallic, roughness, transmission, transmission_roughness, ior, specular_scale,
    specular_tint, anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss."""
    kind: int = TR_MAT_PHONG
    ka: tuple = (0.0, 0.0, 0.0)
    kd: tuple = (0.0, 0.0, 0.0)
    ks: tuple = (0.0, 0.0, 0.0)
    ns: float = 1.0
    base_color: tuple = (0.0, 0.0, 0.0)
    subsurface: float = 0.0
    metallic: float = 0.0
    specular: float = 0.0
    specular_tint: float = 0.0
    roughness: float = 0.0
    anisotropic: float = 0.0
    sheen: float = 0.0
    sheen_tint: float = 0.0
    clearcoat: float = 0.0
    clearcoat_gloss: float = 0.0
    kr: tuple = (0.0, 0.0, 0.0)
    kt: tuple = (0.0, 0.0, 0.0)
    ior: float = 1.0
    color: tuple = (0.0, 0.0, 0.0)
    eta: tuple = (0.0, 0.0, 0.0)
    k: tuple = (0.0, 0.0, 0.0)
    transmission: float = 0.0
    transmission_roughness: float = 0.0
    specular_scale: tuple = (0.0, 0.0, 0.0)
    tex_ka: int = 0  # Phong maps: 0 the constant, k the scene's textures[k - 1]
    tex_kd: int = 0
    tex_ks: int = 0
    tex_ns: int = 0
    # maps of the other kinds, per factory argument in the factory's order (tr_material.tex_param)
    tex_param: tuple = (0,) * 13

    def to_c(self) -> TrMaterial:
        m = TrMaterial()
        m.kind = self.kind
        m.ka[:] = self.ka
        m.kd[:] = self.kd
        m.ks[:] = self.ks
        m.ns = self.ns
        m.base_color[:] = self.base_color
        for k in ("subsurface", "metallic", "specular", "specular_tint", "roughness", "anisotropic",
                  "sheen", "sheen_tint", "clearcoat", "clearcoat_gloss", "ior", "transmission",
                  "transmission_roughness"):
            setattr(m, k, getattr(self, k))
        m.kr[:] = self.kr
        m.kt[:] = self.kt
        m.color[:] = self.color
        m.specular_scale[:] = self.specular_scale
        m.tex_ka, m.tex_kd, m.tex_ks, m.tex_ns = self.tex_ka, self.tex_kd, self.tex_ks, self.tex_ns
        m.eta[:] = self.eta
        m.k[:] = self.k
        for i, t in enumerate(self.tex_param):
            m.tex_param[i] = t
        return m


@dataclass
class SceneBuffers:
    """Owns the arrays of one scene and hands out a tr_scene_desc over them."""
    positions: np.ndarray            # (V,3) f32
    normals: np.ndarray              # (V,3) f32
    uvs: np.ndarray                  # (V,2) f32
    indices: np.ndarray              # (T,3) i32
    sphere_radius: np.ndarray        # (S,) f32
    sphere_to_world: np.ndarray      # (S,16) f32
    sphere_to_local: np.ndarray      # (S,16) f32
    materials: list                  # [Material]
    prim_shape: np.ndarray           # (P,) i32
    prim_material: np.ndarray        # (P,) i32
    prim_emission: np.ndarray        # (P,3) f32
    light_prims: np.ndarray          # (L,) i32
    max_leaf_prims: int = 3
    env_texels: np.ndarray | None = None    # (H,W,3) f32 environment map, row y at v = y / (H - 1)
    env_texels8: np.ndarray | None = None   # (H,W,3) u8 map (ImageTexture2D) used instead when set
    textures: list = field(default_factory=list)  # (H,W,3) f32 (HDR) or u8 (8-bit) images for tex_* fields
    env_to_light: np.ndarray | None = None  # (16,) f32 world_to_light; identity when None
    env_to_world: np.ndarray | None = None  # (16,) f32 its inverse
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> TrSceneDesc:
        arrs = {}
        for name in ("positions", "normals", "uvs", "sphere_radius", "sphere_to_world", "sphere_to_local",
                     "prim_emission"):
            arrs[name] = np.ascontiguousarray(getattr(self, name), dtype=np.float32)
        for name in ("indices", "prim_shape", "prim_material", "light_prims"):
            arrs[name] = np.ascontiguousarray(getattr(self, name), dtype=np.int32)
        mats = (TrMaterial * max(1, len(self.materials)))(*[m.to_c() for m in self.materials])
        self._keep = [arrs, mats]
        d = TrSceneDesc()
        d.num_vertices = len(arrs["positions"])
        d.positions = ptr(arrs["positions"], C.c_float)
        d.normals = ptr(arrs["normals"], C.c_float)
        d.uvs = ptr(arrs["uvs"], C.c_float)
        d.num_triangles = len(arrs["indices"])
        d.indices = ptr(arrs["indices"], C.c_int32)
        d.num_spheres = len(arrs["sphere_radius"])
        d.sphere_radius = ptr(arrs["sphere_radius"], C.c_float)
        d.sphere_to_world = ptr(arrs["sphere_to_world"], C.c_float)
        d.sphere_to_local = ptr(arrs["sphere_to_local"], C.c_float)
        d.num_materials = len(self.materials)
        d.materials = C.cast(mats, C.POINTER(TrMaterial))
        d.num_prims = len(arrs["prim_shape"])
        d.prim_shape = ptr(arrs["prim_shape"], C.c_int32)
        d.prim_material = ptr(arrs["prim_material"], C.c_int32)
        d.prim_emission = ptr(arrs["prim_emission"], C.c_float)
        d.num_lights = len(arrs["light_prims"])
        d.light_prims = ptr(arrs["light_prims"], C.c_int32)
        d.max_leaf_prims = int(self.max_leaf_prims)
        if self.textures:
            recs = (TrTexture * len(self.textures))()
            for i, img in enumerate(self.textures):
                eight = np.asarray(img).dtype == np.uint8
                arr = np.ascontiguousarray(img, dtype=np.uint8 if eight else np.float32)
                if arr.ndim != 3 or arr.shape[2] != 3:
                    raise ValueError("textures must be (height, width, 3)")
                self._keep.append(arr)
                recs[i].height, recs[i].width = arr.shape[0], arr.shape[1]
                if eight:
                    recs[i].texels8 = arr.ctypes.data_as(C.POINTER(C.c_uint8))
                else:
                    recs[i].texels = ptr(arr, C.c_float)
            self._keep.append(recs)
            d.num_textures = len(self.textures)
            d.textures = C.cast(recs, C.POINTER(TrTexture))
        if self.env_texels is not None or self.env_texels8 is not None:
            ldr = self.env_texels is None
            tex = np.ascontiguousarray(self.env_texels8 if ldr else self.env_texels,
                                       dtype=np.uint8 if ldr else np.float32)
            if tex.ndim != 3 or tex.shape[2] != 3:
                raise ValueError("environment texels must be (height, width, 3)")
            eye = np.eye(4, dtype=np.float32).ravel()
            to_l = np.ascontiguousarray(eye if self.env_to_light is None else self.env_to_light, dtype=np.float32)
            to_w = np.ascontiguousarray(eye if self.env_to_world is None else self.env_to_world, dtype=np.float32)
            self._keep += [tex, to_l, to_w]
            d.env_height, d.env_width = tex.shape[0], tex.shape[1]
            if ldr:
                d.env_texels8 = tex.ctypes.data_as(C.POINTER(C.c_uint8))
            else:
                d.env_texels = ptr(tex, C.c_float)
            d.env_to_light = ptr(to_l, C.c_float)
            d.env_to_world = ptr(to_w, C.c_float)
        return d


def make_camera(aspect, pos, target, up, fov_rad, lens_radius=0.0, focal_dist=1.0) -> TrCamera:
    c = TrCamera()
    c.film_aspect = aspect
    c.pos[:] = pos
    c.target[:] = target
    c.up[:] = up
    c.fov = fov_rad
    c.lens_radius = lens_radius
    c.focal_dist = focal_dist
    return c


def make_filter(radius=0.5, alpha=0.6) -> TrFilter:
    f = TrFilter()
    f.radius = radius
    f.alpha = alpha
    return f


def make_guide(alpha: float, box_lo, box_hi, record: bool | int = False, max_records: int = 0,
               light_guide: bool = False, light_record: bool = False, max_depth: int = 0) -> "TrGuideParams":
    """record: False/0 none, True/1 every sample, n the first of every n samples of a pixel;
    light_guide / light_record: learned light sampling from / statistics into the light table;
    max_depth: guide vertices at path depth < max_depth only (0: all)."""
    g = TrGuideParams()
    g.max_depth = max_depth
    g.light_guide = int(light_guide)
    g.light_record = int(light_record)
    g.alpha = alpha
    g.box_lo[:] = box_lo
    g.box_hi[:] = box_hi
    g.record = int(record)
    g.max_records = max_records
    return g


def make_params(width, height, spp, min_depth, max_depth, seed_base=0, direct_light_sample_num=1, flags=0):
    p = TrRenderParams()
    p.flags = flags
    p.width, p.height, p.spp = width, height, spp
    p.min_depth, p.max_depth = min_depth, max_depth
    p.direct_light_sample_num = direct_light_sample_num
    p.seed_base = seed_base
    return p
