"""Seeded synthetic workloads with the shapes of the reference's configurations.

The reference ships no scene data (its OBJ demo scenes are not in its
repository), so every workload here is procedural and seeded:

* ``cornell``      -- Cornell box, 36 triangles, 2 emissive triangles, Lambert
                      (Phong with ks = 0) walls, pinhole camera at (0,0,3.5).
* ``traversal``    -- 1,048,576 random small triangles in the unit cube and
                      rays from the cube surface (closest-hit and shadow).
* ``disney_grid``  -- 16x16 Disney12 spheres on a ground quad, two 2x2 area
                      lights at height 6.
* ``random_scene`` -- small mixed triangle/sphere scenes for parity tests.

Vertex data is emitted in world space exactly as ``tr_scene_desc`` wants it.
Vertex normals are made fixed points of the reference's normalisation
(``normalize(normalize(n)) == normalize(n)``): the reference re-normalises the
stored mesh normals in place on every hit (src/shape/triangle.cpp:182-184), so
only fixed points keep its results independent of hit order.
"""
from __future__ import annotations

import math

import numpy as np

from .abi import (RAY_DTYPE, TR_MAT_DISNEY12, TR_MAT_DISNEY15, TR_MAT_GLASS, TR_MAT_METAL, TR_MAT_PHONG, Material, SceneBuffers, make_camera,
                  make_filter, make_params)

F32_MAX = np.float32(np.finfo(np.float32).max)


def ref_normalize(v: np.ndarray) -> np.ndarray:
    """The reference's normalize (src/utility/geometry.hpp:429-445,570-572),
    vectorised: float32 sum of squares left to right, double sqrt, double
    reciprocal, double product, rounded to float32. Each numpy ufunc is one
    IEEE operation, so nothing fuses."""
    v = np.asarray(v, dtype=np.float32)
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    s = np.multiply(x, x, dtype=np.float32)
    s = np.add(s, np.multiply(y, y, dtype=np.float32), dtype=np.float32)
    s = np.add(s, np.multiply(z, z, dtype=np.float32), dtype=np.float32)
    length = np.sqrt(s.astype(np.float64))
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.float64(1.0) / length
        out = np.stack([(x.astype(np.float64) * inv).astype(np.float32),
                        (y.astype(np.float64) * inv).astype(np.float32),
                        (z.astype(np.float64) * inv).astype(np.float32)], axis=-1)
    return out


def fixed_normal(n) -> np.ndarray:
    """Unit normal that the reference's normalize maps to itself."""
    v0 = np.asarray(n, dtype=np.float64)
    v0 = (v0 / np.linalg.norm(v0)).astype(np.float32)
    for attempt in range(64):
        # some directions cycle under the rounding; nudge one component by ulps
        v = v0.copy()
        if attempt:
            k = attempt % 3
            v[k] = np.nextafter(v[k], np.float32(np.inf) if attempt % 2 else np.float32(-np.inf))
            v0 = v.copy()
        for _ in range(8):
            w = ref_normalize(v)
            if np.array_equal(w.view(np.uint32), v.view(np.uint32)):
                return v
            v = w
    raise ValueError(f"no fixed point for normal {n}")


def settle_normals(n: np.ndarray) -> np.ndarray:
    """Vectorised fixed_normal: each row normalised, then iterated to a fixed
    point of the reference's normalize (rows caught in a 2-cycle get an ulp
    nudge, as fixed_normal does)."""
    v = ref_normalize(np.asarray(n, dtype=np.float64).astype(np.float32))
    for attempt in range(64):
        for _ in range(8):
            w = ref_normalize(v)
            if np.array_equal(w.view(np.uint32), v.view(np.uint32)):
                return v
            v = w
        bad = np.nonzero((ref_normalize(v).view(np.uint32) != v.view(np.uint32)).any(-1))[0]
        k = attempt % 3
        v[bad, k] = np.nextafter(v[bad, k], np.float32(np.inf) if attempt % 2 else np.float32(-np.inf))
    raise ValueError("normals without a fixed point")


def make_rays(o: np.ndarray, d: np.ndarray, t_min, t_max) -> np.ndarray:
    """Rays through the reference Ray constructor (direction normalised in double)."""
    n = len(o)
    r = np.zeros(n, dtype=RAY_DTYPE)
    r["o"] = np.asarray(o, dtype=np.float32)
    r["d"] = ref_normalize(d)
    r["t_min"] = t_min
    r["t_max"] = t_max
    return r


class _Builder:
    """Accumulates primitives as array chunks; finish() concatenates them."""

    def __init__(self):
        self.pos, self.nrm, self.uv, self.idx = [], [], [], []
        self.nv = 0  # vertices so far
        self.nt = 0  # triangles so far
        self.sph_r, self.sph_m, self.sph_inv = [], [], []
        self.mats: list[Material] = []
        self.prim_shape, self.prim_mat, self.prim_em = [], [], []
        self.lights = []
        self.np = 0  # primitives so far

    def material(self, m: Material) -> int:
        self.mats.append(m)
        return len(self.mats) - 1

    def _prims(self, shapes, mat, emission):
        k = len(shapes)
        self.prim_shape.append(np.asarray(shapes, np.int32))
        self.prim_mat.append(np.full(k, mat, np.int32))
        self.prim_em.append(np.tile(np.asarray(emission, np.float32), (k, 1)))
        first = self.np
        self.np += k
        return first

    def triangle(self, a, b, c, n, mat, emission=(0, 0, 0), uvs=((0, 0), (1, 0), (1, 1)), light=None):
        nn = fixed_normal(n)
        self.pos.append(np.asarray([a, b, c], dtype=np.float32).reshape(3, 3) + np.float32(0))  # no -0.0
        self.nrm.append(np.tile(nn, (3, 1)))
        self.uv.append(np.asarray(uvs, dtype=np.float32))
        self.idx.append(np.array([[self.nv, self.nv + 1, self.nv + 2]], np.int32))
        self.nv += 3
        pid = self._prims([self.nt], mat, emission)
        self.nt += 1
        if any(e != 0 for e in emission) and light is not False:
            self.lights.append(pid)
        return pid

    def quad(self, p0, p1, p2, p3, normal, mat, emission=(0, 0, 0)):
        """Two triangles (p0,p1,p2), (p0,p2,p3), wound so cross(AB, AC) points along normal."""
        p0, p1, p2, p3 = (np.asarray(p, dtype=np.float64) for p in (p0, p1, p2, p3))
        if np.dot(np.cross(p1 - p0, p2 - p0), normal) < 0:
            p1, p3 = p3, p1
        self.triangle(p0, p1, p2, normal, mat, emission, ((0, 0), (1, 0), (1, 1)))
        self.triangle(p0, p2, p3, normal, mat, emission, ((0, 0), (1, 1), (0, 1)))

    def box(self, center, size, rot_y_deg, mat):
        c = np.asarray(center, dtype=np.float64)
        h = np.asarray(size, dtype=np.float64) / 2
        th = math.radians(rot_y_deg)
        R = np.array([[math.cos(th), 0, math.sin(th)], [0, 1, 0], [-math.sin(th), 0, math.cos(th)]])
        def P(sx, sy, sz):
            return c + R @ (h * np.array([sx, sy, sz], dtype=np.float64))
        for axis in range(3):
            for sgn in (-1, 1):
                n = np.zeros(3); n[axis] = sgn
                u_ax, v_ax = [a for a in range(3) if a != axis]
                corners = []
                for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                    s = [0, 0, 0]; s[axis] = sgn; s[u_ax] = su; s[v_ax] = sv
                    corners.append(P(*s))
                self.quad(*corners, R @ n, mat)

    def sphere(self, center, radius, mat):
        cx, cy, cz = (float(np.float32(v)) for v in center)
        # translate(delta) builds m and its explicit inverse (src/utility/transform.cpp:163-173)
        m = np.array([1, 0, 0, cx, 0, 1, 0, cy, 0, 0, 1, cz, 0, 0, 0, 1], dtype=np.float32)
        inv = np.array([1, 0, 0, -cx, 0, 1, 0, -cy, 0, 0, 1, -cz, 0, 0, 0, 1], dtype=np.float32)
        self.sph_r.append(radius)
        self.sph_m.append(m)
        self.sph_inv.append(inv)
        return self._prims([~(len(self.sph_r) - 1)], mat, (0, 0, 0))

    def mesh(self, tris: np.ndarray, normals: np.ndarray, mat: int, settle: bool = True):
        """Bulk triangles: tris (T, 3, 3) positions, normals (T, 3, 3) per
        vertex (settled to fixed points of the reference normalize unless
        settle is False; the upload normalises them either way)."""
        T = len(tris)
        if T == 0:
            return
        self.pos.append(np.asarray(tris, np.float32).reshape(-1, 3) + np.float32(0))
        n = np.asarray(normals, np.float64).reshape(-1, 3)
        self.nrm.append(settle_normals(n) if settle else (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32))
        self.uv.append(np.tile(np.array([[0, 0], [1, 0], [1, 1]], np.float32), (T, 1)))
        self.idx.append((self.nv + 3 * np.arange(T, dtype=np.int64)[:, None] + np.arange(3)[None, :]).astype(np.int32))
        self.nv += 3 * T
        self._prims(np.arange(self.nt, self.nt + T), mat, (0, 0, 0))
        self.nt += T

    def finish(self, max_leaf_prims: int) -> SceneBuffers:
        def cat(chunks, cols, dt):
            return np.concatenate(chunks).astype(dt, copy=False) if chunks else np.zeros((0, cols), dt)

        def arr(x, shape, dt):
            return np.asarray(x, dtype=dt).reshape(shape) if len(x) else np.zeros(tuple(0 if d < 0 else d for d in shape), dtype=dt)
        return SceneBuffers(
            positions=cat(self.pos, 3, np.float32), normals=cat(self.nrm, 3, np.float32),
            uvs=cat(self.uv, 2, np.float32), indices=cat(self.idx, 3, np.int32),
            sphere_radius=arr(self.sph_r, (-1,), np.float32), sphere_to_world=arr(self.sph_m, (-1, 16), np.float32),
            sphere_to_local=arr(self.sph_inv, (-1, 16), np.float32), materials=self.mats,
            prim_shape=np.concatenate(self.prim_shape).astype(np.int32) if self.prim_shape else np.zeros(0, np.int32),
            prim_material=np.concatenate(self.prim_mat).astype(np.int32) if self.prim_mat else np.zeros(0, np.int32),
            prim_emission=(np.concatenate(self.prim_em).astype(np.float32) if self.prim_em
                           else np.zeros((0, 3), np.float32)),
            light_prims=arr(self.lights, (-1,), np.int32), max_leaf_prims=max_leaf_prims)


def lambert(albedo) -> Material:
    """create_phong_material(0, kd, 0, 1): the reference's Lambertian material."""
    return Material(kind=TR_MAT_PHONG, kd=tuple(albedo), ks=(0.0, 0.0, 0.0), ns=1.0)


def checker(n=16, cells=4, c0=(0.8, 0.8, 0.8), c1=(0.1, 0.3, 0.7), eight_bit=True):
    """An n x n checkerboard texture of `cells` x `cells` squares, 8-bit or float."""
    y, x = np.mgrid[0:n, 0:n]
    odd = ((x * cells // n + y * cells // n) % 2 == 1)[..., None]
    img = np.where(odd, np.array(c1), np.array(c0))
    return (img * 255.0).astype(np.uint8) if eight_bit else img.astype(np.float32)


def cornell(width=256, height=256, spp=16, max_depth=5, min_depth=5, glass=False, metal=False, textured=False):
    """Cornell box [-1,1]^3 open at +z: 10 wall triangles, two boxes (12 each),
    a 0.5x0.5 ceiling light at y = 0.99 emitting (17,12,4): 36 triangles,
    2 lights. Pinhole camera at (0,0,3.5), 40 degree fov. min_depth >= max_depth
    disables Russian roulette. glass: the tall box is glass (kr = kt = 1,
    ior 1.5), which takes paths through the specular branch. metal: the short
    box is a rough anisotropic metal (GGX with a painted conductor Fresnel).
    textured: the floor's kd is an 8-bit checkerboard, the back wall's kd, ks
    and ns float maps (Phong with image textures)."""
    b = _Builder()
    white = b.material(lambert((0.73, 0.73, 0.73)))
    floor, back = white, white
    textures = []
    if textured:
        textures = [checker(16, 4), checker(12, 3, (0.9, 0.2, 0.1), (0.2, 0.8, 0.3), eight_bit=False),
                    np.full((4, 4, 3), 0.15, np.float32),
                    np.linspace(5.0, 60.0, 8 * 8 * 3, dtype=np.float32).reshape(8, 8, 3)]
        floor = b.material(Material(kind=TR_MAT_PHONG, kd=(0.73, 0.73, 0.73), ns=1.0, tex_kd=1))
        back = b.material(Material(kind=TR_MAT_PHONG, kd=(0.5, 0.5, 0.5), ks=(0.1, 0.1, 0.1), ns=10.0,
                                   tex_kd=2, tex_ks=3, tex_ns=4))
    tall = b.material(Material(kind=TR_MAT_GLASS, kr=(1.0, 1.0, 1.0), kt=(1.0, 1.0, 1.0), ior=1.5)) if glass else white
    red = b.material(lambert((0.65, 0.05, 0.05)))
    green = b.material(lambert((0.12, 0.45, 0.15)))
    b.quad((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (0, 1, 0), floor)    # floor
    b.quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), (0, -1, 0), white)       # ceiling
    b.quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (0, 0, 1), back)     # back
    b.quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), (1, 0, 0), red)      # left
    b.quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), (-1, 0, 0), green)       # right
    short = b.material(Material(kind=TR_MAT_METAL, color=(0.95, 0.64, 0.54), eta=(0.2, 0.92, 1.1), k=(3.9, 2.45, 2.14),
                                roughness=0.35, anisotropic=0.4)) if metal else white
    b.box((-0.35, -0.7, -0.3), (0.6, 0.6, 0.6), 15.0, short)
    b.box((0.35, -0.4, 0.3), (0.6, 1.2, 0.6), -18.0, tall)
    b.quad((-0.25, 0.99, -0.25), (0.25, 0.99, -0.25), (0.25, 0.99, 0.25), (-0.25, 0.99, 0.25), (0, -1, 0),
           white, emission=(17.0, 12.0, 4.0))
    scene = b.finish(max_leaf_prims=3)
    scene.textures = textures
    cam = make_camera(width / height, (0, 0, 3.5), (0, 0, 0), (0, 1, 0), math.radians(40.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def disney_grid(width=1024, height=1024, spp=64, max_depth=8, min_depth=5, seed=0, n=16):
    """n x n Disney12 spheres (radius 0.4, spacing 1.0) on a 40x40 ground quad,
    parameters uniform in [0,1] from `seed` (sheen_tint fixed at 0.5), two 2x2
    area lights at height 6 emitting 8 (4 emissive triangles)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    ground = b.material(lambert((0.5, 0.5, 0.5)))
    b.quad((-20, 0, -20), (20, 0, -20), (20, 0, 20), (-20, 0, 20), (0, 1, 0), ground)
    for cx, cz in ((-3.0, -2.0), (3.0, 2.0)):
        b.quad((cx - 1, 6, cz - 1), (cx + 1, 6, cz - 1), (cx + 1, 6, cz + 1), (cx - 1, 6, cz + 1), (0, -1, 0),
               ground, emission=(8.0, 8.0, 8.0))
    for i in range(n):
        for j in range(n):
            p = rng.random(12).astype(np.float32)
            m = Material(kind=TR_MAT_DISNEY12, base_color=tuple(float(v) for v in p[0:3]),
                         metallic=float(p[3]), roughness=float(p[4]), specular=float(p[5]),
                         specular_tint=float(p[6]), sheen=float(p[7]), clearcoat=float(p[8]),
                         clearcoat_gloss=float(p[9]), anisotropic=float(p[10]), subsurface=float(p[11]),
                         sheen_tint=0.5)
            mat = b.material(m)
            b.sphere(((i - (n - 1) / 2) * 1.0, 0.4, (j - (n - 1) / 2) * 1.0), 0.4, mat)
    scene = b.finish(max_leaf_prims=3)
    cam = make_camera(width / height, (0, 9, 14), (0, 0, 0), (0, 1, 0), math.radians(45.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def sky_map(width=64, height=32, sun=(0.55, 1.2), sun_radiance=300.0):
    """A synthetic HDR environment map in the IBL's (u, v) = (phi / 2pi, theta / pi)
    layout (row y at theta = pi * y / (height - 1)): a sky brightening toward
    the horizon, a dim ground below it and a small sun disc of high radiance
    centred at (theta, phi) = `sun`."""
    y, x = np.mgrid[0:height, 0:width]
    theta = np.pi * y / max(height - 1, 1)
    phi = 2 * np.pi * x / max(width - 1, 1)
    t = np.clip(theta / (np.pi / 2), 0, 1)[..., None]
    sky = (1 - t) * np.array([0.25, 0.45, 0.9]) + t * np.array([0.9, 0.9, 1.0])
    ground = np.array([0.18, 0.14, 0.1]) * np.ones_like(sky)
    img = np.where((theta <= np.pi / 2)[..., None], sky, ground)
    d = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], -1)
    st, sp = sun
    s = np.array([np.sin(st) * np.cos(sp), np.sin(st) * np.sin(sp), np.cos(st)])
    img = img + np.where(((d @ s) > np.cos(0.12))[..., None], sun_radiance * np.array([1.0, 0.9, 0.75]), 0.0)
    return img.astype(np.float32)


def rotate_x(theta):
    """rotate_x (src/utility/transform.cpp:139-145) in float: the matrix and its
    transpose as the Transform's inverse, row-major."""
    s, c = np.float32(math.sin(np.float32(theta))), np.float32(math.cos(np.float32(theta)))
    m = np.array([1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1], dtype=np.float32)
    return m, np.ascontiguousarray(m.reshape(4, 4).T).ravel()


def outdoor(width=96, height=64, spp=8, max_depth=6, min_depth=3, env_size=(64, 32), area_light=True, glass=True,
            env_8bit=False, textured=False):
    """An open scene under an environment light: a ground quad, Disney12,
    metal, glass (Lambertian when `glass` is False) and Lambertian spheres,
    optionally one small area light; the
    sky map of `sky_map` with world +y as the light's +z (world_to_light =
    rotate_x(pi/2), as the reference's demo does)."""
    b = _Builder()
    ground = b.material(lambert((0.45, 0.42, 0.4)))
    b.quad((-6, 0, -6), (6, 0, -6), (6, 0, 6), (-6, 0, 6), (0, 1, 0), ground)
    if area_light:
        b.quad((1.5, 3, -0.5), (2.5, 3, -0.5), (2.5, 3, 0.5), (1.5, 3, 0.5), (0, -1, 0), ground,
               emission=(6.0, 6.0, 6.0))
    mats = [b.material(Material(kind=TR_MAT_DISNEY12, base_color=(0.8, 0.3, 0.2), metallic=0.2, roughness=0.4,
                                specular=0.5, clearcoat=0.5, clearcoat_gloss=0.7, sheen_tint=0.5)),
            b.material(Material(kind=TR_MAT_METAL, color=(0.95, 0.64, 0.54), eta=(0.2, 0.92, 1.1),
                                k=(3.9, 2.45, 2.14), roughness=0.25, anisotropic=0.0)),
            b.material(Material(kind=TR_MAT_GLASS, kr=(1.0, 1.0, 1.0), kt=(1.0, 1.0, 1.0), ior=1.5) if glass
                       else lambert((0.7, 0.7, 0.7))),
            b.material(Material(kind=TR_MAT_PHONG, kd=(0.2, 0.5, 0.3), ns=1.0, tex_kd=1 if textured else 0))]
    for k, m in enumerate(mats):
        b.sphere((-2.25 + 1.5 * k, 0.6, 0.0), 0.6, m)
    scene = b.finish(max_leaf_prims=3)
    if textured:  # the last sphere's kd: a checkerboard over its (phi, theta) uv
        scene.textures = [checker(32, 8, (0.9, 0.9, 0.2), (0.1, 0.2, 0.6))]
    if env_8bit:  # the map as 8-bit values (an ImageTexture2D), the sun at full scale
        scene.env_texels8 = np.clip(sky_map(*env_size, sun_radiance=1.0) * 255.0, 0, 255).astype(np.uint8)
    else:
        scene.env_texels = sky_map(*env_size)
    scene.env_to_light, scene.env_to_world = rotate_x(math.pi / 2)
    cam = make_camera(width / height, (0, 1.6, 6.5), (0, 0.9, 0), (0, 1, 0), math.radians(50.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def env_only(texels, width=16, height=16, spp=2):
    """No geometry at all, only an environment light over `texels` (H, W, 3):
    every camera ray leaves the scene at once."""
    sb = SceneBuffers(positions=np.zeros((0, 3), np.float32), normals=np.zeros((0, 3), np.float32),
                      uvs=np.zeros((0, 2), np.float32), indices=np.zeros((0, 3), np.int32),
                      sphere_radius=np.zeros(0, np.float32), sphere_to_world=np.zeros((0, 16), np.float32),
                      sphere_to_local=np.zeros((0, 16), np.float32), materials=[lambert((0.5, 0.5, 0.5))],
                      prim_shape=np.zeros(0, np.int32), prim_material=np.zeros(0, np.int32),
                      prim_emission=np.zeros((0, 3), np.float32), light_prims=np.zeros(0, np.int32))
    sb.env_texels = np.asarray(texels, np.float32)
    sb.env_to_light, sb.env_to_world = rotate_x(math.pi / 2)
    cam = make_camera(width / height, (0, 1, 5), (0, 0, 0), (0, 1, 0), math.radians(60.0), 0.0, 1.0)
    return sb, cam, make_filter(0.5, 0.6), make_params(width, height, spp, 3, 5)


def disney15_row(width=96, height=48, spp=8, max_depth=6, min_depth=3, env=True):
    """Five spheres of the 2015 Disney BSDF (create_disney) on a ground quad
    under a small area light and (by default) the sky map: a rough
    dielectric, a metal, a clearcoated sheen layer, a rough transmitter and a
    smooth anisotropic transmitter."""
    b = _Builder()
    ground = b.material(lambert((0.45, 0.42, 0.4)))
    b.quad((-6, 0, -6), (6, 0, -6), (6, 0, 6), (-6, 0, 6), (0, 1, 0), ground)
    b.quad((-0.5, 3, -0.5), (0.5, 3, -0.5), (0.5, 3, 0.5), (-0.5, 3, 0.5), (0, -1, 0), ground,
           emission=(8.0, 8.0, 8.0))
    params = [dict(base_color=(0.8, 0.3, 0.2), roughness=0.5, specular_scale=(1.0, 1.0, 1.0), ior=1.5),
              dict(base_color=(0.9, 0.7, 0.4), metallic=0.9, roughness=0.3, anisotropic=0.5, ior=1.5),
              dict(base_color=(0.2, 0.4, 0.8), roughness=0.6, sheen=0.8, sheen_tint=0.5, clearcoat=0.7,
                   clearcoat_gloss=0.6, specular_tint=0.3, specular_scale=(0.5, 0.5, 0.5), ior=1.4),
              dict(base_color=(0.9, 0.9, 0.9), roughness=0.2, transmission=0.8, transmission_roughness=0.3,
                   specular_scale=(1.0, 1.0, 1.0), ior=1.5),
              dict(base_color=(0.7, 0.9, 0.7), roughness=0.1, transmission=0.5, transmission_roughness=0.05,
                   anisotropic=0.6, metallic=0.1, ior=1.33)]
    for k, p in enumerate(params):
        m = b.material(Material(kind=TR_MAT_DISNEY15, **p))
        b.sphere((-3.0 + 1.5 * k, 0.6, 0.0), 0.6, m)
    scene = b.finish(max_leaf_prims=3)
    if env:
        scene.env_texels = sky_map(64, 32)
        scene.env_to_light, scene.env_to_world = rotate_x(math.pi / 2)
    cam = make_camera(width / height, (0, 1.8, 7.0), (0, 0.7, 0), (0, 1, 0), math.radians(50.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def mapped_materials(width=96, height=48, spp=8, max_depth=6, min_depth=3, env=True):
    """Image maps on every material kind that takes them: a ground of
    Disney12 with a base-colour checker and a roughness ramp; spheres of
    metal (colour and roughness maps), Disney 2015 (base colour, roughness,
    transmission and sheen maps), glass (kr map and an ior map) and Disney12
    (base colour, metallic, clearcoat maps) beside a constant Phong sphere,
    under a small area light and (by default) the sky map. Maps are 8-bit
    checkers and float ramps (create_image_texture2d, create_hdr_texture2d)."""
    b = _Builder()
    ramp = np.linspace(0.05, 0.95, 8 * 4 * 3, dtype=np.float32).reshape(4, 8, 3)
    ior_map = np.linspace(1.2, 1.8, 6 * 6 * 3, dtype=np.float32).reshape(6, 6, 3)
    textures = [checker(16, 4),                                                        # 1: 8-bit colours
                ramp,                                                                  # 2: float ramp
                checker(8, 2, (0.9, 0.9, 0.9), (0.1, 0.1, 0.1), eight_bit=False),      # 3: float 0.9/0.1
                ior_map,                                                               # 4: float 1.2..1.8
                checker(12, 3, (0.95, 0.64, 0.54), (0.3, 0.7, 0.9))]                   # 5: 8-bit colours
    ground = b.material(Material(kind=TR_MAT_DISNEY12, base_color=(0.5, 0.5, 0.5), roughness=0.5, specular=0.5,
                                 tex_param=(1, 0, 0, 0, 0, 2) + (0,) * 7))
    b.quad((-6, 0, -6), (6, 0, -6), (6, 0, 6), (-6, 0, 6), (0, 1, 0), ground)
    light = b.material(lambert((0.5, 0.5, 0.5)))
    b.quad((-0.5, 3, -0.5), (0.5, 3, -0.5), (0.5, 3, 0.5), (-0.5, 3, 0.5), (0, -1, 0), light,
           emission=(8.0, 8.0, 8.0))
    mats = [Material(kind=TR_MAT_METAL, color=(0.95, 0.64, 0.54), eta=(0.2, 0.92, 1.1), k=(3.9, 2.45, 2.14),
                     roughness=0.3, anisotropic=0.3, tex_param=(5, 0, 0, 2, 0) + (0,) * 8),
            Material(kind=TR_MAT_DISNEY15, base_color=(0.8, 0.3, 0.2), roughness=0.5, specular_scale=(1.0, 1.0, 1.0),
                     ior=1.5, tex_param=(1, 0, 2, 3, 0, 0, 0, 0, 0, 2, 0, 0, 0)),
            Material(kind=TR_MAT_GLASS, kr=(1.0, 1.0, 1.0), kt=(1.0, 1.0, 1.0), ior=1.5,
                     tex_param=(5, 0, 4) + (0,) * 10),
            Material(kind=TR_MAT_DISNEY12, base_color=(0.2, 0.4, 0.8), roughness=0.4, specular=0.5, clearcoat=0.3,
                     clearcoat_gloss=0.5, tex_param=(5, 0, 3, 0, 0, 0, 0, 0, 0, 2, 0) + (0, 0)),
            lambert((0.6, 0.6, 0.2))]
    for k, m in enumerate(mats):
        b.sphere((-3.0 + 1.5 * k, 0.6, 0.0), 0.6, b.material(m))
    scene = b.finish(max_leaf_prims=3)
    scene.textures = textures
    if env:
        scene.env_texels = sky_map(64, 32)
        scene.env_to_light, scene.env_to_world = rotate_x(math.pi / 2)
    cam = make_camera(width / height, (0, 1.8, 7.0), (0, 0.7, 0), (0, 1, 0), math.radians(50.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def traversal(n_tris=1 << 20, seed=0, max_leaf_prims=4):
    """n_tris triangles: centres uniform in [0,1]^3, each vertex the centre plus
    an edge vector uniform in [-0.01,0.01]^3. numpy PCG64(seed)."""
    rng = np.random.default_rng(seed)
    c = rng.random((n_tris, 3), dtype=np.float64)
    e = rng.uniform(-0.01, 0.01, size=(n_tris, 3, 3))
    v = (c[:, None, :] + e).astype(np.float32).reshape(-1, 3) + np.float32(0)
    idx = np.arange(3 * n_tris, dtype=np.int32).reshape(-1, 3)
    nrm = np.tile(np.array([0, 0, 1], dtype=np.float32), (3 * n_tris, 1))
    uv = np.zeros((3 * n_tris, 2), dtype=np.float32)
    white = lambert((0.7, 0.7, 0.7))
    return SceneBuffers(positions=v, normals=nrm, uvs=uv, indices=idx,
                        sphere_radius=np.zeros(0, np.float32), sphere_to_world=np.zeros((0, 16), np.float32),
                        sphere_to_local=np.zeros((0, 16), np.float32), materials=[white],
                        prim_shape=np.arange(n_tris, dtype=np.int32), prim_material=np.zeros(n_tris, np.int32),
                        prim_emission=np.zeros((n_tris, 3), np.float32), light_prims=np.zeros(0, np.int32),
                        max_leaf_prims=max_leaf_prims)


def cube_surface_points(rng, n):
    face = rng.integers(0, 6, n)
    uv = rng.random((n, 2))
    p = np.empty((n, 3))
    ax = face // 2
    for a in range(3):
        m = ax == a
        others = [k for k in range(3) if k != a]
        p[m, a] = (face[m] % 2).astype(np.float64)
        p[m, others[0]] = uv[m, 0]
        p[m, others[1]] = uv[m, 1]
    return p.astype(np.float32)


def traversal_rays(n_rays=1 << 22, seed=0, shadow=False):
    """Closest-hit rays (t_max = FLT_MAX) or shadow rays (t_max ~ U(0,1)),
    origins uniform on the unit-cube surface, directions uniform on the sphere,
    t_min = 0; through the reference Ray constructor. numpy PCG64(seed + 1/2)."""
    rng = np.random.default_rng(seed + (2 if shadow else 1))
    o = cube_surface_points(rng, n_rays)
    d = rng.normal(size=(n_rays, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tmax = rng.random(n_rays).astype(np.float32) if shadow else F32_MAX
    return make_rays(o, d, 0.0, tmax)


def adversarial_rays(sc, seed=0):
    """Closest-hit rays at a scene's triangles' edge cases: aimed from random
    origins exactly at each triangle's vertices, the midpoint of its first
    edge and its centroid; and axis-parallel rays whose origin's x lies on a
    vertex's coordinate (infinite inverse directions, slab planes through the
    origin). Through the reference Ray constructor; t_min 0, t_max FLT_MAX."""
    rng = np.random.default_rng(100 + seed)
    tri = sc.positions[sc.indices]  # (T, 3, 3)
    targets = np.concatenate([tri[:, 0], tri[:, 1], tri[:, 2],
                              ((tri[:, 0] + tri[:, 1]) * np.float32(0.5)).astype(np.float32),
                              ((tri[:, 0] + tri[:, 1] + tri[:, 2]) / np.float32(3)).astype(np.float32)])
    origins = rng.uniform(-3, 3, (len(targets), 3)).astype(np.float32)
    aimed = make_rays(origins, (targets - origins).astype(np.float32), 0.0, F32_MAX)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [1, 1, 0], [0, -1, 1], [1, 0, -1]], np.float32)
    o_ax = np.repeat(tri[:, 0], len(axes), axis=0) - np.float32(2) * np.tile(axes, (len(tri), 1))
    o_ax[:, 0] = np.repeat(tri[:, 1, 0], len(axes))
    parallel = make_rays(o_ax, np.tile(axes, (len(tri), 1)), 0.0, F32_MAX)
    return np.concatenate([aimed, parallel])


def shadow_rays_at_hits(rays, prim, t, step):
    """The rays that hit something, as shadow rays with t_max at the hit
    distance (step 0) or one ulp below (-1) or above (+1) it."""
    hit = prim >= 0
    s = rays[hit].copy()
    s["t_max"] = np.nextafter(t[hit], np.float32(np.inf if step > 0 else -np.inf)) if step else t[hit]
    return s


def random_scene(seed=0, n_tris=64, n_spheres=8, n_lights=2, disney_frac=0.5, max_leaf_prims=3):
    """Small closed-ish scene for parity tests: a floor, random triangles and
    spheres in [-1,1]^3, emissive triangles overhead."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    mats = []
    for k in range(6):
        if rng.random() < disney_frac:
            p = rng.random(12)
            mats.append(b.material(Material(kind=TR_MAT_DISNEY12, base_color=tuple(p[0:3]), metallic=p[3],
                                            roughness=p[4], specular=p[5], specular_tint=p[6], sheen=p[7],
                                            clearcoat=p[8], clearcoat_gloss=p[9], anisotropic=p[10],
                                            subsurface=p[11], sheen_tint=0.5)))
        else:
            kd = tuple(0.2 + 0.7 * rng.random(3))
            ks = tuple(0.3 * rng.random(3)) if rng.random() < 0.5 else (0.0, 0.0, 0.0)
            mats.append(b.material(Material(kind=TR_MAT_PHONG, kd=kd, ks=ks, ns=float(1 + 40 * rng.random()))))
    b.quad((-3, -1, -3), (3, -1, -3), (3, -1, 3), (-3, -1, 3), (0, 1, 0), mats[0])
    for _ in range(n_lights):
        c = rng.uniform(-1, 1, 3) * np.array([1.0, 0.0, 1.0]) + np.array([0.0, 2.0, 0.0])
        s = 0.2 + 0.3 * rng.random()
        b.triangle(c + [-s, 0, -s], c + [s, 0, -s], c + [0, 0, s], (0, -1, 0), mats[0],
                   emission=tuple(float(v) for v in 2 + 10 * rng.random(3)))
        # winding of (a,b,c) above gives cross(AB,AC) along -y
    for _ in range(n_tris):
        c = rng.uniform(-1, 1, 3)
        e = rng.uniform(-0.4, 0.4, (2, 3))
        a, bb, cc = c, c + e[0], c + e[1]
        nrm = np.cross(bb - a, cc - a)
        if np.linalg.norm(nrm) < 1e-6:
            continue
        b.triangle(a, bb, cc, nrm, mats[int(rng.integers(0, 6))], uvs=tuple(map(tuple, rng.random((3, 2)))))
    for _ in range(n_spheres):
        b.sphere(rng.uniform(-1, 1, 3), float(0.1 + 0.3 * rng.random()), mats[int(rng.integers(0, 6))])
    scene = b.finish(max_leaf_prims=max_leaf_prims)
    return scene


def mixed_scene(seed=0, n_tris=80, n_spheres=10, env=True):
    """random_scene's geometry with materials of every kind drawn at random:
    Phong (some with 8-bit or float image maps), Disney12, Disney 2015,
    glass and metal; with the sky map as an environment light when `env`."""
    sc = random_scene(seed, n_tris=n_tris, n_spheres=n_spheres)
    rng = np.random.default_rng(1000 + seed)
    sc.textures = [checker(8, 2), checker(6, 3, (0.9, 0.4, 0.1), (0.1, 0.1, 0.9), eight_bit=False),
                   np.linspace(2.0, 40.0, 4 * 4 * 3, dtype=np.float32).reshape(4, 4, 3)]
    mats = []
    for k in range(len(sc.materials)):
        if k == 0:  # the floor and the lights keep theirs
            mats.append(sc.materials[0])
            continue
        kind = int(rng.integers(0, 6))
        p = rng.random(14)
        if kind == 0:
            mats.append(Material(kind=TR_MAT_PHONG, kd=tuple(0.2 + 0.7 * p[0:3]), ks=tuple(0.3 * p[3:6]),
                                 ns=float(1 + 40 * p[6]), tex_kd=int(rng.integers(0, 3)),
                                 tex_ns=3 if p[7] < 0.5 else 0))
        elif kind == 1:
            mats.append(Material(kind=TR_MAT_DISNEY12, base_color=tuple(p[0:3]), metallic=p[3], roughness=p[4],
                                 specular=p[5], specular_tint=p[6], sheen=p[7], clearcoat=p[8],
                                 clearcoat_gloss=p[9], anisotropic=p[10], subsurface=p[11], sheen_tint=0.5))
        elif kind == 2:
            mats.append(Material(kind=TR_MAT_DISNEY15, base_color=tuple(p[0:3]), metallic=p[3], roughness=p[4],
                                 transmission=p[5], transmission_roughness=p[6], ior=1.2 + p[7],
                                 specular_scale=tuple(p[8:11]), specular_tint=p[11], anisotropic=p[12],
                                 sheen=p[13], clearcoat=p[0] * p[1], clearcoat_gloss=p[2]))
        elif kind == 3:
            mats.append(Material(kind=TR_MAT_GLASS, kr=tuple(0.5 + 0.5 * p[0:3]), kt=tuple(0.5 + 0.5 * p[3:6]),
                                 ior=1.2 + 0.6 * p[6]))
        elif kind == 4:
            mats.append(Material(kind=TR_MAT_METAL, color=tuple(0.3 + 0.7 * p[0:3]), eta=tuple(0.1 + p[3:6]),
                                 k=tuple(1 + 3 * p[6:9]), roughness=0.05 + 0.6 * p[9], anisotropic=p[10]))
        else:
            mats.append(Material(kind=TR_MAT_PHONG, kd=tuple(0.2 + 0.7 * p[0:3]), ns=1.0))
    sc.materials = mats
    if env:
        sc.env_texels = sky_map(32, 16)
        sc.env_to_light, sc.env_to_world = rotate_x(math.pi / 2)
    return sc


def random_camera(width, height, seed=0):
    rng = np.random.default_rng(seed + 1000)
    pos = (float(rng.uniform(-1, 1)), float(rng.uniform(0.0, 1.5)), float(4 + rng.uniform(0, 1)))
    return make_camera(width / height, pos, (0, 0, 0), (0, 1, 0), math.radians(45.0), 0.0, 1.0)


_MAT_FIELDS = ("ka", "kd", "ks", "ns", "base_color", "subsurface", "metallic", "specular", "specular_tint",
               "roughness", "anisotropic", "sheen", "sheen_tint", "clearcoat", "clearcoat_gloss",
               # added later: fixtures packed before them have shorter rows and keep the defaults
               "kr", "kt", "ior", "color", "eta", "k", "transmission", "transmission_roughness", "specular_scale",
               "tex_ka", "tex_kd", "tex_ks", "tex_ns", "tex_param")


def pack_scene(s: SceneBuffers, prefix: str = "") -> dict:
    """Flat arrays of a scene (for fixtures)."""
    mats = []
    for m in s.materials:
        row = [float(m.kind)]
        for f in _MAT_FIELDS:
            v = getattr(m, f)
            row.extend(list(v) if isinstance(v, (tuple, list)) else [float(v)])
        mats.append(row)
    out = {"positions": s.positions, "normals": s.normals, "uvs": s.uvs, "indices": s.indices,
           "sphere_radius": s.sphere_radius, "sphere_to_world": s.sphere_to_world,
           "sphere_to_local": s.sphere_to_local, "materials": np.asarray(mats, np.float32),
           "prim_shape": s.prim_shape, "prim_material": s.prim_material, "prim_emission": s.prim_emission,
           "light_prims": s.light_prims, "max_leaf_prims": np.int32(s.max_leaf_prims)}
    if s.env_texels is not None or s.env_texels8 is not None:
        out["env_texels"] = s.env_texels if s.env_texels is not None else s.env_texels8
        out["env_to_light"], out["env_to_world"] = s.env_to_light, s.env_to_world
    for k, t in enumerate(s.textures):
        out[f"texture{k}"] = t
    return {prefix + k: np.asarray(v) for k, v in out.items()}


def unpack_scene(d, prefix: str = "") -> SceneBuffers:
    mats = []
    for row in np.asarray(d[prefix + "materials"], np.float64):
        m = Material(kind=int(row[0]))
        i = 1
        for f in _MAT_FIELDS:
            if i >= len(row):
                break
            cur = getattr(m, f)
            if isinstance(cur, tuple):
                n = len(cur)
                cast = int if f == "tex_param" else float
                setattr(m, f, tuple(cast(x) for x in row[i:i + n]))
                i += n
            else:
                setattr(m, f, int(row[i]) if isinstance(cur, int) and f.startswith("tex_") else float(row[i]))
                i += 1
        mats.append(m)
    g = lambda k: np.asarray(d[prefix + k])
    sb = SceneBuffers(positions=g("positions"), normals=g("normals"), uvs=g("uvs"), indices=g("indices"),
                      sphere_radius=g("sphere_radius"), sphere_to_world=g("sphere_to_world"),
                      sphere_to_local=g("sphere_to_local"), materials=mats, prim_shape=g("prim_shape"),
                      prim_material=g("prim_material"), prim_emission=g("prim_emission"),
                      light_prims=g("light_prims"), max_leaf_prims=int(g("max_leaf_prims")))
    if prefix + "env_texels" in d:
        env = g("env_texels")
        if env.dtype == np.uint8:
            sb.env_texels8 = env
        else:
            sb.env_texels = env
        sb.env_to_light, sb.env_to_world = g("env_to_light"), g("env_to_world")
    k = 0
    while prefix + f"texture{k}" in d:
        sb.textures.append(g(f"texture{k}"))
        k += 1
    return sb


def pack_view(cam, filt, par, prefix: str = "") -> dict:
    return {prefix + "camera": np.array([cam.film_aspect, *cam.pos, *cam.target, *cam.up, cam.fov,
                                         cam.lens_radius, cam.focal_dist], np.float32),
            prefix + "filter": np.array([filt.radius, filt.alpha], np.float32),
            prefix + "params": np.array([par.width, par.height, par.spp, par.min_depth, par.max_depth,
                                         par.direct_light_sample_num, par.seed_base], np.int64)}


def unpack_view(d, prefix: str = ""):
    c = np.asarray(d[prefix + "camera"], np.float32)
    cam = make_camera(float(c[0]), tuple(c[1:4]), tuple(c[4:7]), tuple(c[7:10]), float(c[10]), float(c[11]),
                      float(c[12]))
    f = np.asarray(d[prefix + "filter"], np.float32)
    p = np.asarray(d[prefix + "params"], np.int64)
    par = make_params(int(p[0]), int(p[1]), int(p[2]), int(p[3]), int(p[4]), seed_base=int(p[6]),
                      direct_light_sample_num=int(p[5]))
    return cam, make_filter(float(f[0]), float(f[1])), par


def _grid_box(center, size, rot_y, k):
    """Box tessellated into k x k quads per face: (12 k^2, 3, 3) triangles
    with outward winding, and their normals."""
    c = np.asarray(center, np.float64)
    h = np.asarray(size, np.float64) / 2
    cs, sn = math.cos(rot_y), math.sin(rot_y)
    R = np.array([[cs, 0, sn], [0, 1, 0], [-sn, 0, cs]])
    t = np.linspace(-1.0, 1.0, k + 1)
    tris, nrms = [], []
    for axis in range(3):
        u, v = (axis + 1) % 3, (axis + 2) % 3
        for sgn in (-1.0, 1.0):
            P = np.zeros((k + 1, k + 1, 3))
            P[..., axis] = sgn
            P[..., u] = t[:, None]
            P[..., v] = t[None, :]
            P = c + (P * h) @ R.T
            a, b, cc, d = P[:-1, :-1], P[1:, :-1], P[1:, 1:], P[:-1, 1:]
            if sgn > 0:
                q = np.concatenate([np.stack([a, b, cc], -2), np.stack([a, cc, d], -2)], 0)
            else:
                q = np.concatenate([np.stack([a, cc, b], -2), np.stack([a, d, cc], -2)], 0)
            q = q.reshape(-1, 3, 3)
            n = np.zeros(3)
            n[axis] = sgn
            tris.append(q)
            nrms.append(np.broadcast_to(R @ n, q.shape))
    return np.concatenate(tris), np.concatenate(nrms)


def _cylinder(center, radius, height, segs, rings):
    """Upright capped cylinder: side 2 * segs * rings triangles with radial
    normals, two caps of segs triangles."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0, 2 * math.pi, segs + 1)
    y = np.linspace(0, height, rings + 1)
    ring = np.stack([np.cos(th), np.zeros_like(th), np.sin(th)], -1)  # (segs+1, 3)
    P = c + radius * ring[None, :, :] + y[:, None, None] * np.array([0, 1, 0])
    N = np.broadcast_to(ring[None], P.shape)
    a, b, cc, d = P[:-1, :-1], P[:-1, 1:], P[1:, 1:], P[1:, :-1]
    na, nb, nc, nd = N[:-1, :-1], N[:-1, 1:], N[1:, 1:], N[1:, :-1]
    # outward winding: (a, d, c) and (a, c, b) have cross pointing along the radial normal
    side = np.concatenate([np.stack([a, d, cc], -2), np.stack([a, cc, b], -2)], 0).reshape(-1, 3, 3)
    sn = np.concatenate([np.stack([na, nd, nc], -2), np.stack([na, nc, nb], -2)], 0).reshape(-1, 3, 3)
    top_c = c + np.array([0, height, 0])
    r0, r1 = P[-1, :-1], P[-1, 1:]
    top = np.stack([np.broadcast_to(top_c, r0.shape), r1, r0], -2)
    b0, b1 = P[0, :-1], P[0, 1:]
    bot = np.stack([np.broadcast_to(c, b0.shape), b0, b1], -2)
    tris = np.concatenate([side, top, bot])
    nrms = np.concatenate([sn, np.broadcast_to([0.0, 1.0, 0.0], top.shape),
                           np.broadcast_to([0.0, -1.0, 0.0], bot.shape)])
    return tris, nrms


def occluded_room(width=1024, height=768, spp=16, max_depth=10, min_depth=3, n_tris=500_000, seed=0):
    """The occluded-light room: a closed 8 x 4 x 6 m room (x in [-4, 4],
    y in [0, 4], z in [-3, 3]) of Lambertian walls (albedo 0.7). The only
    light is a 3 m emissive cube (12 triangles, Le 50) outside the +x wall,
    seen from inside through a 0.1 m x 3 m slit in that wall. n_tris
    triangles of furniture (tessellated boxes and cylinders on the floor),
    each piece a Disney12 material with roughness uniform in [0.05, 1].
    Camera near the -x wall looking toward the slit, 60 degree fov."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    wall = b.material(lambert((0.7, 0.7, 0.7)))
    X, Y, Z = 4.0, 4.0, 3.0
    b.quad((-X, 0, -Z), (X, 0, -Z), (X, 0, Z), (-X, 0, Z), (0, 1, 0), wall)         # floor
    b.quad((-X, Y, -Z), (X, Y, -Z), (X, Y, Z), (-X, Y, Z), (0, -1, 0), wall)         # ceiling
    b.quad((-X, 0, -Z), (X, 0, -Z), (X, Y, -Z), (-X, Y, -Z), (0, 0, 1), wall)        # back (z = -3)
    b.quad((-X, 0, Z), (X, 0, Z), (X, Y, Z), (-X, Y, Z), (0, 0, -1), wall)           # front (z = +3)
    b.quad((-X, 0, -Z), (-X, Y, -Z), (-X, Y, Z), (-X, 0, Z), (1, 0, 0), wall)        # -x wall
    # +x wall with the slit z in [-0.05, 0.05], y in [0.5, 3.5]
    g, y0, y1 = 0.05, 0.5, 3.5
    b.quad((X, 0, -Z), (X, Y, -Z), (X, Y, -g), (X, 0, -g), (-1, 0, 0), wall)
    b.quad((X, 0, g), (X, Y, g), (X, Y, Z), (X, 0, Z), (-1, 0, 0), wall)
    b.quad((X, 0, -g), (X, y0, -g), (X, y0, g), (X, 0, g), (-1, 0, 0), wall)
    b.quad((X, y1, -g), (X, Y, -g), (X, Y, g), (X, y1, g), (-1, 0, 0), wall)
    # furniture: boxes and cylinders until n_tris
    pieces, total = [], 0
    while total < n_tris:
        kind = rng.random() < 0.5
        cx, cz = rng.uniform(-3.3, 2.8), rng.uniform(-2.4, 2.4)
        if kind:
            k = int(rng.integers(8, 33))
            size = (rng.uniform(0.3, 1.2), rng.uniform(0.3, 1.6), rng.uniform(0.3, 1.2))
            tris, nrm = _grid_box((cx, size[1] / 2, cz), size, rng.uniform(0, math.pi), k)
        else:
            segs, rings = int(rng.integers(32, 129)), int(rng.integers(8, 64))
            tris, nrm = _cylinder((cx, 0.0, cz), rng.uniform(0.1, 0.5), rng.uniform(0.3, 2.0), segs, rings)
        tris, nrm = tris[: n_tris - total], nrm[: n_tris - total]
        p = rng.random(4)
        mat = b.material(Material(kind=TR_MAT_DISNEY12, base_color=tuple(float(v) for v in 0.2 + 0.6 * rng.random(3)),
                                  metallic=float(0.3 * p[0]), roughness=float(0.05 + 0.95 * p[1]),
                                  specular=0.5, specular_tint=float(p[2]), sheen=0.0, sheen_tint=0.5,
                                  clearcoat=float(0.5 * p[3]), clearcoat_gloss=0.5, anisotropic=0.0,
                                  subsurface=0.0))
        b.mesh(tris, nrm, mat)
        total += len(tris)
    # the light: a 3 m cube outside the slit, every face emitting outward
    emit = (50.0, 50.0, 50.0)
    lo, hi = np.array([X + 0.5, 0.5, -1.5]), np.array([X + 3.5, 3.5, 1.5])
    for axis in range(3):
        u, v = (axis + 1) % 3, (axis + 2) % 3
        for sgn in (-1, 1):
            n = [0, 0, 0]
            n[axis] = sgn
            corners = []
            for su, sv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                q = [0.0, 0.0, 0.0]
                q[axis] = hi[axis] if sgn > 0 else lo[axis]
                q[u] = hi[u] if su else lo[u]
                q[v] = hi[v] if sv else lo[v]
                corners.append(q)
            b.quad(*corners, n, wall, emission=emit)
    scene = b.finish(max_leaf_prims=3)
    cam = make_camera(width / height, (-3.6, 1.8, 2.4), (2.0, 1.6, -0.6), (0, 1, 0), math.radians(60.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(width, height, spp, min_depth, max_depth)


def _uv_sphere(center, radius, segs, rings):
    """UV sphere: 2 * segs * rings triangles with radial normals."""
    th = np.linspace(0.0, math.pi, rings + 1)
    ph = np.linspace(0.0, 2 * math.pi, segs + 1)
    N = np.stack([np.sin(th)[:, None] * np.cos(ph)[None], np.cos(th)[:, None] * np.ones_like(ph)[None],
                  np.sin(th)[:, None] * np.sin(ph)[None]], -1)
    P = np.asarray(center) + radius * N
    a, b, c, d = P[:-1, :-1], P[:-1, 1:], P[1:, 1:], P[1:, :-1]
    na, nb, nc, nd = N[:-1, :-1], N[:-1, 1:], N[1:, 1:], N[1:, :-1]
    # (a, b, c): b steps along phi, c along theta and phi; cross(phi, theta) points outward
    tris = np.concatenate([np.stack([a, b, c], -2), np.stack([a, c, d], -2)], 0).reshape(-1, 3, 3)
    nrms = np.concatenate([np.stack([na, nb, nc], -2), np.stack([na, nc, nd], -2)], 0).reshape(-1, 3, 3)
    keep = np.linalg.norm(np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]), axis=1) > 0
    return tris[keep], nrms[keep]


def _torus(center, R, r, nu, nv):
    """Torus around the y axis: 2 * nu * nv triangles, normals from the tube centre."""
    u = np.linspace(0.0, 2 * math.pi, nu + 1)
    v = np.linspace(0.0, 2 * math.pi, nv + 1)
    cu, su, cv, sv = np.cos(u)[:, None], np.sin(u)[:, None], np.cos(v)[None], np.sin(v)[None]
    N = np.stack([cv * cu, sv * np.ones_like(cu), cv * su], -1)
    C = np.stack([R * cu * np.ones_like(cv), np.zeros_like(cu * cv), R * su * np.ones_like(cv)], -1)
    P = np.asarray(center) + C + r * N
    a, b, c, d = P[:-1, :-1], P[:-1, 1:], P[1:, 1:], P[1:, :-1]
    na, nb, nc, nd = N[:-1, :-1], N[:-1, 1:], N[1:, 1:], N[1:, :-1]
    tris = np.concatenate([np.stack([a, b, c], -2), np.stack([a, c, d], -2)], 0).reshape(-1, 3, 3)
    nrms = np.concatenate([np.stack([na, nb, nc], -2), np.stack([na, nc, nd], -2)], 0).reshape(-1, 3, 3)
    return tris, nrms


def batch_scene(seed: int, tri_range=(10_000, 2_000_000)):
    """One scene of the batched-rendering workload: a ground quad and one to
    five tessellated spheres, boxes or tori sharing a triangle count drawn
    log-uniformly from tri_range, each Lambertian or Disney12 at random,
    one to four 1x1 area-light quads; film 128^2 .. 1024^2, 4, 16 or 64 spp,
    max depth 6. Returns (scene, camera, filter, params)."""
    rng = np.random.default_rng(1000 + seed)
    total = int(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1]))))
    res = int(rng.choice([128, 256, 512, 1024]))
    spp = int(rng.choice([4, 16, 64]))
    b = _Builder()
    ground = b.material(lambert((0.6, 0.6, 0.6)))
    b.quad((-6, 0, -6), (6, 0, -6), (6, 0, 6), (-6, 0, 6), (0, 1, 0), ground)
    nobj = int(rng.integers(1, 6))
    share = np.maximum(rng.dirichlet(np.ones(nobj)) * total, 100).astype(int)
    for k in range(nobj):
        if rng.random() < 0.5:
            mat = b.material(lambert(tuple(float(v) for v in 0.2 + 0.7 * rng.random(3))))
        else:
            q = rng.random(6)
            mat = b.material(Material(kind=TR_MAT_DISNEY12, base_color=tuple(float(v) for v in 0.2 + 0.7 * rng.random(3)),
                                      metallic=float(q[0]), roughness=float(0.05 + 0.95 * q[1]), specular=0.5,
                                      specular_tint=float(q[2]), sheen=float(q[3]), sheen_tint=0.5,
                                      clearcoat=float(q[4]), clearcoat_gloss=float(q[5]), anisotropic=0.0,
                                      subsurface=0.0))
        c = (rng.uniform(-3.5, 3.5), 0.0, rng.uniform(-3.5, 3.5))
        kind = int(rng.integers(0, 3))
        t = int(share[k])
        if kind == 0:
            n = max(4, int(math.sqrt(t / 4)))
            rad = rng.uniform(0.4, 1.2)
            tris, nrm = _uv_sphere((c[0], rad, c[2]), rad, 2 * n, n)
        elif kind == 1:
            kk = max(1, int(math.sqrt(t / 12)))
            size = rng.uniform(0.5, 2.0, 3)
            tris, nrm = _grid_box((c[0], size[1] / 2, c[2]), size, rng.uniform(0, math.pi), kk)
        else:
            n = max(4, int(math.sqrt(t / 2)))
            Rr = rng.uniform(0.6, 1.2)
            tris, nrm = _torus((c[0], 0.45 * Rr, c[2]), Rr, 0.4 * Rr, n, n)
        b.mesh(tris, nrm, mat, settle=False)
    for _ in range(int(rng.integers(1, 5))):
        x, z = rng.uniform(-4, 4), rng.uniform(-4, 4)
        y = rng.uniform(4.0, 6.0)
        b.quad((x - 0.5, y, z - 0.5), (x + 0.5, y, z - 0.5), (x + 0.5, y, z + 0.5), (x - 0.5, y, z + 0.5), (0, -1, 0),
               ground, emission=tuple(float(v) for v in 10 + 20 * rng.random(3)))
    scene = b.finish(max_leaf_prims=3)
    cam = make_camera(1.0, (0.0, 5.0, 11.0), (0.0, 0.5, 0.0), (0, 1, 0), math.radians(50.0), 0.0, 1.0)
    return scene, cam, make_filter(0.5, 0.6), make_params(res, res, spp, 3, 6, seed_base=seed * 7919)


def batch(n: int = 64, seed: int = 0, tri_range=(10_000, 2_000_000)):
    """The batched-rendering workload: n scenes of batch_scene."""
    return [batch_scene(seed * 1000 + k, tri_range) for k in range(n)]
