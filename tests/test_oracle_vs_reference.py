"""The oracle against the reference's own sources compiled here (oracle/_ref).
Skipped where the reference checkout is absent (the fixtures in
test_oracle_golden.py cover that case)."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_units_random():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(20000, 3)).astype(np.float32) * rng.choice([1e-8, 1, 1e8], size=(20000, 1)).astype(np.float32)
    b = rng.normal(size=(20000, 3)).astype(np.float32)
    for name, args in (("cross", (a, b)), ("normalize", (a,))):
        x = oracle.unit("port", name, *args, out_shape=(20000, 3), n=20000)
        y = oracle.unit("reference", name, *args, out_shape=(20000, 3), n=20000)
        assert np.array_equal(bits(x), bits(y)), name
    for s in (0, 99, -7, 2**31 - 1):
        assert np.array_equal(oracle.pcg_uniform("port", s, 5000), oracle.pcg_uniform("reference", s, 5000))


@pytest.mark.parametrize("seed", range(4))
def test_random_scenes(seed):
    sc = scenes.random_scene(seed, n_tris=70, n_spheres=9)
    cam = scenes.random_camera(40, 32, seed)
    par = scenes.make_params(40, 32, 3, seed % 3, 6, seed_base=seed)
    filt = scenes.make_filter(0.5, 0.6)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    n0, o0 = port.bvh()
    n1, o1 = ref.bvh()
    assert np.array_equal(n0, n1) and np.array_equal(o0, o1)
    rng = np.random.default_rng(seed)
    rays = scenes.make_rays(rng.uniform(-2, 2, (4000, 3)).astype(np.float32),
                            rng.normal(size=(4000, 3)).astype(np.float32), 0.0, scenes.F32_MAX)
    p0, t0 = port.trace_closest(rays)
    p1, t1 = ref.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(bits(t0), bits(t1))
    srays = rays.copy()
    srays["t_max"] = rng.uniform(0, 3, 4000).astype(np.float32)
    assert np.array_equal(port.trace_any(srays), ref.trace_any(srays))
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


def test_traversal_workload_subset():
    sc = scenes.traversal(1 << 14, seed=1)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    rays = scenes.traversal_rays(1 << 14, seed=1)
    p0, t0 = port.trace_closest(rays)
    p1, t1 = ref.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(bits(t0), bits(t1))


def test_wide_filter_and_disney():
    sc, cam, filt, par = scenes.disney_grid(24, 24, 2, min_depth=2)
    filt = scenes.make_filter(1.5, 0.6)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("min_depth", [8, 2])
def test_glass_cornell(min_depth):
    """Glass (a delta BSDF) and the specular branch of eval_pixel_li."""
    sc, cam, filt, par = scenes.cornell(32, 24, 4, max_depth=8, min_depth=min_depth, glass=True)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("min_depth,glass", [(8, False), (2, False), (2, True)])
def test_metal_cornell(min_depth, glass):
    """Metal (an anisotropic GGX conductor with the painted Fresnel that
    create_metal builds), alone and beside glass."""
    sc, cam, filt, par = scenes.cornell(32, 24, 4, max_depth=8, min_depth=min_depth, glass=glass, metal=True)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("area_light,env_size,min_depth", [(True, (64, 32), 3), (False, (400, 200), 2),
                                                             (True, (37, 19), 6)])
def test_environment_light(area_light, env_size, min_depth):
    """The IBL environment light: emission of escaping rays, its light
    sample and the MIS ray's share, with its luminance distribution built
    over the full map and over a downsampled 360 x 180 grid."""
    sc, cam, filt, par = scenes.outdoor(32, 24, 4, min_depth=min_depth, env_size=env_size, area_light=area_light)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("maker", ["cornell", "outdoor"])
def test_phong_image_textures(maker):
    """Phong materials with image maps (8-bit and float kd, float ks and ns)
    looked up at the hit's uv: barycentric on triangles, (phi, theta) on a
    sphere."""
    if maker == "cornell":
        sc, cam, filt, par = scenes.cornell(32, 32, 4, textured=True)
    else:
        sc, cam, filt, par = scenes.outdoor(32, 24, 4, textured=True, glass=False)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("case", ["sky", "black", "1x1", "black_with_geometry"])
def test_environment_light_edge_cases(case):
    """No geometry (every ray leaves at once), an all-black map (a uniform
    distribution whose samples are all empty) and a 1 x 1 map."""
    if case == "black_with_geometry":
        sc, cam, filt, par = scenes.outdoor(24, 16, 2)
        sc.env_texels = np.zeros((8, 16, 3), np.float32)
    else:
        tex = {"sky": scenes.sky_map(16, 8), "black": np.zeros((8, 16, 3), np.float32),
               "1x1": np.full((1, 1, 3), 2.0, np.float32)}[case]
        sc, cam, filt, par = scenes.env_only(tex)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("min_depth", [3, 1])
def test_environment_light_8bit(min_depth):
    """An environment light over an 8-bit map (ImageTexture2D): its byte
    arithmetic (each weighted texel truncated to a byte) in the lookups and in
    the luminance distribution."""
    sc, cam, filt, par = scenes.outdoor(32, 24, 4, min_depth=min_depth, env_8bit=True, env_size=(53, 27))
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("env,min_depth", [(True, 3), (False, 8), (True, 1)])
def test_disney15(env, min_depth):
    """The 2015 Disney BSDF (create_disney): rough transmission and inner
    reflection, the specular, sheen and clearcoat lobes and its lobe choice."""
    sc, cam, filt, par = scenes.disney15_row(48, 24, 4, min_depth=min_depth, env=env)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("env", [True, False])
def test_mixed_random_scenes(seed, env):
    """Random triangles and spheres with materials of every kind (Phong with
    and without image maps, Disney12, Disney 2015, glass, metal), Russian
    roulette from depth 2, with and without the environment light."""
    sc = scenes.mixed_scene(seed, env=env)
    cam = scenes.random_camera(32, 24, seed)
    par = scenes.make_params(32, 24, 4, 2, 7, seed_base=seed * 31)
    filt = scenes.make_filter(0.5, 0.6)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    assert np.array_equal(bits(port.render(par)), bits(ref.render(par)))


def test_make_ray():
    for o, d in (((0, 0, 0), (1, 2, 3)), ((1, -1, 0.5), (1e-9, 1, 0)), ((0, 0, 0), (-0.0, 0.0, -3))):
        a = oracle.make_ray("port", o, d, 0.0, 1.0)
        b = oracle.make_ray("reference", o, d, 0.0, 1.0)
        assert bytes(a) == bytes(b)


def test_thin_lens_camera():
    """ThinLensCamera with a lens (src/camera/thin_lens_camera.cpp:40-59):
    the lens sample, the focal plane at focal_dist and look_at's frame."""
    sc, _, filt, par = scenes.cornell(40, 32, 4)
    cam = scenes.make_camera(40 / 32, (0.3, 0.2, 3.5), (0, -0.2, 0), (0, 1, 0), np.radians(40.0), 0.12, 3.1)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    a, b = port.render(par), ref.render(par)
    assert np.array_equal(bits(a), bits(b))
    # the lens matters: the same scene through a pinhole gives another film
    pin = scenes.make_camera(40 / 32, (0.3, 0.2, 3.5), (0, -0.2, 0), (0, 1, 0), np.radians(40.0), 0.0, 3.1)
    port.set_camera(pin, filt)
    assert not np.array_equal(bits(port.render(par)), bits(a))


def test_traversal_workload_full_size():
    """The traversal workload at its configured size: the port's BVH over
    1,048,576 triangles is the reference build's node for node, and a
    quarter of the 4M closest-hit and shadow rays give the same results."""
    sc = scenes.traversal(1 << 20, seed=0)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    n0, o0 = port.bvh()
    n1, o1 = ref.bvh()
    assert np.array_equal(n0, n1) and np.array_equal(o0, o1)
    rays = scenes.traversal_rays(1 << 22, seed=0)[::4]
    p0, t0 = port.trace_closest(rays)
    p1, t1 = ref.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(bits(t0), bits(t1))
    srays = scenes.traversal_rays(1 << 22, seed=0, shadow=True)[::4]
    assert np.array_equal(port.trace_any(srays), ref.trace_any(srays))


@pytest.mark.parametrize("env", [True, False])
def test_image_maps_on_every_material_kind(env):
    """Image maps on the arguments of glass, metal, the 2015 Disney BSDF and
    Disney12 (8-bit checkers and float ramps on colours, roughness,
    transmission, ior, ...), evaluated at each hit's uv by the materials'
    shading (src/material/glass.cpp:117-140, metal.cpp:33-56,
    disney.cpp:604-639, disney_brdf.cpp:278-302): bit-exact films."""
    import dataclasses
    sc, cam, filt, par = scenes.mapped_materials(48, 24, 4, env=env)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    port.set_camera(cam, filt)
    ref.set_camera(cam, filt)
    a = port.render(par)
    assert np.array_equal(bits(a), bits(ref.render(par)))
    # the maps matter: the same scene with constants only renders another film
    sc.materials = [dataclasses.replace(m, tex_param=(0,) * 13) for m in sc.materials]
    flat = oracle.Oracle(sc, "port")
    flat.set_camera(cam, filt)
    assert not np.array_equal(bits(flat.render(par)), bits(a))


@pytest.mark.parametrize("seed", [0, 1])
def test_adversarial_rays(seed):
    """Rays aimed exactly at triangle vertices, edge midpoints and centroids;
    axis-parallel rays whose origins lie on vertex coordinates (infinite
    inverse directions, slab planes through the origin); shadow rays whose
    t_max is the closest hit's distance and one ulp either side of it. Hits
    and occlusion flags equal the reference build's bit for bit."""
    sc = scenes.random_scene(seed, n_tris=400, n_spheres=6)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    rays = scenes.adversarial_rays(sc, seed)
    p0, t0 = port.trace_closest(rays)
    p1, t1 = ref.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(bits(t0), bits(t1))
    assert (p0 >= 0).mean() > 0.3
    for step in (-1, 0, 1):
        s = scenes.shadow_rays_at_hits(rays, p0, t0, step)
        assert np.array_equal(port.trace_any(s), ref.trace_any(s)), step


@pytest.mark.parametrize("seed", [0, 1])
def test_sphere_edge_rays(seed):
    """Rays passing each sphere at 1 - 1e-6 to 1 + 1e-5 radii from its centre
    (the hit/miss transition of the quadratic lies in between), rays from
    its centre and from a point on its surface: hits, distances and
    occlusion flags equal the reference build's."""
    sc = scenes.random_scene(seed, n_tris=20, n_spheres=12)
    port, ref = oracle.Oracle(sc, "port"), oracle.Oracle(sc, "reference")
    m = sc.sphere_to_world.reshape(-1, 4, 4)
    centre = m[:, :3, 3].astype(np.float32)
    r = (sc.sphere_radius * np.abs(m[:, 0, 0])).astype(np.float32)  # uniform scale in these scenes
    o, d = [], []
    for c, rad in zip(centre, r):
        for k, axis in enumerate(np.eye(3, dtype=np.float32)):
            side = np.eye(3, dtype=np.float32)[(k + 1) % 3]
            for f in (1 - 1e-6, 1.0, 1 + 1e-6, 1 + 2e-6, 1 + 3e-6, 1 + 5e-6, 1 + 1e-5):
                o.append(c + side * np.float32(rad * f) - axis * np.float32(3))
                d.append(axis)
            o.append(c)  # from the centre
            d.append(axis)
            o.append(c + side * rad)  # from the surface, into the sphere and out of it
            d.append(-side)
            o.append(c + side * rad)
            d.append(side)
    rays = scenes.make_rays(np.array(o, np.float32), np.array(d, np.float32), 0.0, scenes.F32_MAX)
    p0, t0 = port.trace_closest(rays)
    p1, t1 = ref.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(bits(t0), bits(t1))
    for step in (-1, 0, 1):
        s = scenes.shadow_rays_at_hits(rays, p0, t0, step)
        assert np.array_equal(port.trace_any(s), ref.trace_any(s)), step
