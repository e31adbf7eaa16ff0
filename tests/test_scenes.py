"""Synthetic workloads: sizes and invariants the parity tests rely on."""
import numpy as np

from tracer_gb300 import scenes


def test_cornell_shape():
    sc, cam, filt, par = scenes.cornell()
    assert len(sc.indices) == 36 and len(sc.light_prims) == 2
    assert (par.width, par.height, par.spp, par.max_depth) == (256, 256, 16, 5)
    assert par.min_depth >= par.max_depth  # no Russian roulette
    assert np.allclose(sc.prim_emission[sc.light_prims], [17, 12, 4])


def test_disney_grid_shape():
    sc, cam, filt, par = scenes.disney_grid(64, 64, 1)
    assert len(sc.sphere_radius) == 256 and len(sc.light_prims) == 4
    assert all(m.sheen_tint == 0.5 for m in sc.materials[1:])


def test_normals_are_fixed_points():
    sc = scenes.random_scene(3, n_tris=200)
    n = sc.normals
    assert np.array_equal(scenes.ref_normalize(n).view(np.uint32), n.view(np.uint32))


def test_no_negative_zero_positions():
    sc = scenes.cornell()[0]
    assert not np.any(np.signbit(sc.positions) & (sc.positions == 0))


def test_traversal_rays():
    r = scenes.traversal_rays(1000, seed=0)
    s = scenes.traversal_rays(1000, seed=0, shadow=True)
    o = r["o"]
    on_face = np.any((o == 0) | (o == 1), axis=1)
    assert on_face.all()
    assert (s["t_max"] >= 0).all() and (s["t_max"] < 1).all()
    assert np.allclose(np.linalg.norm(r["d"], axis=1), 1, atol=1e-6)


def test_pack_roundtrip():
    sc = scenes.random_scene(1, n_tris=10, n_spheres=3)
    sc2 = scenes.unpack_scene(scenes.pack_scene(sc))
    for k in ("positions", "normals", "indices", "prim_shape", "sphere_to_local"):
        assert np.array_equal(getattr(sc, k), getattr(sc2, k))
    assert [m.to_c().kind for m in sc.materials] == [m.to_c().kind for m in sc2.materials]
