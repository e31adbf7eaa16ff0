"""The occluder cache of a render (tr_tuning.occluder_cache): each (pixel
slot, light) remembers the primitive that last blocked its shadow ray and
tests it, after its BVH leaf's box, before walking the tree. A ray that
passes the leaf's box passes every box above it (the slab test is monotone
under box containment), so the reference's any-hit walk
(src/accelerator/bvh.cpp:112-147) would reach that primitive: the occlusion
answers, and so the films, are bit-identical with the cache on and off."""
import numpy as np
import pytest

from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _cases():
    yield "cornell", scenes.cornell(64, 64, 8)
    yield "room", scenes.occluded_room(64, 48, 8, n_tris=20000)
    sc = scenes.random_scene(2, n_tris=200, n_spheres=20)
    yield "random_spheres", (sc, scenes.random_camera(48, 40, 2), scenes.make_filter(0.5, 0.6),
                             scenes.make_params(48, 40, 8, 1, 7, seed_base=3))
    yield "outdoor_env", scenes.outdoor(48, 32, 8)
    yield "disney_grid", scenes.disney_grid(48, 48, 4)
    yield "metal_glass", scenes.cornell(48, 48, 8, max_depth=8, min_depth=2, glass=True, metal=True)


@pytest.mark.parametrize("case", range(6))
@pytest.mark.parametrize("mode", ["wavefront", "persistent"])
def test_occluder_cache_keeps_the_film(gpu, case, mode):
    """Both execution models: the wavefront's k_shadow (binary and four-wide
    any-hit trees) and the persistent kernel's per-lane cache."""
    from conftest import tuned
    from tracer_gb300.abi import TR_RENDER_MODE_PERSISTENT, TR_RENDER_MODE_WAVEFRONT
    rm = TR_RENDER_MODE_WAVEFRONT if mode == "wavefront" else TR_RENDER_MODE_PERSISTENT
    name, (sc, cam, filt, par) = list(_cases())[case]
    gpu.upload(sc)
    with tuned(gpu, occluder_cache=0, render_mode=rm):
        off, st0 = gpu.render(cam, filt, par)
    for width in ((2, 4) if mode == "wavefront" else (2,)):
        with tuned(gpu, occluder_cache=1, any_node_width=width, render_mode=rm):
            on, st1 = gpu.render(cam, filt, par)
        assert (st1.iterations == 1) == (mode == "persistent")
        print(f"{name} {mode} width {width}: shadow rays {st1.shadow_rays}, answered by the cache {st1.occluder_hits}")
        assert st0.occluder_hits == 0
        assert st1.shadow_rays == st0.shadow_rays
        assert np.array_equal(on.view(np.uint32), off.view(np.uint32))
    if name in ("cornell", "room"):
        assert st1.occluder_hits > 0
