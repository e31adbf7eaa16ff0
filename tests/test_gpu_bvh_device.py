"""The device BVH builder (TR_BVH_DEVICE, parallel locally-ordered
clustering): its tree differs from the reference's, so hits are compared
with the oracle's up to equal-distance ties, and renders with the renders
over the reference tree (same seeds: identical paths wherever every hit is
the same)."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


class device_tree:
    def __init__(self, gpu):
        self.gpu = gpu

    def __enter__(self):
        self.gpu.set_bvh_builder(True)
        return self.gpu

    def __exit__(self, *exc):
        self.gpu.set_bvh_builder(False)


def _rays(rng, n, lo, hi, shadow):
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    tmax = rng.uniform(0.0, 3.0, n).astype(np.float32) if shadow else scenes.F32_MAX
    return scenes.make_rays(o, d, 0.0, tmax)


@pytest.mark.parametrize("case", ["random", "traversal", "room"])
def test_device_tree_hits_equal_the_oracle(gpu, case):
    rng = np.random.default_rng(3)
    if case == "random":
        sc = scenes.random_scene(5, n_tris=3000, n_spheres=0)
        rays, srays = _rays(rng, 40000, -2, 2, False), _rays(rng, 40000, -2, 2, True)
    elif case == "traversal":
        sc = scenes.traversal(1 << 16, seed=2)
        rays = scenes.traversal_rays(1 << 16, seed=2)
        srays = scenes.traversal_rays(1 << 16, seed=2, shadow=True)
    else:
        sc = scenes.occluded_room(32, 24, 1, n_tris=30000)[0]
        rays, srays = _rays(rng, 40000, [-3.9, 0.1, -2.9], [3.9, 3.9, 2.9], False), \
            _rays(rng, 40000, [-3.9, 0.1, -2.9], [3.9, 3.9, 2.9], True)
    orc = oracle.Oracle(sc, "port")
    p0, t0 = orc.trace_closest(rays)
    a0 = orc.trace_any(srays)
    with device_tree(gpu):
        gpu.upload(sc)
        p1, t1 = gpu.trace_closest(rays)
        a1 = gpu.trace_any(srays)
    gpu.upload(sc)  # back to the reference tree for later tests
    same_t = t0.view(np.uint32) == t1.view(np.uint32)
    same_p = p0 == p1
    print(case, "closest: t equal", same_t.mean(), "prim equal", same_p.mean(), "any equal", (a0 == a1).mean())
    # a different primitive only at the same distance (a tie), except for
    # the rare ray whose box the reference's slab test culls
    assert same_t.mean() >= 0.999
    assert (same_p | same_t).mean() >= 0.999
    assert (a0 == a1).mean() >= 0.999
    assert ((p1 >= 0) == (p0 >= 0)).mean() >= 0.999


@pytest.mark.parametrize("make", [lambda: scenes.cornell(64, 64, 4), lambda: scenes.occluded_room(64, 48, 4, n_tris=20000),
                                  lambda: scenes.outdoor(64, 48, 4, glass=False)])
def test_device_tree_renders_the_same_image(gpu, make):
    sc, cam, filt, par = make()
    gpu.upload(sc)
    ref, rs = gpu.render(cam, filt, par)
    with device_tree(gpu):
        gpu.upload(sc)
        got, ds = gpu.render(cam, filt, par)
    gpu.upload(sc)
    same = np.all(ref.view(np.uint32) == got.view(np.uint32), axis=-1)
    print("pixels bit-identical", same.mean(), "samples", rs.samples, ds.samples)
    assert rs.samples == ds.samples
    assert same.mean() >= 0.99
    img = lambda a: a[..., :3] / a[..., 3:4]
    # the few pixels whose paths part (a tie) draw different random numbers
    # from there on: their difference is noise
    assert abs(img(ref).mean() - img(got).mean()) <= 1e-2 * img(ref).mean()


def test_device_tree_scene_set(gpu):
    import torch
    items = [scenes.batch_scene(k, tri_range=(2000, 20000)) for k in range(4)]
    films = {}
    for device in (False, True):
        gpu.set_bvh_builder(device)
        gpu.upload_set([it[0] for it in items])
        fs = [torch.zeros((p.height, p.width, 4), device="cuda:0") for _, _, _, p in items]
        torch.cuda.synchronize()
        gpu.render_batch_dev([(k, it[1], it[2], it[3], fs[k].data_ptr()) for k, it in enumerate(items)])
        films[device] = [f.cpu().numpy() for f in fs]
    gpu.set_bvh_builder(False)
    for a, b in zip(films[False], films[True]):
        same = np.all(a.view(np.uint32) == b.view(np.uint32), axis=-1)
        print("scene pixels bit-identical", same.mean())
        assert same.mean() >= 0.98


def test_device_tree_refuses_export(gpu):
    from tracer_gb300.native import TracerError
    sc = scenes.cornell(8, 8, 1)[0]
    with device_tree(gpu):
        gpu.upload(sc)
        with pytest.raises(TracerError):
            gpu.bvh()
    gpu.upload(sc)
