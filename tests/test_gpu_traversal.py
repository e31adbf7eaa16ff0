"""GPU traversal parity: closest-hit primitive ids and distances, and any-hit
flags, bit-exact against the oracle on the same rays (the reference's
Scene::intersect_p / Scene::intersect, src/core/scene.cpp:32-38)."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def _random_rays(rng, n, lo=-2.0, hi=2.0, shadow=False):
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    tmax = rng.uniform(0.0, 3.0, n).astype(np.float32) if shadow else scenes.F32_MAX
    return scenes.make_rays(o, d, 0.0, tmax)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_random_scene_closest_and_any(gpu, seed):
    sc = scenes.random_scene(seed, n_tris=120, n_spheres=12)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    rng = np.random.default_rng(seed)
    rays = _random_rays(rng, 20000)
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1)
    assert _same_bits(t0, t1)
    srays = _random_rays(rng, 20000, shadow=True)
    assert np.array_equal(orc.trace_any(srays), gpu.trace_any(srays))


@pytest.mark.parametrize("seed", [0, 1])
def test_adversarial_rays(gpu, seed):
    """Rays aimed exactly at triangle vertices, edge midpoints and centroids,
    axis-parallel rays with origins on vertex coordinates, and shadow rays
    ending exactly at (or one ulp either side of) the closest hit: the same
    hits, distances and occlusion flags as the oracle, which equals the
    reference build on these rays."""
    sc = scenes.random_scene(seed, n_tris=400, n_spheres=6)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    rays = scenes.adversarial_rays(sc, seed)
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1)
    assert _same_bits(t0, t1)
    for step in (-1, 0, 1):
        s = scenes.shadow_rays_at_hits(rays, p0, t0, step)
        assert np.array_equal(orc.trace_any(s), gpu.trace_any(s)), step


def test_bvh_matches_oracle(gpu):
    sc = scenes.random_scene(7, n_tris=300, n_spheres=20)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    n0, o0 = orc.bvh()
    n1, o1 = gpu.bvh()
    assert np.array_equal(n0, n1) and np.array_equal(o0, o1)


def test_traversal_workload_subset(gpu):
    """The 1M-triangle traversal workload's shapes at 1/16 scale."""
    sc = scenes.traversal(1 << 16, seed=0)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    rays = scenes.traversal_rays(1 << 16, seed=0)
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1)
    assert _same_bits(t0, t1)
    srays = scenes.traversal_rays(1 << 16, seed=0, shadow=True)
    assert np.array_equal(orc.trace_any(srays), gpu.trace_any(srays))


def test_uploaded_oracle_bvh(gpu):
    """Traversal of an externally built tree (tr_bvh_upload) matches too."""
    sc = scenes.random_scene(11, n_tris=200, n_spheres=5)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    nodes, order = orc.bvh()
    gpu.upload_bvh(nodes, order)
    rays = _random_rays(np.random.default_rng(5), 5000)
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1) and _same_bits(t0, t1)


def test_edge_cases(gpu):
    # axis-parallel directions (inverse direction = +-inf), rays from vertices
    # and edges (ties), NaN rays (miss, as in the reference)
    sc = scenes.cornell(8, 8, 1)[0]
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    o = []
    d = []
    for ax in range(3):
        for s in (-1.0, 1.0):
            dd = [0.0, 0.0, 0.0]
            dd[ax] = s
            for oo in ([0, 0, 0], [0.25, 0.5, -0.25], [-0.25, 0.99, -0.25], [1, 1, 1], [0.5, -1, 0.3]):
                o.append(oo)
                d.append(dd)
    pos = sc.positions[:30]
    for p in pos:
        o.append(p + np.float32(0.0))
        d.append([0.3, -1.0, 0.2])
    rays = scenes.make_rays(np.array(o, np.float32), np.array(d, np.float32), 0.0, scenes.F32_MAX)
    nan = rays[:3].copy()
    nan["d"][:, 0] = np.nan
    rays = np.concatenate([rays, nan])
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1) and _same_bits(t0, t1)
    assert np.array_equal(orc.trace_any(rays), gpu.trace_any(rays))


def test_empty_and_single(gpu):
    one = scenes._Builder()
    m = one.material(scenes.lambert((0.5, 0.5, 0.5)))
    one.triangle((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), m)
    sc = one.finish(3)
    gpu.upload(sc)
    rays = scenes.make_rays(np.array([[0.2, 0.2, 1.0], [2, 2, 1]], np.float32),
                            np.array([[0, 0, -1], [0, 0, -1]], np.float32), 0.0, scenes.F32_MAX)
    p, t = gpu.trace_closest(rays)
    assert p[0] == 0 and p[1] == -1 and t[0] == np.float32(1.0)
    empty = scenes._Builder()
    empty.material(scenes.lambert((0.5, 0.5, 0.5)))
    gpu.upload(empty.finish(3))
    p, t = gpu.trace_closest(rays)
    assert (p == -1).all()
    assert not gpu.trace_any(rays).any()


def test_trace_visit_counts_equal_the_oracle(gpu):
    """Boxes and primitives tested per traversal (the roofline's units)
    against the reference traversal's on the same rays: equal for closest
    hits. For any hits the primitive tests are equal; the boxes can only be
    more, because both child boxes are tested when their parent is visited
    while the reference tests a box when it pops it, and an early exit
    leaves pushed entries the reference never pops."""
    import torch
    import oracle
    sc = scenes.traversal(1 << 14, seed=3)
    rays_c = scenes.traversal_rays(1 << 13, seed=3, shadow=False)
    rays_a = scenes.traversal_rays(1 << 13, seed=3, shadow=True)
    orc = oracle.Oracle(sc, "port")
    _, _, cn, cp = orc.trace_closest(rays_c, counts=True)
    _, an, ap = orc.trace_any(rays_a, counts=True)
    gpu.upload(sc)
    dc = torch.from_numpy(rays_c.view(np.uint8)).to("cuda:0")
    da = torch.from_numpy(rays_a.view(np.uint8)).to("cuda:0")
    torch.cuda.synchronize()
    from conftest import tuned
    with tuned(gpu, any_node_width=2):
        got_c = gpu.trace_count_dev(dc.data_ptr(), len(rays_c), False)
        got_a = gpu.trace_count_dev(da.data_ptr(), len(rays_a), True)
    print("closest", got_c, (int(cn.sum()), int(cp.sum())), "any", got_a, (int(an.sum()), int(ap.sum())))
    assert got_c == (int(cn.sum()), int(cp.sum()))
    assert got_a[1] == int(ap.sum()) and int(an.sum()) <= got_a[0] <= int(an.sum()) * 1.05


@pytest.mark.parametrize("case", ["random0", "random1", "random2", "traversal", "room", "edges"])
def test_four_wide_any_hit_equals_the_oracle(gpu, case):
    """Any-hit traversal of the four-wide tree collapsed from the reference's
    binary BVH: the occlusion flags are the oracle's, bit for bit, and the
    primitive tests stay within the binary walk's set (an early exit can
    only stop sooner or elsewhere)."""
    from conftest import tuned
    rng = np.random.default_rng(17)
    if case.startswith("random"):
        sc = scenes.random_scene(int(case[-1]), n_tris=400, n_spheres=30)
        rays = _random_rays(rng, 30000, shadow=True)
    elif case == "traversal":
        sc = scenes.traversal(1 << 16, seed=1)
        rays = scenes.traversal_rays(1 << 16, seed=1, shadow=True)
    elif case == "edges":
        # axis-parallel rays (infinite inverse directions, NaN slabs where an
        # origin lies on a box plane) from vertices, from box-plane values and
        # from random points, with finite lengths
        sc = scenes.cornell(8, 8, 1)[0]
        pts = np.concatenate([sc.positions.astype(np.float32),
                              rng.choice(np.float32([-1, -0.5, 0, 0.25, 0.5, 0.99, 1]), (200, 3)),
                              rng.uniform(-1.2, 1.2, (200, 3)).astype(np.float32)])
        o, d = [], []
        for p in pts:
            for ax in range(3):
                for sgn in (-1.0, 1.0):
                    dd = np.zeros(3, np.float32)
                    dd[ax] = sgn
                    o.append(p)
                    d.append(dd)
        o, d = np.array(o, np.float32), np.array(d, np.float32)
        rays = scenes.make_rays(o, d, 0.0, rng.uniform(0.1, 3.0, len(o)).astype(np.float32))
    else:
        sc, cam, filt, par = scenes.occluded_room(32, 24, 1, n_tris=30000)
        o = rng.uniform([-3.9, 0.1, -2.9], [3.9, 3.9, 2.9], (30000, 3)).astype(np.float32)
        tgt = rng.uniform([4.5, 0.5, -1.5], [7.5, 3.5, 1.5], (30000, 3)).astype(np.float32)
        rays = scenes.make_rays(o, tgt - o, 0.0, np.linalg.norm(tgt - o, axis=1).astype(np.float32) * 0.999)
    orc = oracle.Oracle(sc, "port")
    gpu.upload(sc)
    nodes4, bound = gpu.any_tree_info()
    print(case, "four-wide nodes", nodes4, "stack bound", bound)
    assert nodes4 > 0 and bound <= 96
    want = orc.trace_any(rays)
    with tuned(gpu, any_node_width=4):
        assert gpu.tuning().any_node_width == 4
        got = gpu.trace_any(rays)
    print(case, "occluded", int(want.sum()), "of", len(rays))
    assert np.array_equal(want, got)


@pytest.mark.parametrize("bits,treelet", [(3, 0), (0, 64), (4, 256), (5, 1024), (2, 1)])
def test_binning_and_treelet_keep_results(gpu, bits, treelet):
    """Ray binning (the queue visited in octant/cell order) and the
    shared-memory treelet (the top of the tree read from shared memory)
    change only the order of work and where nodes are read from: hits stay
    bit-exact, on random scenes with spheres, the traversal workload and the
    occluded room."""
    from conftest import tuned
    rng = np.random.default_rng(bits * 100 + treelet)
    cases = [(scenes.random_scene(bits, n_tris=300, n_spheres=20), _random_rays(rng, 20000),
              _random_rays(rng, 20000, shadow=True)),
             (scenes.traversal(1 << 15, seed=2), scenes.traversal_rays(1 << 15, seed=2),
              scenes.traversal_rays(1 << 15, seed=2, shadow=True))]
    room = scenes.occluded_room(32, 24, 1, n_tris=30000)[0]
    o = rng.uniform([-3.9, 0.1, -2.9], [3.9, 3.9, 2.9], (20000, 3)).astype(np.float32)
    tgt = rng.uniform([4.5, 0.5, -1.5], [7.5, 3.5, 1.5], (20000, 3)).astype(np.float32)
    cases.append((room, scenes.make_rays(o, rng.normal(size=(20000, 3)).astype(np.float32), 0.0, scenes.F32_MAX),
                  scenes.make_rays(o, tgt - o, 0.0, np.linalg.norm(tgt - o, axis=1).astype(np.float32) * 0.999)))
    for sc, rays, srays in cases:
        orc = oracle.Oracle(sc, "port")
        p0, t0 = orc.trace_closest(rays)
        h0 = orc.trace_any(srays)
        gpu.upload(sc)
        with tuned(gpu, ray_bin_bits=bits, treelet_nodes=treelet):
            for width in (2, 4):
                with tuned(gpu, any_node_width=width):
                    p1, t1 = gpu.trace_closest(rays)
                    assert np.array_equal(p0, p1) and _same_bits(t0, t1)
                    assert np.array_equal(h0, gpu.trace_any(srays))


@pytest.mark.parametrize("order", [1, 2])
def test_any_hit_order_keeps_results(gpu, order):
    """tr_tuning.any_hit_order: a binary any-hit walk enters the far child,
    or the child with the larger box, first. Occlusion answers equal the
    oracle's (the reference's near-first walk) on random scenes with spheres,
    the traversal workload and the occluded room, and a wavefront render of
    the room is bit-identical."""
    from conftest import tuned
    from tracer_gb300.abi import TR_RENDER_MODE_WAVEFRONT
    rng = np.random.default_rng(40 + order)
    room = scenes.occluded_room(32, 24, 1, n_tris=30000)[0]
    o = rng.uniform([-3.9, 0.1, -2.9], [3.9, 3.9, 2.9], (20000, 3)).astype(np.float32)
    tgt = rng.uniform([4.5, 0.5, -1.5], [7.5, 3.5, 1.5], (20000, 3)).astype(np.float32)
    cases = [(scenes.random_scene(order, n_tris=300, n_spheres=20), _random_rays(rng, 20000, shadow=True)),
             (scenes.traversal(1 << 15, seed=3), scenes.traversal_rays(1 << 15, seed=3, shadow=True)),
             (room, scenes.make_rays(o, tgt - o, 0.0, np.linalg.norm(tgt - o, axis=1).astype(np.float32) * 0.999))]
    for sc, srays in cases:
        want = oracle.Oracle(sc, "port").trace_any(srays)
        gpu.upload(sc)
        with tuned(gpu, any_hit_order=order, any_node_width=2):
            assert np.array_equal(gpu.trace_any(srays), want)
    sc, cam, filt, par = scenes.occluded_room(48, 36, 4, n_tris=20000)
    gpu.upload(sc)
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        base, _ = gpu.render(cam, filt, par)
        with tuned(gpu, any_hit_order=order):
            got, _ = gpu.render(cam, filt, par)
    assert np.array_equal(got.view(np.uint32), base.view(np.uint32))
