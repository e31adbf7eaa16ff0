"""Batched rendering of a scene set (with an environment light, glass, metal
and Disney 2015 scenes among area-lit ones): every job's film equals the
film of the same render done alone, and CUDA-graph replay changes nothing."""
import numpy as np
import pytest

from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _set():
    a = scenes.cornell(40, 32, 4)
    b = (scenes.random_scene(3, n_tris=60, n_spheres=8), scenes.random_camera(24, 20, 3), scenes.make_filter(0.5, 0.6),
         scenes.make_params(24, 20, 8, 1, 7, seed_base=39))
    c = scenes.disney_grid(32, 24, 2)
    d = scenes.occluded_room(48, 36, 4, n_tris=5000)
    e = scenes.outdoor(32, 24, 4)  # environment light, glass and metal
    f = scenes.disney15_row(32, 16, 2, env=False)
    g = scenes.outdoor(24, 16, 2, glass=False, textured=True)  # image maps (texture indices offset in the set)
    h = scenes.cornell(24, 24, 2, textured=True)
    return [a, b, c, d, e, f, g, h]


def test_batch_equals_single_renders(gpu):
    import torch
    items = _set()
    singles = []
    for sc, cam, filt, par in items:
        gpu.upload(sc)
        out, st = gpu.render(cam, filt, par)
        singles.append((out, st.samples))
    gpu.upload_set([it[0] for it in items])
    films = [torch.zeros((par.height, par.width, 4), device="cuda:0") for _, _, _, par in items]
    torch.cuda.synchronize()
    # scenes in another order than the set, one scene twice
    extra = torch.zeros_like(films[0])
    jobs = [(k, items[k][1], items[k][2], items[k][3], films[k].data_ptr()) for k in (2, 5, 7, 0, 4, 3, 6, 1)]
    jobs.append((0, items[0][1], items[0][2], items[0][3], extra.data_ptr()))
    torch.cuda.synchronize()
    st = gpu.render_batch_dev(jobs)
    assert st.samples == sum(s for _, s in singles) + singles[0][1]
    for k in range(len(items)):
        got = films[k].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), singles[k][0].view(np.uint32)), k
    assert np.array_equal(extra.cpu().numpy().view(np.uint32), singles[0][0].view(np.uint32))


def test_graph_replay_changes_nothing(gpu):
    sc, cam, filt, par = scenes.occluded_room(64, 48, 8, n_tris=5000)
    gpu.upload(sc)
    old = gpu.tuning()
    try:
        outs = []
        for g in (0, 2, 8, 16):
            gpu.set_tuning(graph_iterations=g)
            out, st = gpu.render(cam, filt, par)
            assert st.samples == 64 * 48 * 8
            outs.append(out)
        for o in outs[1:]:
            assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
    finally:
        gpu.set_tuning(old.trav_refill_lanes, old.trav_blocks_per_sm, old.shade_blocks_per_sm, old.graph_iterations,
                       old.any_node_width, old.ray_bin_bits, old.treelet_nodes, old.occluder_cache,
                       old.render_mode)


def test_scene_set_traversal_uses_scene_zero(gpu):
    sc0, _, _, _ = scenes.cornell(8, 8, 1)
    sc1 = scenes.random_scene(1, n_tris=30, n_spheres=3)
    gpu.upload(sc0)
    rays = scenes.make_rays(np.tile([[0.0, 0.0, 3.0]], (64, 1)), np.random.default_rng(0).normal(size=(64, 3)) +
                            [0, 0, -3], 0.0, 3.4e38)
    p0, t0 = gpu.trace_closest(rays)
    gpu.upload_set([sc0, sc1])
    p1, t1 = gpu.trace_closest(rays)
    assert np.array_equal(p0, p1) and np.array_equal(t0.view(np.uint32), t1.view(np.uint32))


def test_autotune_picks_a_valid_tuning_and_keeps_results(gpu):
    import torch
    items = _set()
    gpu.upload_set([it[0] for it in items])
    films = [torch.zeros((p.height, p.width, 4), device="cuda:0") for _, _, _, p in items]
    torch.cuda.synchronize()
    jobs = [(k, it[1], it[2], it[3], films[k].data_ptr()) for k, it in enumerate(items)]
    gpu.render_batch_dev(jobs)
    before = [f.cpu().numpy() for f in films]
    old = gpu.tuning()
    try:
        best, ms = gpu.autotune(jobs, probe_spp=1)
        assert ms > 0
        t = gpu.tuning()
        fields = ("trav_refill_lanes", "trav_blocks_per_sm", "shade_blocks_per_sm", "graph_iterations", "any_node_width")
        assert [getattr(t, f) for f in fields] == [getattr(best, f) for f in fields]
        assert 1 <= t.trav_refill_lanes <= 32 and t.shade_blocks_per_sm >= 1 and t.any_node_width in (2, 4)
        gpu.render_batch_dev(jobs)
        for b, f in zip(before, films):
            assert np.array_equal(b.view(np.uint32), f.cpu().numpy().view(np.uint32))
    finally:
        gpu.set_tuning(old.trav_refill_lanes, old.trav_blocks_per_sm, old.shade_blocks_per_sm, old.graph_iterations,
                       old.any_node_width, old.ray_bin_bits, old.treelet_nodes, old.occluder_cache,
                       old.render_mode)
