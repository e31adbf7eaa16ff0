"""The persistent render kernel (tr_tuning.render_mode = TR_RENDER_MODE_PERSISTENT):
every camera sample of a render, or of a batch of renders, in one launch,
each thread running a pixel's samples (eval_pixel_li,
src/renderer/path_trace_renderer.cpp:27-210, in the pixel order of
src/renderer/pixel_sampler_renderer.cpp:60-94) with its path state in
registers. It repeats the wavefront's arithmetic, random draws and sums, so
films are bit-identical to the wavefront's (and so as close to the oracle as
those); rays traced are the same count."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes
from tracer_gb300.abi import TR_RENDER_MODE_PERSISTENT, TR_RENDER_MODE_WAVEFRONT

pytestmark = pytest.mark.gpu


def _cases():
    yield "cornell", scenes.cornell(64, 64, 8)
    yield "room", scenes.occluded_room(64, 48, 8, n_tris=20000)
    sc = scenes.random_scene(4, n_tris=200, n_spheres=20)
    yield "random_spheres_rr", (sc, scenes.random_camera(48, 40, 4), scenes.make_filter(0.5, 0.6),
                                scenes.make_params(48, 40, 8, 1, 7, seed_base=9))
    yield "outdoor_env_glass_metal", scenes.outdoor(48, 32, 8)
    yield "disney15", scenes.disney15_row(48, 24, 8)
    yield "textured", scenes.cornell(48, 48, 8, textured=True)
    yield "disney_grid", scenes.disney_grid(48, 48, 4)
    yield "glass_rr", scenes.cornell(48, 48, 8, max_depth=8, min_depth=2, glass=True)
    sc = scenes.mixed_scene(1)
    yield "mixed", (sc, scenes.random_camera(48, 32, 1), scenes.make_filter(0.5, 0.6),
                    scenes.make_params(48, 32, 8, 2, 7, seed_base=31))


@pytest.mark.parametrize("case", range(9))
def test_persistent_equals_wavefront(gpu, case):
    from conftest import tuned
    name, (sc, cam, filt, par) = list(_cases())[case]
    gpu.upload(sc)
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        want, s0 = gpu.render(cam, filt, par)
    for graphs in (8, 0):
        with tuned(gpu, render_mode=TR_RENDER_MODE_PERSISTENT, graph_iterations=graphs):
            got, s1 = gpu.render(cam, filt, par)
        print(f"{name} graphs {graphs}: samples {s1.samples}, extend {s1.extend_rays} ({s0.extend_rays}), "
              f"shadow {s1.shadow_rays} ({s0.shadow_rays}), {s1.device_ms:.2f} ms vs {s0.device_ms:.2f} ms")
        assert s1.iterations == 1  # one launch
        assert s1.samples == s0.samples == par.width * par.height * par.spp
        assert s1.extend_rays == s0.extend_rays and s1.shadow_rays == s0.shadow_rays
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_persistent_fp64_and_wide_filter(gpu):
    from conftest import tuned
    sc, cam, filt, par = scenes.cornell(32, 32, 4)
    gpu.upload(sc)
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        w64, _ = gpu.render(cam, filt, par, fp64=True)
    with tuned(gpu, render_mode=TR_RENDER_MODE_PERSISTENT):
        p64, _ = gpu.render(cam, filt, par, fp64=True)
    assert np.array_equal(w64.view(np.uint64), p64.view(np.uint64))
    # a filter wider than a pixel scatters into neighbours with atomics:
    # the order of the additions is not fixed in either mode
    wide = scenes.make_filter(1.5, 0.6)
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        a, _ = gpu.render(cam, wide, par)
    with tuned(gpu, render_mode=TR_RENDER_MODE_PERSISTENT):
        b, _ = gpu.render(cam, wide, par)
    np.testing.assert_allclose(b, a, rtol=1e-5, atol=1e-6)


def test_persistent_against_the_oracle(gpu):
    """The Cornell box configuration (256 x 256 at 16 spp, depth 5) renders
    with the persistent kernel by default and agrees with the oracle like
    the wavefront does."""
    from test_gpu_render import _compare
    sc, cam, filt, par = scenes.cornell(256, 256, 16)
    gpu.upload(sc)
    out, st = gpu.render(cam, filt, par)
    assert st.iterations == 1 and st.samples == 256 * 256 * 16
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    rows = np.arange(0, 256, 16)
    ref, _ = orc.render_rows(par, rows)
    _compare(out[rows], ref, 0.9)


def test_persistent_batch(gpu):
    """A batch of renders of several scenes, sizes and sample counts as one
    launch of the persistent kernel: films equal the wavefront's."""
    import torch
    from conftest import tuned
    from tracer_gb300.abi import TrBatchJob
    sets = [scenes.cornell(8, 8, 1)[0], scenes.random_scene(3, n_tris=80, n_spheres=6),
            scenes.occluded_room(8, 8, 1, n_tris=5000)[0]]
    gpu.upload_set(sets)
    specs = [(0, 40, 32, 4, 5, 5), (1, 24, 24, 8, 1, 6), (2, 48, 36, 2, 3, 10), (0, 16, 16, 16, 2, 7)]
    films_w, films_p, jobs_w, jobs_p = [], [], [], []
    for i, (scn, W, H, spp, mind, maxd) in enumerate(specs):
        cam = scenes.cornell(W, H, 1)[1] if scn == 0 else (scenes.random_camera(W, H, 3) if scn == 1 else
                                                             scenes.occluded_room(W, H, 1, n_tris=5000)[1])
        for films, jobs in ((films_w, jobs_w), (films_p, jobs_p)):
            f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda:0")
            films.append(f)
            jobs.append((scn, cam, scenes.make_filter(0.5, 0.6),
                         scenes.make_params(W, H, spp, mind, maxd, seed_base=100 * i), f.data_ptr()))
    torch.cuda.synchronize()
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        sw = gpu.render_batch_dev(jobs_w)
    with tuned(gpu, render_mode=TR_RENDER_MODE_PERSISTENT):
        sp = gpu.render_batch_dev(jobs_p)
    assert sp.iterations == 1 and sp.samples == sw.samples
    for a, b in zip(films_w, films_p):
        assert np.array_equal(a.cpu().numpy().view(np.uint32), b.cpu().numpy().view(np.uint32))
