"""Parity at the configured sizes, not only at scaled-down ones.

* The traversal workload at full size: 1,048,576 triangles (SAH BVH, leaves
  of at most 4), 4,194,304 closest-hit rays and 4,194,304 shadow rays. The
  BVH is node-for-node the oracle's; closest-hit primitive ids and t bits and
  any-hit flags are bit-exact against the oracle (the reference's
  BVHAccel::intersect_p / intersect, src/accelerator/bvh.cpp:112-185), for
  the binary and the four-wide any-hit trees.
* The occluded-light room the bench renders: 500,000 triangles of furniture,
  12 emissive triangles, 1024 x 768 at 16 spp, depth 10. The BVH is the
  oracle's node for node, and every closest/any query that the oracle's
  integrator makes for 8,192 pixels spread over the whole frame replays on
  the GPU with identical results. That covers the deep tree, the 96-entry
  traversal stack and the speculative walk on the benchmarked geometry.
* A thin-lens camera (lens radius > 0, focal distance != 1,
  src/camera/thin_lens_camera.cpp:40-59): replayed traces and the image.
"""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def traversal_full():
    sc = scenes.traversal(1 << 20, seed=0)
    return sc, oracle.Oracle(sc, "port")


def test_traversal_full_size_bvh(gpu, traversal_full):
    sc, orc = traversal_full
    gpu.upload(sc)
    n0, o0 = orc.bvh()
    n1, o1 = gpu.bvh()
    print("nodes", len(n0))
    assert len(n0) > (1 << 18)
    assert np.array_equal(n0, n1) and np.array_equal(o0, o1)


def test_traversal_full_size_closest(gpu, traversal_full):
    sc, orc = traversal_full
    gpu.upload(sc)
    rays = scenes.traversal_rays(1 << 22, seed=0)
    p0, t0 = orc.trace_closest(rays)
    p1, t1 = gpu.trace_closest(rays)
    print("closest hits", int((p0 >= 0).sum()), "of", len(rays))
    assert np.array_equal(p0, p1)
    assert np.array_equal(_bits(t0), _bits(t1))


@pytest.mark.parametrize("width", [2, 4])
def test_traversal_full_size_any(gpu, traversal_full, width):
    from conftest import tuned
    sc, orc = traversal_full
    gpu.upload(sc)
    rays = scenes.traversal_rays(1 << 22, seed=0, shadow=True)
    want = orc.trace_any(rays)
    with tuned(gpu, any_node_width=width):
        got = gpu.trace_any(rays)
    print("occluded", int(want.sum()), "of", len(rays))
    assert np.array_equal(want, got)


@pytest.fixture(scope="module")
def room_full():
    sc, cam, filt, par = scenes.occluded_room(1024, 768, 16)
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    return sc, cam, filt, par, orc


def test_room_full_size_bvh(gpu, room_full):
    sc, _, _, _, orc = room_full
    assert len(sc.prim_shape) >= 500_000
    gpu.upload(sc)
    n0, o0 = orc.bvh()
    n1, o1 = gpu.bvh()
    print("nodes", len(n0))
    assert np.array_equal(n0, n1) and np.array_equal(o0, o1)


def test_room_full_size_replay(gpu, room_full):
    """Every query of 32 runs of 256 pixels, evenly spaced over the frame,
    at the bench's 16 spp and depth 10."""
    from conftest import tuned
    sc, cam, filt, par, orc = room_full
    npix = par.width * par.height
    logs = [orc.render_log(par, p0, p0 + 256) for p0 in range(0, npix, npix // 32)]
    cr = np.concatenate([l[0] for l in logs])
    cp = np.concatenate([l[1] for l in logs])
    ct = np.concatenate([l[2] for l in logs])
    ar = np.concatenate([l[3] for l in logs])
    ah = np.concatenate([l[4] for l in logs])
    print("closest queries", len(cr), "hits", int((cp >= 0).sum()), "shadow queries", len(ar),
          "occluded", int(ah.sum()))
    assert len(cr) > 1_000_000 and len(ar) > 1_000_000
    gpu.upload(sc)
    p, t = gpu.trace_closest(cr)
    assert np.array_equal(p, cp)
    assert np.array_equal(_bits(t), _bits(ct))
    for width in (2, 4):
        with tuned(gpu, any_node_width=width):
            assert np.array_equal(gpu.trace_any(ar), ah)


def _thin_lens_cornell(w, h, spp):
    sc, _, filt, par = scenes.cornell(w, h, spp)
    cam = scenes.make_camera(w / h, (0.3, 0.2, 3.5), (0, -0.2, 0), (0, 1, 0), np.radians(40.0), 0.12, 3.1)
    return sc, cam, filt, par


def test_thin_lens_replay(gpu):
    sc, cam, filt, par = _thin_lens_cornell(32, 32, 4)
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    cr, cp, ct, ar, ah = orc.render_log(par, 0, 32 * 32)
    # camera rays start on the lens disk around the camera position, not at it
    off = np.linalg.norm(cr["o"] - np.float32([0.3, 0.2, 3.5]), axis=1)
    on_lens = off <= 0.1201
    assert on_lens.sum() >= 32 * 32 * 4 and (off[on_lens] > 0).mean() > 0.99
    gpu.upload(sc)
    p, t = gpu.trace_closest(cr)
    assert np.array_equal(p, cp)
    assert np.array_equal(_bits(t), _bits(ct))
    assert np.array_equal(gpu.trace_any(ar), ah)


def test_thin_lens_image(gpu):
    from test_gpu_render import _compare
    sc, cam, filt, par = _thin_lens_cornell(64, 64, 8)
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    ref = orc.render(par)
    gpu.upload(sc)
    out, stats = gpu.render(cam, filt, par)
    assert stats.samples == 64 * 64 * 8
    _compare(out, ref, 0.9)
