"""Learned light sampling of guided renders (tr_guide_light_init /
tr_guide_light_update, tr_guide_params.light_guide / light_record).

Next-event estimation samples a point on every light per vertex
(sample_area_light, src/renderer/direct_illumination.cpp:35-71, through
UniformSampleTriangle, src/shape/triangle.cpp:61-97). With a light table the
point is drawn from a learned distribution over cells of the light's sample
square instead of uniformly, and the estimate is divided by that density over
the uniform one; the MIS weights stay the reference's. The estimate's
expectation is unchanged, so the image converges to the plain renderer's:
these tests compare block means at high sample counts, and check that the
learned table lowers the error of the occluded-light room."""
import numpy as np
import pytest

from tracer_gb300 import scenes
from tracer_gb300.abi import TR_ERR_ARG, TR_ERR_STATE, make_guide
from tracer_gb300.native import TracerError

pytestmark = pytest.mark.gpu

ROOM_BOX = ((-4.0, 0.0, -3.0), (4.0, 4.0, 3.0))


def _film(gpu, cam, filt, par, guide):
    import torch
    out = torch.zeros((par.height, par.width, 4), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    st = gpu.render_guided_dev(cam, filt, par, guide, out.data_ptr(), True)
    return out.cpu().numpy(), st


def _image(acc):
    w = acc[..., 3:4]
    return np.where(w > 0, acc[..., :3] / np.where(w > 0, w, 1), 0)


def test_light_table_arguments(gpu):
    sc, cam, filt, par = scenes.cornell(16, 16, 1)
    gpu.upload(sc)
    with pytest.raises(TracerError) as e:
        _film(gpu, cam, filt, par, make_guide(0.0, (-1, -1, -1), (1, 1, 1), light_guide=True))
    assert e.value.status == TR_ERR_STATE  # no table for this scene yet
    gpu.guide_light_init((4, 4, 4), 4)
    with pytest.raises(TracerError) as e:
        _film(gpu, cam, filt, par, make_guide(0.0, (-1, -1, -1), (1, 1, 1), light_record=True))
    assert e.value.status == TR_ERR_ARG  # statistics need the table's bins
    with pytest.raises(TracerError):
        gpu.guide_light_init((4, 4, 4), 17)
    with pytest.raises(TracerError):
        gpu.guide_light_update(0.0)
    out, st = _film(gpu, cam, filt, par, make_guide(0.0, (-1, -1, -1), (1, 1, 1), light_guide=True,
                                                    light_record=True))
    assert st.samples == 16 * 16 and np.isfinite(out).all()
    gpu.guide_light_update(0.3)


def test_uniform_table_keeps_the_plain_expectation(gpu):
    """A fresh table is uniform: the same density as the reference's light
    sample, drawn through the bins (another map of the same two draws), so
    the image keeps the plain expectation. Cornell box, 8x8-pixel blocks at
    1024 spp."""
    sc, cam, filt, _ = scenes.cornell(32, 32, 1)
    gpu.upload(sc)
    gpu.guide_light_init((4, 4, 4), 8)
    par = scenes.make_params(32, 32, 1024, 5, 5, seed_base=1)
    plain, _ = gpu.render(cam, filt, par, fp64=True)
    par_g = scenes.make_params(32, 32, 1024, 5, 5, seed_base=7_000_000)
    guided, st = _film(gpu, cam, filt, par_g, make_guide(0.0, (-1, -1, -1), (1, 1, 1), light_guide=True))
    a = _image(plain).reshape(4, 8, 4, 8, 3).mean((1, 3))
    b = _image(guided).reshape(4, 8, 4, 8, 3).mean((1, 3))
    rel = np.abs(a - b) / np.maximum(a, 1e-3)
    print(f"block means: max rel diff {rel.max():.4f}, image mean plain {a.mean():.5f} light-guided {b.mean():.5f}")
    assert abs(a.mean() - b.mean()) <= 0.01 * a.mean()
    assert rel.max() < 0.08


def _learn_room(gpu, cam, filt, passes=3, spp=16):
    gpu.guide_light_init((16, 8, 12), 8)
    for k in range(passes):
        par = scenes.make_params(64, 48, spp, 3, 10, seed_base=100 + k * 64 * 48)
        _film(gpu, cam, filt, par, make_guide(0.0, *ROOM_BOX, light_guide=True, light_record=True))
        gpu.guide_light_update(0.2)


def test_learned_table_keeps_the_plain_expectation_in_the_room(gpu):
    """The occluded-light room with a learned table: the light samples now
    concentrate on the part of the light cube seen through the slit. Block
    means over 16x16-pixel blocks at 4096 spp match the plain renderer's."""
    sc, cam, filt, _ = scenes.occluded_room(64, 48, 8, n_tris=20000)
    gpu.upload(sc)
    _learn_room(gpu, cam, filt)
    par = scenes.make_params(64, 48, 4096, 3, 10, seed_base=1)
    plain, _ = gpu.render(cam, filt, par, fp64=True)
    par_g = scenes.make_params(64, 48, 4096, 3, 10, seed_base=9_000_000)
    guided, st = _film(gpu, cam, filt, par_g, make_guide(0.0, *ROOM_BOX, light_guide=True))
    assert st.samples == 64 * 48 * 4096
    a = _image(plain).reshape(3, 16, 4, 16, 3).mean((1, 3))
    b = _image(guided).reshape(3, 16, 4, 16, 3).mean((1, 3))
    rel = np.abs(a - b) / np.maximum(a, 1e-3)
    print(f"room block means: max rel diff {rel.max():.4f}, image mean plain {a.mean():.5f} guided {b.mean():.5f}")
    assert abs(a.mean() - b.mean()) <= 0.01 * a.mean()
    assert rel.max() < 0.04


def test_learned_table_lowers_the_error(gpu):
    """At equal sample counts the learned light sample has lower error
    against a converged image than the uniform one (the variance the slit
    causes: most uniform light samples are blocked)."""
    sc, cam, filt, _ = scenes.occluded_room(64, 48, 8, n_tris=20000)
    gpu.upload(sc)
    ref, _ = gpu.render(cam, filt, scenes.make_params(64, 48, 4096, 3, 10, seed_base=5), fp64=True)
    ref = _image(ref)
    _learn_room(gpu, cam, filt)

    def rel_mse(img):
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))
    par = scenes.make_params(64, 48, 32, 3, 10, seed_base=77_000_000)
    plain, _ = gpu.render(cam, filt, par, fp64=True)
    learned, _ = _film(gpu, cam, filt, par, make_guide(0.0, *ROOM_BOX, light_guide=True))
    e_plain, e_learned = rel_mse(_image(plain)), rel_mse(_image(learned))
    print(f"relMSE at 32 spp: uniform light samples {e_plain:.4f}, learned {e_learned:.4f}")
    assert e_learned < 0.8 * e_plain
