"""The output path on the device against the oracle's restatement (itself
equal to the reference's post-processors, tests/test_post.py): film
resolve, ACES tone mapping, gamma correction, the 8-bit image and RGBE."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _film(gpu):
    import torch
    sc, cam, filt, par = scenes.cornell(48, 32, 4)
    gpu.upload(sc)
    film, _ = gpu.render(cam, filt, par)
    film[0, 0] = 0.0  # a pixel with no weight
    return film, torch.from_numpy(film).to("cuda:0")


def test_resolve_aces_gamma(gpu):
    import torch
    film, d_film = _film(gpu)
    n = film.shape[0] * film.shape[1]
    d_rgb = torch.zeros((film.shape[0], film.shape[1], 3), device="cuda:0")
    gpu.film_resolve_dev(d_film.data_ptr(), n, d_rgb.data_ptr())
    gpu.synchronize()
    want = oracle.post_resolve(film)
    assert np.array_equal(d_rgb.cpu().numpy().view(np.uint32), want.view(np.uint32))
    for exposure in (1.0, 3.5, -2.0):
        d = d_rgb.clone()
        gpu.aces_tone_map_dev(d.data_ptr(), n, exposure)
        gpu.synchronize()
        w = oracle.post_process("port", want, "aces", exposure)
        assert np.array_equal(d.cpu().numpy().view(np.uint32), w.view(np.uint32))
    for gamma in (1 / 2.2, 2.2, 0.0):
        d = d_rgb.clone()
        gpu.gamma_correct_dev(d.data_ptr(), n, gamma)
        gpu.synchronize()
        w = oracle.post_process("port", want, "gamma", gamma)
        got = d.cpu().numpy()
        # CUDA's powf against glibc's: within 2 units in the last place
        ulps = np.abs(got.view(np.int32).astype(np.int64) - w.view(np.int32).astype(np.int64))
        assert ulps.max() <= 2


def test_rgb8_and_rgbe(gpu):
    import torch
    film, d_film = _film(gpu)
    h, w = film.shape[:2]
    n = h * w
    img = oracle.post_resolve(film)
    img[1, 1] = [np.nan, np.inf, -1.0]
    d_rgb = torch.from_numpy(img).to("cuda:0")
    d8 = torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda:0")
    d4 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda:0")
    gpu.to_rgb8_dev(d_rgb.data_ptr(), n, d8.data_ptr())
    gpu.to_rgbe_dev(d_rgb.data_ptr(), n, d4.data_ptr())
    gpu.synchronize()
    got8, want8 = d8.cpu().numpy().astype(int), oracle.post_rgb8(img).astype(int)
    assert np.abs(got8 - want8).max() <= 1 and (got8 == want8).mean() >= 0.999
    assert np.array_equal(d4.cpu().numpy(), oracle.post_rgbe(img))
