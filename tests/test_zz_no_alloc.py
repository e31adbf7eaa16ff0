"""tr_render_dev_noalloc (no reference counterpart): the render with all
scratch in the library's static device array gives the same film as
tr_render_dev on two consecutive calls, and rejects films whose scratch
would not fit. Collected last so it also runs after every other GPU test
(it must pass alone as well)."""
import ctypes as C

import numpy as np
import pytest

from tracer_gb300 import scenes
from tracer_gb300.abi import TR_ERR_ARG, TrCamera, TrFilter, TrRenderParams, TrStats

pytestmark = pytest.mark.gpu

RTOL = 1e-6  # same kernels in the same order: expected bit-identical, checked to 1e-6 relative


def _noalloc(ctx):
    f = ctx.L.tr_render_dev_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.POINTER(TrCamera), C.POINTER(TrFilter), C.POINTER(TrRenderParams), C.c_void_p,
                  C.POINTER(TrStats)]
    return f


def _cases():
    sc, cam, filt, par = scenes.cornell(64, 64, 4)
    yield "cornell", sc, cam, filt, par
    sc = scenes.random_scene(0, n_tris=60, n_spheres=8)
    yield ("random", sc, scenes.random_camera(48, 40, 0), scenes.make_filter(0.5, 0.6),
           scenes.make_params(48, 40, 4, 1, 7, seed_base=5))
    sc, cam, filt, par = scenes.outdoor(48, 32, 4)  # environment light, glass, metal
    yield "outdoor", sc, cam, filt, par
    sc, cam, filt, par = scenes.disney15_row(48, 24, 4)
    yield "disney15", sc, cam, filt, par


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_noalloc_matches_render_dev_on_consecutive_calls(gpu, case):
    import torch
    name, sc, cam, filt, par = list(_cases())[case]
    H, W = par.height, par.width
    gpu.upload(sc)
    ref = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    st_ref = gpu.render_dev(cam, filt, par, ref.data_ptr())
    want = ref.cpu().numpy()
    f = _noalloc(gpu)
    for call in range(2):
        out = torch.full((H, W, 4), float("nan"), dtype=torch.float32, device="cuda:0")
        torch.cuda.synchronize()  # the fill runs on torch's stream, the render on the context's
        st = TrStats()
        free_before = torch.cuda.mem_get_info(0)[0]
        s = f(gpu.h, C.byref(cam), C.byref(filt), C.byref(par), out.data_ptr(), C.byref(st))
        assert s == 0, gpu.L.tr_ctx_last_error(gpu.h).decode()
        if call == 1:
            # after a first call (module and symbol set-up) the call takes no device memory
            assert torch.cuda.mem_get_info(0)[0] == free_before
        got = out.cpu().numpy()
        assert st.samples == st_ref.samples == W * H * par.spp
        assert st.extend_rays == st_ref.extend_rays and st.shadow_rays == st_ref.shadow_rays
        print(f"{name} call {call}: bit-identical pixels "
              f"{(got.view(np.uint32) == want.view(np.uint32)).all(-1).mean():.4f}")
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)


def test_noalloc_rejects_image_maps(gpu):
    """Materials with image maps need per-slot set-ups the static scratch has no room for."""
    import torch
    from tracer_gb300.abi import TR_ERR_UNSUPPORTED
    sc, cam, filt, par = scenes.cornell(16, 16, 1, textured=True)
    gpu.upload(sc)
    out = torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    assert _noalloc(gpu)(gpu.h, C.byref(cam), C.byref(filt), C.byref(par), out.data_ptr(), None) == TR_ERR_UNSUPPORTED


def test_noalloc_rejects_oversize_film(gpu):
    import torch
    sc, cam, filt, par = scenes.cornell(1024, 1024, 1)
    gpu.upload(sc)
    out = torch.zeros((1024, 1024, 4), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    f = _noalloc(gpu)
    s = f(gpu.h, C.byref(cam), C.byref(filt), C.byref(par), out.data_ptr(), None)
    assert s == TR_ERR_ARG
    msg = gpu.L.tr_ctx_last_error(gpu.h).decode()
    assert "scratch" in msg and "16777216" in msg, msg
    # a film that fits still renders after the rejection
    small = scenes.make_params(32, 32, 2, 5, 5)
    out = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    st = TrStats()
    assert f(gpu.h, C.byref(cam), C.byref(filt), C.byref(small), out.data_ptr(), C.byref(st)) == 0
    assert st.samples == 32 * 32 * 2


def test_noalloc_rejects_depth_beyond_16_bits(gpu):
    """The path depth is kept in 16 bits: max_depth above 65515 is an
    argument error for both render entry points, before any device work."""
    import torch
    sc, cam, filt, _ = scenes.cornell(8, 8, 1)
    gpu.upload(sc)
    out = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    deep = scenes.make_params(8, 8, 1, 70000, 70000)
    assert _noalloc(gpu)(gpu.h, C.byref(cam), C.byref(filt), C.byref(deep), out.data_ptr(), None) == TR_ERR_ARG
    assert "65515" in gpu.L.tr_ctx_last_error(gpu.h).decode()
    with pytest.raises(Exception):
        gpu.render_dev(cam, filt, deep, out.data_ptr())
