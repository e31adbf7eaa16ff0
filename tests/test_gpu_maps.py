"""Image maps on the arguments of glass, metal, the 2015 Disney BSDF and
Disney12 on the GPU: at each hit of such a material its mapped arguments are
evaluated at the hit's uv and the material is set up again (the shading
functions src/material/glass.cpp:117-140, metal.cpp:33-56,
disney.cpp:604-639, disney_brdf.cpp:278-302), against the oracle, which is
pinned bit for bit to the reference build on the same scene
(test_oracle_vs_reference.py)."""
import numpy as np
import pytest

import oracle
from tracer_gb300 import scenes
from tracer_gb300.abi import TR_RENDER_MODE_PERSISTENT, TR_RENDER_MODE_WAVEFRONT

pytestmark = pytest.mark.gpu


def _image(acc):
    w = acc[..., 3:4]
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(w > 0, acc[..., :3] / w, 0.0)


@pytest.mark.parametrize("env", [True, False])
def test_maps_on_every_kind_against_the_oracle(gpu, env):
    sc, cam, filt, par = scenes.mapped_materials(96, 48, 8, env=env)
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    ref = orc.render(par)
    gpu.upload(sc)
    out, st = gpu.render(cam, filt, par)
    assert st.samples == 96 * 48 * 8
    # Paths agree until a last-bit difference of CUDA's and glibc's
    # transcendentals enters refraction in the glass sphere: most pixels
    # agree within 1e-5, the image mean within 1%.
    a, b = _image(out.astype(np.float64)), _image(ref.astype(np.float64))
    rel = (np.abs(a - b) / np.maximum(np.abs(b), 1e-6)).max(-1)
    print(f"within 1e-5: {(rel <= 1e-5).mean():.4f}, image means {a.mean():.5f} {b.mean():.5f}")
    assert (rel <= 1e-5).mean() >= 0.8
    assert abs(a.mean() - b.mean()) <= 0.01 * b.mean()


def test_maps_replay_recorded_rays(gpu):
    """Every trace of the oracle's integrator in the mapped scene, replayed."""
    sc, cam, filt, par = scenes.mapped_materials(32, 16, 4)
    orc = oracle.Oracle(sc, "port")
    orc.set_camera(cam, filt)
    cr, cp, ct, ar, ah = orc.render_log(par, 0, 32 * 16)
    gpu.upload(sc)
    p, t = gpu.trace_closest(cr)
    assert np.array_equal(p, cp)
    assert np.array_equal(t.view(np.uint32), ct.view(np.uint32))
    assert np.array_equal(gpu.trace_any(ar), ah)


def test_maps_matter_and_persistent_equals_wavefront(gpu):
    """The maps change the film (the same scene with constants renders
    another), and the persistent kernel sets the maps up like the wavefront:
    bit-identical films."""
    import dataclasses
    from conftest import tuned
    sc, cam, filt, par = scenes.mapped_materials(48, 24, 4)
    gpu.upload(sc)
    with tuned(gpu, render_mode=TR_RENDER_MODE_WAVEFRONT):
        want, _ = gpu.render(cam, filt, par)
    with tuned(gpu, render_mode=TR_RENDER_MODE_PERSISTENT):
        got, st = gpu.render(cam, filt, par)
    assert st.iterations == 1
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    sc.materials = [dataclasses.replace(m, tex_param=(0,) * 13) for m in sc.materials]
    gpu.upload(sc)
    flat, _ = gpu.render(cam, filt, par)
    assert not np.array_equal(flat.view(np.uint32), want.view(np.uint32))
