"""Generates tests/golden/*.npz from the REFERENCE's own sources.

Run in a checkout where the reference exists (make -C oracle ref builds it):
    python tests/golden/make_golden.py
Each fixture stores its inputs (scene arrays, rays, camera, parameters) and
the reference's outputs, so checking it needs neither the reference nor the
random generator that made the inputs.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tracer_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def units():
    rng = np.random.default_rng(100)
    a = rng.normal(size=(512, 3)).astype(np.float32)
    b = rng.normal(size=(512, 3)).astype(np.float32)
    a[:16] *= np.float32(1e-20)
    a[16:32] *= np.float32(1e15)
    a[32:40] = [[0, 0, 1], [0, 1, 0], [1, 0, 0], [0, 0, -1], [1e-30, 0, 0], [3, 4, 0], [-0.0, 0.0, 1.0], [1, 1, 1]]
    seeds = np.array([0, 1, 7, 12345, -3, 2**31 - 1], np.int64)
    pcg = np.stack([oracle.pcg_uniform("reference", int(s), 64) for s in seeds])
    return dict(a=a, b=b, cross=oracle.unit("reference", "cross", a, b, out_shape=(512, 3), n=512),
                normalize=oracle.unit("reference", "normalize", a, out_shape=(512, 3), n=512),
                seeds=seeds, pcg=pcg)


def traversal():
    sc = scenes.traversal(4096, seed=3)
    ref = oracle.Oracle(sc, "reference", threads=8)
    rays = scenes.traversal_rays(2048, seed=3)
    srays = scenes.traversal_rays(2048, seed=3, shadow=True)
    prim, t = ref.trace_closest(rays)
    hit = ref.trace_any(srays)
    nodes, order = ref.bvh()
    d = scenes.pack_scene(sc)
    d.update(rays=rays.view(np.uint8), shadow_rays=srays.view(np.uint8), prim=prim, t=t, hit=hit,
             nodes=nodes.view(np.uint8), order=order)
    return d


def mixed():
    sc = scenes.random_scene(21, n_tris=80, n_spheres=10, n_lights=2)
    cam = scenes.random_camera(40, 32, 21)
    par = scenes.make_params(40, 32, 4, 1, 6, seed_base=5)
    filt = scenes.make_filter(0.5, 0.6)
    ref = oracle.Oracle(sc, "reference", threads=8)
    ref.set_camera(cam, filt)
    rng = np.random.default_rng(22)
    o = rng.uniform(-2, 2, (2048, 3)).astype(np.float32)
    dd = rng.normal(size=(2048, 3)).astype(np.float32)
    rays = scenes.make_rays(o, dd, 0.0, scenes.F32_MAX)
    prim, t = ref.trace_closest(rays)
    nodes, order = ref.bvh()
    d = scenes.pack_scene(sc)
    d.update(scenes.pack_view(cam, filt, par))
    d.update(rays=rays.view(np.uint8), prim=prim, t=t, nodes=nodes.view(np.uint8), order=order,
             rgbw=ref.render(par))
    return d


def render(name, maker):
    sc, cam, filt, par = maker()
    ref = oracle.Oracle(sc, "reference", threads=8)
    ref.set_camera(cam, filt)
    d = scenes.pack_scene(sc)
    d.update(scenes.pack_view(cam, filt, par))
    d["rgbw"] = ref.render(par)
    return d


def image_cases():
    """(name, file bytes) of the 8-bit image reader's cases: files from the
    reference's own encoders (stb_image_write's JPEG at three qualities and
    grey, TGA raw and run-length, BMP) and from tests/jpeg_writer.py (the JPEG
    layouts those encoders never write: 4:2:2, 4:4:0, 4:1:1, mixed sampling,
    restart intervals, one scan per component, RGB component ids, grey with
    2x2 sampling, a 3x5 image)."""
    import ctypes as C
    import tempfile
    sys.path.insert(0, os.path.dirname(OUT))
    from jpeg_writer import write_jpeg
    lib = C.CDLL(oracle.REF_SO)
    rng = np.random.default_rng(11)
    yy, xx = np.mgrid[0:45, 0:61]
    img = np.stack([xx * 4, yy * 5, (xx * yy) % 256], -1).clip(0, 255).astype(np.uint8)
    img[10:20, 10:30] = (rng.random((10, 20, 3)) * 255).astype(np.uint8)
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, kind, src, q in (("stb_q50.jpg", 0, img, 50), ("stb_q85.jpg", 0, img, 85), ("stb_q95.jpg", 0, img, 95),
                                   ("stb_grey.jpg", 0, img[..., :1], 80), ("stb_rle.tga", 1, img, 1),
                                   ("stb_raw_rgba.tga", 1, np.dstack([img, img[..., :1]]), 0),
                                   ("stb_grey.tga", 1, img[..., 1:2], 1), ("stb.bmp", 2, img, 0),
                                   ("stb_rgba.bmp", 2, np.dstack([img, img[..., :1]]), 0)):
            p = os.path.join(tmp, name)
            src = np.ascontiguousarray(src)
            h, w, c = src.shape
            assert lib.ref_write_image(p.encode(), kind, w, h, c, src.ctypes.data_as(C.c_void_p), q) == 1
            cases.append((name, open(p, "rb").read()))
    for name, kw, src in (("w_422.jpg", dict(sampling=((2, 1), (1, 1), (1, 1))), img),
                          ("w_440.jpg", dict(sampling=((1, 2), (1, 1), (1, 1))), img),
                          ("w_411.jpg", dict(sampling=((4, 1), (1, 1), (1, 1))), img),
                          ("w_mixed.jpg", dict(sampling=((2, 2), (2, 1), (1, 2))), img),
                          ("w_restart.jpg", dict(restart=3), img),
                          ("w_scans_422_restart.jpg", dict(sampling=((2, 1), (1, 1), (1, 1)), interleaved=False,
                                                           restart=5), img),
                          ("w_rgb_ids.jpg", dict(sampling=((1, 1), (1, 1), (1, 1)), ids=(82, 71, 66)), img),
                          ("w_grey_22.jpg", dict(sampling=((2, 2),)), img[..., 1]),
                          ("w_tiny.jpg", dict(), img[:3, :5])):
        cases.append((name, write_jpeg(src, **kw)))
    return cases


def image_files():
    """The reader's cases with the reference's decodes (load_image_from_file)."""
    import ctypes as C
    import tempfile
    lib = C.CDLL(oracle.REF_SO)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for k, (name, data) in enumerate(image_cases()):
            p = os.path.join(tmp, name)
            open(p, "wb").write(data)
            w, h = C.c_int(), C.c_int()
            assert lib.ref_load_image(p.encode(), C.byref(w), C.byref(h), None) == 0, name
            px = np.zeros((h.value, w.value, 3), np.uint8)
            lib.ref_load_image(p.encode(), C.byref(w), C.byref(h), px.ctypes.data_as(C.c_void_p))
            out[f"name{k}"] = np.array(name)
            out[f"file{k}"] = np.frombuffer(data, np.uint8)
            out[f"rgb{k}"] = px
    return out


def mapped():
    """Image maps on glass, metal, Disney 2015 and Disney12 arguments."""
    return render("mapped", lambda: scenes.mapped_materials(32, 16, 2))


def main():
    if not oracle.ref_available():
        oracle.build_ref()
    np.savez_compressed(os.path.join(OUT, "units.npz"), **units())
    np.savez_compressed(os.path.join(OUT, "traversal_4k.npz"), **traversal())
    np.savez_compressed(os.path.join(OUT, "mixed_scene.npz"), **mixed())
    np.savez_compressed(os.path.join(OUT, "cornell_32x32_4spp.npz"),
                        **render("cornell", lambda: scenes.cornell(32, 32, 4)))
    np.savez_compressed(os.path.join(OUT, "disney_grid_32x32_2spp.npz"),
                        **render("disney", lambda: scenes.disney_grid(32, 32, 2, min_depth=3)))
    # the rows beyond the configured scenes: glass and metal, Disney 2015, the
    # environment light (HDR and 8-bit maps) and Phong image maps
    np.savez_compressed(os.path.join(OUT, "cornell_glass_metal_24x24_2spp.npz"),
                        **render("glass_metal", lambda: scenes.cornell(24, 24, 2, max_depth=8, min_depth=2,
                                                                        glass=True, metal=True)))
    np.savez_compressed(os.path.join(OUT, "disney15_row_32x16_2spp.npz"),
                        **render("disney15", lambda: scenes.disney15_row(32, 16, 2, env=False)))
    np.savez_compressed(os.path.join(OUT, "outdoor_env_24x16_2spp.npz"),
                        **render("outdoor", lambda: scenes.outdoor(24, 16, 2, env_size=(32, 16))))
    np.savez_compressed(os.path.join(OUT, "outdoor_env8_textured_24x16_2spp.npz"),
                        **render("outdoor8", lambda: scenes.outdoor(24, 16, 2, env_size=(32, 16), env_8bit=True,
                                                                     textured=True, glass=False)))
    np.savez_compressed(os.path.join(OUT, "cornell_textured_24x24_2spp.npz"),
                        **render("textured", lambda: scenes.cornell(24, 24, 2, textured=True)))
    np.savez_compressed(os.path.join(OUT, "mapped_materials_32x16_2spp.npz"), **mapped())
    np.savez_compressed(os.path.join(OUT, "image_files.npz"), **image_files())
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
