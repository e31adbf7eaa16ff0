"""CPU-baseline record -- TEST INFRASTRUCTURE ONLY.

Times the reference path tracer on the host cores, next to the oracle port,
on the configured scenes:

* ``stock``: the reference's own create_pt_renderer(PTRendererParams{
  worker_count, task_tile_size = 16, spp, min_depth, max_depth,
  direct_light_sample_num = 1}) -> Renderer::render (src/factory/renderer.hpp:12-21,
  src/renderer/pixel_sampler_renderer.cpp:24-109), built from the reference's
  sources by ``make -C oracle ref`` (-O2 -DNDEBUG -ffp-contract=off) and
  ``make -C oracle ref-O0`` (the as-shipped -O0: the reference's CMake build
  sets no build type). Timed inside the harness around render() only (no
  BVH build), std::chrono::steady_clock.
* ``port``: the oracle restatement (oracle/tracer_oracle.cpp) rendering the
  same film with per-pixel pcg32 seeds (the GPU's seeding), all frame rows
  spread over the threads.

Each figure is the median of three runs, in camera samples per second, at
all host threads and at one thread. Films are smaller than the GPU bench's
where a full frame would take minutes on one core; samples per second do not
depend on the film size. Needs the reference checkout (oracle/_ref).

    python -m oracle.cpu_baseline [--quick]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tracer_gb300 import scenes  # noqa: E402


def workloads(quick: bool):
    """(name, scene maker, film W, H, spp for all threads, spp for one thread)."""
    s = 4 if quick else 1
    return [
        ("cornell_256x256_16spp_depth5", lambda: scenes.cornell(256, 256, 16), 256 // s, 256 // s, 16, 4),
        ("disney_grid_16x16_spheres_64spp_depth8", lambda: scenes.disney_grid(1024, 1024, 64), 256 // s, 256 // s,
         16, 2),
        ("occluded_room_500k_tris_16spp_depth10", lambda: scenes.occluded_room(1024, 768, 16), 128 // s, 96 // s,
         16, 2),
    ]


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def median_rate(fn, samples: int, runs: int = 3) -> float:
    ts = []
    for _ in range(runs):
        ts.append(fn())
    return samples / statistics.median(ts) / 1e6


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="quarter-size films (a check that it runs)")
    args = ap.parse_args()
    if not oracle.ref_available():
        oracle.build_ref()
    if not os.path.exists(oracle.REF_SO_O0):
        import subprocess
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref-O0", f"REF_ROOT={oracle.REF_ROOT}"], check=True)
    threads = os.cpu_count() or 1
    rows = []
    for name, make, W, H, spp_all, spp_one in workloads(args.quick):
        sc, cam, filt, _ = make()
        cam.film_aspect = W / H
        kinds = {k: oracle.Oracle(sc, k) for k in ("reference", "reference-O0", "port")}
        for o in kinds.values():
            o.set_camera(cam, filt)
        row = {"workload": name, "film": f"{W}x{H}", "primitives": int(len(sc.prim_shape))}
        for nthreads, spp in ((threads, spp_all), (1, spp_one)):
            par = scenes.make_params(W, H, spp, _.min_depth, _.max_depth)
            n = W * H * spp
            for kind in ("reference", "reference-O0"):
                o = kinds[kind]
                row[f"stock_{'O2' if kind == 'reference' else 'O0'}_{nthreads}t"] = round(
                    median_rate(lambda: o.render_stock_seconds(par, nthreads), n), 4)
            port = kinds["port"]
            port.threads = nthreads

            def run_port():
                t0 = time.perf_counter()
                port.render(par)
                return time.perf_counter() - t0
            row[f"port_{nthreads}t"] = round(median_rate(run_port, n), 4)
            row[f"spp_{nthreads}t"] = spp
        rows.append(row)
        print(json.dumps(row), flush=True)
    print(json.dumps({"cpu": cpu_model(), "threads": threads, "machine": platform.machine(), "rows": rows}))


if __name__ == "__main__":
    main()
