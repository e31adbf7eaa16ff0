"""Benchmark of the GPU path tracer (plain unidirectional path tracing).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload disney_grid|cornell]

A step renders one full frame of the workload: by default the 16x16
Disney12-sphere grid at 1024x1024, 64 spp, max depth 8 (67,108,864 camera
samples), all geometry and path state resident on the device. `value` is
camera samples per second over exactly K steps (CUDA events on the
renderer's stream, synchronised on both sides, maximum over ranks); `e2e`
repeats the measurement through the C ABI's host-buffer entry point
(tr_render), which copies the film back every step.

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement in oracle/ (the reference's own build needs its source
checkout, which this machine may not have), all host threads, a bounded
sample of the same frame per step.

Multiple GPUs (torchrun, one rank per GPU) render independent replicas:
per-GPU work is fixed, so scaling is weak and there is no collective on the
data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from tracer_gb300 import scenes  # noqa: E402
from tracer_gb300.abi import TR_RENDER_TIME_STAGES  # noqa: E402

METRIC = "Msamples/s (plain GPU path tracing)"
UNIT = "Msamples/s"

# Bytes each stage must move per work item through HBM (the SoA path state,
# queues and shadow records of render.cu; scene data is read-only and stays in
# cache): the roofline numerator. nl = number of lights.
def stage_bytes(stage: str, nl: int) -> int:
    if stage == "shade":
        # reads: P0-P3 64, rng 8, hit 16, P4 16, shadow contributions 16*nl, MIS hit+state 64
        # writes: P0-P4 80, rng 8, MIS state 48, shadow records 48*nl, queue entries 4*(3+nl)
        return 168 + 16 * nl + 148 + 52 * nl
    if stage == "extend":
        return 4 + 32 + 16  # queue entry, ray, hit record
    return 4 + 32 + 4  # shadow: queue entry, ray record, occlusion flag


def workload(name: str):
    if name == "cornell":
        sc, cam, filt, par = scenes.cornell(256, 256, 16)
        label = "cornell_box_36tris_256x256_16spp_depth5"
    else:
        sc, cam, filt, par = scenes.disney_grid(1024, 1024, 64, max_depth=8, min_depth=5)
        label = "disney12_sphere_grid_16x16_1024x1024_64spp_depth8"
    return label, sc, cam, filt, par


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def usable_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(sc, cam, filt, par, seconds_target=1.0, max_rows=64):
    """Reference algorithm (oracle port) on the host cores over spread rows of
    the same frame; returns (Msamples/s, threads, description)."""
    import oracle
    threads = usable_cores()
    orc = oracle.Oracle(sc, "port", threads=threads)
    orc.set_camera(cam, filt)
    H = par.height
    nrows = max(threads, 1)
    best = None
    while True:
        rows = np.linspace(0, H - 1, nrows).round().astype(np.int32)
        t0 = time.perf_counter()
        _, n = orc.render_rows(par, rows)
        dt = time.perf_counter() - t0
        best = (n / dt / 1e6, n, nrows, dt)
        if dt >= seconds_target or nrows >= max_rows:
            break
        nrows = min(max_rows, nrows * 2)
    rate, n, nrows, dt = best
    desc = (f"{nrows} rows spread evenly over the {par.width}x{par.height} frame at {par.spp} spp "
            f"({n} samples, {dt:.2f} s wall, {dt * threads:.1f} CPU-s), per-pixel pcg32 seeds as on the GPU")
    return rate, threads, desc


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    label, sc, cam, filt, par = workload(args.workload)
    import oracle
    threads = usable_cores()
    orc = oracle.Oracle(sc, "port", threads=threads)
    orc.set_camera(cam, filt)
    nrows = 2 * threads
    rows = np.linspace(0, par.height - 1, nrows).round().astype(np.int32)
    for _ in range(args.warmup):
        orc.render_rows(par, rows[:threads])
    t0 = time.perf_counter()
    total = 0
    for k in range(args.steps):
        r = (rows + k) % par.height
        _, n = orc.render_rows(par, r)
        total += n
    dt = time.perf_counter() - t0
    value = total / dt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)",
            "config": {"workload": label, "width": par.width, "height": par.height, "spp": par.spp,
                       "max_depth": par.max_depth, "min_depth": par.min_depth},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{nrows} rows spread over the frame per step at {par.spp} spp, "
                                       "CPU restatement of the reference (oracle/tracer_oracle.cpp)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    from tracer_gb300.native import GpuContext

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    label, sc, cam, filt, par = workload(args.workload)
    ctx = GpuContext(local)
    ctx.upload(sc)
    nl = len(sc.light_prims)
    W, H = par.width, par.height
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    film = torch.empty((H, W, 4), dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")  # 256 MiB > L2

    def barrier():
        ctx.synchronize()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    par.flags = TR_RENDER_TIME_STAGES  # also in warm-up: allocates the timing events
    for _ in range(args.warmup):
        ctx.render_dev(cam, filt, par, film.data_ptr())
    stats = []
    barrier()
    with ClockSampler(local) as clocks:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            if k:
                with torch.cuda.stream(stream):
                    flush.zero_()
            stats.append(ctx.render_dev(cam, filt, par, film.data_ptr()))
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    samples = sum(s.samples for s in stats)
    value = world * samples / (ms / 1e3) / 1e6

    # end to end through the host-buffer C ABI call (film copied back each step)
    par.flags = 0
    host_film = np.zeros((H, W, 4), np.float32)
    barrier()
    t0 = time.perf_counter()
    e2e_samples = 0
    for _ in range(args.steps):
        out, st = ctx.render(cam, filt, par)
        e2e_samples += st.samples
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = world * e2e_samples / e2e_s / 1e6
    del host_film

    if rank != 0:
        ctx.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # roofline of the dominant stage, from the timed steps' own CUDA events
    names = ["extend", "shade", "shadow"]
    stage_ms = [sum(s.stage_ms[i] for s in stats) for i in range(3)]
    items = [sum(s.extend_rays for s in stats), sum(s.shade_items for s in stats),
             sum(s.shadow_rays for s in stats)]
    launches = sum(s.iterations for s in stats)
    dom = int(np.argmax(stage_ms))
    per_launch_bytes = stage_bytes(names[dom], nl) * items[dom] / max(launches, 1)
    per_launch_s = stage_ms[dom] / 1e3 / max(launches, 1)
    achieved = per_launch_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()
    cpu_rate, cpu_threads, cpu_desc = (None, None, None)
    if not args.no_cpu_baseline and world == 1:
        cpu_rate, cpu_threads, cpu_desc = cpu_sample(sc, cam, filt, par)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene, no dataset)",
        "config": {"workload": label, "width": W, "height": H, "spp": par.spp, "max_depth": par.max_depth,
                   "min_depth": par.min_depth, "lights": nl, "primitives": int(len(sc.prim_shape)),
                   "parallelism": f"replicas x{world}",
                   "l2": "path state and queues (~450 MB at 1024x1024) exceed L2; 256 MiB buffer "
                         "written between timed steps"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 100, "d2h_bytes_per_step": W * H * 16},
        "gpu_launches": int(sum(1 + 3 * s.iterations for s in stats)),
        "roofline": {"bound": "hbm", "kernel": "k_" + names[dom], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "bytes_per_item": stage_bytes(names[dom], nl),
                     "stage_ms": dict(zip(names, stage_ms)), "stage_items": dict(zip(names, items))},
        "rays": {"extend": items[0], "shadow": items[2],
                 "mrays_per_s": (items[0] + items[2]) / (ms / 1e3) / 1e6},
        "clocks": clocks.summary(),
    }
    if cpu_rate is not None:
        line["cpu_baseline"] = {"value": cpu_rate, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                                "sample": cpu_desc}
    print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["disney_grid", "cornell"], default="disney_grid")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
