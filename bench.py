"""Benchmark of the GPU path tracer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload occluded_room|disney_grid|cornell] [--size WxHxSPP]
                    [--no-convergence] [--no-cpu-baseline]

A step renders one full frame of the workload. The default is the
occluded-light room: 500k triangles of Disney12 furniture in a closed
Lambertian room lit only through a 0.1 m slit by a 12-triangle emissive
cube, at 1024x768, 16 spp, max depth 10 (12,582,912 camera samples per
step), all geometry and path state resident on the device. `value` is
camera samples per second over exactly K steps (CUDA events on the
renderer's stream, synchronised on both sides, maximum over ranks); `e2e`
repeats the measurement through the C ABI's host-buffer entry point
(tr_render), which copies the film back every step. `convergence` times the
plain and the guided path tracer to 1% relMSE against a 4096-spp FP64
reference of the same scene at 1024x768.

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement in oracle/ (bit-exact with the reference's own build,
which needs the reference checkout this machine may not have), all host
threads, a bounded sample of the same frame per step.

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
from tracer_gb300.abi import (STAGE_NAMES, TR_RENDER_COUNT_VISITS, TR_RENDER_TIME_STAGES,  # noqa: E402
                              TrCamera, TrFilter, TrRenderParams)
import ctypes  # noqa: E402

METRIC = "Msamples/s and time-to-1% relMSE, guided vs plain GPU PT on 1 GB300"
UNIT = "Msamples/s"

# Algorithmic bytes per work item of each kernel (the roofline numerator).
# Traversal kernels (per ray): 32 B per box tested (the reference's
# LinearBVHNode) + 48 B per primitive tested (3 indices + 3 vertices) + the
# 32-B ray + its result (8 B: prim id and t; 1 B for an occlusion flag).
# Shading kernels (per item): the path-state words each one reads and writes
# (float4 SoA records and queue entries of render.cu); scene tables are
# read-only and cache-resident.
def kernel_bytes(stage: str, nl: int, boxes_per_ray=0.0, prims_per_ray=0.0) -> float:
    if stage == "extend":
        return 32 * boxes_per_ray + 48 * prims_per_ray + 32 + 8
    if stage == "shadow":
        return 32 * boxes_per_ray + 48 * prims_per_ray + 32 + 1
    if stage == "logic":
        # queue 4, P0 16, P3 16, HC 16, P4 16, shadow contributions 16*nl, MIS (HM, M0-M2) 64,
        # writes P3 16 + queue 4; finishing samples also write the film (16) and P0-P4 (80)
        return 4 + 16 + 16 + 16 + 16 + 16 * nl + 64 + 16 + 4
    if stage.startswith("material"):
        # queue 4, rng 8 r/w, P0-P2 48, HC 16, P3 16; writes NU 8*nl + queue 4*nl, SC 112,
        # M0-M2 48 + queue 4, P4 16, P0-P2 48, queue 8
        return 4 + 16 + 48 + 16 + 16 + 12 * nl + 112 + 52 + 16 + 48 + 8
    if stage.startswith("nee"):
        # queue 4, SC 112, NU 8, P4 16; writes shadow record 48 + queue 4
        return 4 + 112 + 8 + 16 + 48 + 4
    return 0.0


KERNEL_NAMES = {"extend": "k_extend", "logic": "k_logic", "material_phong": "k_material<0>",
                "material_disney": "k_material<1>", "nee_phong": "k_nee<0>", "nee_disney": "k_nee<1>",
                "shadow": "k_shadow", "bin": "k_bin_count + k_bin_scan + k_bin_scatter"}


def dram_bound(traffic_per_launch: float, launch_ms: float, peak_gbs: float) -> dict:
    """What bounds a kernel, from its measured DRAM bytes per launch: the
    DRAM bandwidth those bytes take over the launch's duration, as a fraction
    of the HBM peak. The tree walks read a few percent of HBM bandwidth (L1
    and L2 serve most node and triangle reads) and stall on dependent loads:
    they are latency-bound, and the algorithmic fraction beside it says how
    many bytes the walk touches, not what limits it."""
    gbs = traffic_per_launch / (launch_ms / 1e3) / 1e9
    frac = gbs / peak_gbs
    return {"bound": "hbm" if frac >= 0.5 else "latency", "dram_gbs": gbs, "dram_frac": frac,
            "frac_is": "algorithmic bytes / launch time / HBM peak; dram_frac: measured DRAM bytes / launch "
                       "time / HBM peak"}


def traffic_per_unit(stage: str):
    """DRAM bytes per work item of a kernel from a committed ncu summary, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            return json.load(f).get(stage)
    except (OSError, ValueError):
        return None


WORKLOADS = ("occluded_room", "disney_grid", "cornell", "batch64", "traversal")


def workload(name: str, size: str | None = None):
    """(label, scene, camera, filter, params); size "WxHxSPP" overrides the
    film and sample count (small cases for profiler captures)."""
    W, H, S = {"cornell": (256, 256, 16), "disney_grid": (1024, 1024, 64), "occluded_room": (1024, 768, 16)}[name]
    if size:
        W, H, S = (int(v) for v in size.lower().split("x"))
    if name == "cornell":
        sc, cam, filt, par = scenes.cornell(W, H, S)
        label = f"cornell_box_36tris_{W}x{H}_{S}spp_depth5"
    elif name == "disney_grid":
        sc, cam, filt, par = scenes.disney_grid(W, H, S, max_depth=8, min_depth=5)
        label = f"disney12_sphere_grid_16x16_{W}x{H}_{S}spp_depth8"
    else:
        sc, cam, filt, par = scenes.occluded_room(W, H, S, max_depth=10, min_depth=3)
        label = f"occluded_light_room_500k_tris_12_lights_{W}x{H}_{S}spp_depth10"
    return label, sc, cam, filt, par


def rel_mse(img: np.ndarray, ref: np.ndarray) -> float:
    """mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2)."""
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def _image(acc: np.ndarray) -> np.ndarray:
    w = acc[..., 3:4]
    return np.where(w > 0, acc[..., :3] / np.where(w > 0, w, 1.0), 0.0)


GUIDE_BOX = {"occluded_room": ((-4.0, 0.0, -3.0), (4.0, 4.0, 3.0))}


def convergence(ctx, name: str, size=(1024, 768), ref_spp=4096, pass_spp=8, max_spp=768, target=0.01,
                alpha=0.25, train_steps=24, warm_steps=200, batch=65536, lr=1e-3, record_every=8,
                light_grid=(32, 16, 24), light_bins=8, light_share=0.2):
    """Time for the plain and the guided GPU path tracer to reach `target`
    relMSE against a converged reference of the same scene. The reference
    is ref_spp samples per pixel accumulated in double. Each run adds
    passes of pass_spp samples with fresh per-pixel seeds, accumulated in
    double on the host, until the target or max_spp. The guided run starts
    from an untrained network: its first pass renders plainly (alpha 0) and
    records training data, every later pass samples Lambertian
    continuations from the network's mixture with probability `alpha` and
    traces a ray from the mixture alone for their direct light; every pass
    records the paths of one sample in `record_every` per pixel and is
    followed by `train_steps` Adam steps on `batch` random records
    (`warm_steps` more after the first pass; online training is inside the
    timed region). If a training
    loss is not finite the network is re-initialised and the next pass
    renders plainly (the plain path is the fallback). The guided run also
    learns its light samples: every pass draws each area light's point from
    the light table (`light_grid` cells over the guide box, `light_bins`^2
    cells of the light's sample square, `light_share` of the uniform density
    mixed in) and records its unoccluded light samples, and the table is
    rebuilt from all passes so far after each pass."""
    from tracer_gb300.abi import make_guide
    W, H = size
    _, sc, cam, filt, par = workload(name, f"{W}x{H}x{pass_spp}")
    ctx.upload(sc)
    ref_par = scenes.make_params(W, H, ref_spp, par.min_depth, par.max_depth, seed_base=1 << 30)
    t0 = time.perf_counter()
    ref_acc, _ = ctx.render(cam, filt, ref_par, fp64=True)
    ref_s = time.perf_counter() - t0
    ref = _image(ref_acc)
    box = GUIDE_BOX.get(name)

    def run(guided: bool):
        import torch
        film = torch.zeros((H, W, 4), dtype=torch.float64, device=f"cuda:{torch.cuda.current_device()}")
        acc = np.zeros((H, W, 4), np.float64)
        spent, curve, reached, losses = 0.0, [], None, []
        train_s = light_s = render_s = 0.0
        use_alpha = 0.0
        if guided:
            ctx.guide_init(seed=0)
            ctx.guide_light_init(light_grid, light_bins)
        for k in range(max_spp // pass_spp):
            p = scenes.make_params(W, H, pass_spp, par.min_depth, par.max_depth, seed_base=1 + k * W * H)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if guided:
                ctx.render_guided_dev(cam, filt, p, make_guide(use_alpha, *box, record=record_every,
                                                               light_guide=True, light_record=True),
                                      film.data_ptr(), fp64=True)
                t1 = time.perf_counter()
                render_s += t1 - t0
                ctx.guide_light_update(light_share)
                light_s += time.perf_counter() - t1
                t1 = time.perf_counter()
                loss = ctx.guide_train_on_records(train_steps + (warm_steps if k == 0 else 0), batch, lr, seed=k)
                train_s += time.perf_counter() - t1
                if np.isfinite(loss):
                    use_alpha = alpha
                else:
                    ctx.guide_init(seed=k + 1)
                    use_alpha = 0.0
                losses.append(round(float(loss), 4))
                out = film.cpu().numpy()
            else:
                out, _ = ctx.render(cam, filt, p, fp64=True)
            spent += time.perf_counter() - t0
            acc += out
            spp = (k + 1) * pass_spp
            e = rel_mse(_image(acc), ref)
            if spp & (spp - 1) == 0 or e <= target:
                curve.append([spp, round(spent, 4), round(e, 5)])
            if e <= target:
                reached = (spp, spent)
                break
        res = {"time_to_target_s": reached[1] if reached else None,
               "spp_at_target": reached[0] if reached else None,
               "relmse_curve_spp_s_relmse": curve}
        if guided:
            res.update({"alpha": alpha, "train_steps_per_pass": train_steps, "warm_steps": warm_steps, "batch": batch,
                        "lr": lr, "record_every": record_every, "train_s": round(train_s, 4),
                        "render_s": round(render_s, 4), "light_update_s": round(light_s, 4),
                        "light_table": {"grid": list(light_grid), "bins": light_bins, "uniform_share": light_share},
                        "mean_loss_per_pass": losses[:8] + (["..."] if len(losses) > 9 else []) + losses[-1:]})
        return res

    res = {"resolution": f"{W}x{H}", "reference_spp": ref_spp, "reference_s": round(ref_s, 2),
           "pass_spp": pass_spp, "target_relmse": target,
           "relmse": "mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2)",
           "plain": run(False), "guided": run(True) if box else None}
    pt, gt = res["plain"]["time_to_target_s"], (res["guided"] or {}).get("time_to_target_s")
    res["guided_over_plain_time"] = (gt / pt) if (pt and gt) else None
    return res


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
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0:  # NVML up
                time.sleep(0.05)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark(self) -> int:
        """Index of the next sample (bracket a region with two marks)."""
        return len(self.lines)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, lo: int = 0, hi: int | None = None):
        if hi is not None and hi - lo < 2:
            # a timed region shorter than the sampling period: the samples
            # next to it (warm-up and the work right after)
            lo, hi = max(0, lo - 3), hi + 3
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[lo:hi]:
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


def ranks():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init_ranks(world: int):
    """One process group per job of more than one rank: NCCL on GPUs, gloo
    otherwise (the replicas exchange only timings, never data)."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
    return dist


def max_over_ranks(value: float, dist, device) -> float:
    """The largest value over all ranks (the slowest replica's time)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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
    import oracle
    threads = usable_cores()
    if args.workload == "batch64":
        # rows of the batch's first four jobs, one job per step in turn
        label = "batch_64_scenes_10k_2M_tris_mixed_res_spp_depth6"
        items = scenes.batch(4)
        orcs = []
        for sc, cam, filt, par in items:
            o = oracle.Oracle(sc, "port", threads=threads)
            o.set_camera(cam, filt)
            orcs.append((o, par))
        nrows = 2 * threads
        for _ in range(args.warmup):
            orcs[0][0].render_rows(orcs[0][1], np.arange(threads, dtype=np.int32) % orcs[0][1].height)
        t0 = time.perf_counter()
        total = 0
        for k in range(args.steps):
            o, par = orcs[k % len(orcs)]
            rows = np.linspace(0, par.height - 1, nrows).round().astype(np.int32)
            total += o.render_rows(par, rows)[1]
        dt = time.perf_counter() - t0
        value = total / dt / 1e6
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded procedural scenes)", "config": batch_config(args.gpus),
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"{nrows} rows per step of one of the batch's first four jobs in turn, "
                                           "CPU restatement of the reference (oracle/tracer_oracle.cpp)"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "traversal":
        label = "traversal_1M_tris_leaf4_4M_closest_4M_shadow_rays"
        sc = scenes.traversal(1 << 20)
        orc = oracle.Oracle(sc, "port", threads=threads)
        m = 1 << 17
        closest = scenes.traversal_rays(1 << 22, shadow=False)
        shadow = scenes.traversal_rays(1 << 22, shadow=True)
        for _ in range(args.warmup):
            orc.trace_closest(closest[:m // 4])
        t0 = time.perf_counter()
        for k in range(args.steps):
            sl = slice((k * m) % (1 << 22), (k * m) % (1 << 22) + m)
            orc.trace_closest(closest[sl])
            orc.trace_any(shadow[sl])
        dt = time.perf_counter() - t0
        value = 2 * m * args.steps / dt / 1e6
        line = {"impl": "reference", "metric": "Mrays/s (BVH traversal: closest hit + shadow any hit)",
                "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * dt / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random triangles and rays)",
                "config": traversal_config(args.gpus),
                "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                                 "sample": f"{m} closest-hit and {m} shadow rays per step, CPU restatement of "
                                           "BVHAccel::intersect_p / intersect (oracle/tracer_oracle.cpp)"},
                "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    label, sc, cam, filt, par = workload(args.workload, args.size)
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
            "config": frame_config(label, sc, par, args.gpus),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{nrows} rows spread over the frame per step at {par.spp} spp, "
                                       "CPU restatement of the reference (oracle/tracer_oracle.cpp)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """The batched-rendering workload: 64 scenes (10k-2M triangles each,
    log-uniform) at mixed resolutions and spp rendered as one batch per step
    after the launch autotuner has picked the tuning on a 1-spp probe."""
    import torch
    from tracer_gb300.abi import TR_RENDER_TIME_STAGES as TS
    from tracer_gb300.native import GpuContext
    rank, world, local = ranks()
    dist = init_ranks(world)
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    items = scenes.batch(64)
    gen_s = time.perf_counter() - t0
    ctx = GpuContext(local)
    t0 = time.perf_counter()
    ctx.upload_set([it[0] for it in items])
    upload_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    films = [torch.zeros((p.height, p.width, 4), device=f"cuda:{local}") for _, _, _, p in items]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()
    jobs = [(k, it[1], it[2], it[3], films[k].data_ptr()) for k, it in enumerate(items)]
    t0 = time.perf_counter()
    tuning, probe_ms = ctx.autotune(jobs, probe_spp=1)
    tune_s = time.perf_counter() - t0

    def barrier():
        ctx.synchronize()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        ctx.render_batch_dev(jobs)
    barrier()
    c0 = clocks.mark()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = []
    for k in range(args.steps):
        if k:
            with torch.cuda.stream(stream):
                flush.zero_()
        stats.append(ctx.render_batch_dev(jobs))
    e1.record(stream)
    barrier()
    c1 = clocks.mark()
    clocks.__exit__()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, dist, f"cuda:{local}")
    samples = sum(s.samples for s in stats)
    value = world * samples / (ms / 1e3) / 1e6
    # end to end: the batch call plus every film copied back to the host
    barrier()
    t0 = time.perf_counter()
    e2e_samples = 0
    for _ in range(args.steps):
        st = ctx.render_batch_dev(jobs)
        host = [f.cpu() for f in films]
        e2e_samples += st.samples
    barrier()
    e2e = world * e2e_samples / (time.perf_counter() - t0) / 1e6
    d2h = sum(int(f.numel()) * 4 for f in films)
    del host
    # the execution model the autotuner did not keep, timed the same way
    # (outside the headline): the whole batch as one launch of the persistent
    # kernel, or as the wavefront
    from tracer_gb300.abi import TR_RENDER_MODE_PERSISTENT, TR_RENDER_MODE_WAVEFRONT
    kept_mode = tuning.render_mode
    other = TR_RENDER_MODE_WAVEFRONT if kept_mode == TR_RENDER_MODE_PERSISTENT else TR_RENDER_MODE_PERSISTENT
    ctx.set_tuning(render_mode=other)
    ctx.render_batch_dev(jobs)
    barrier()
    t0 = time.perf_counter()
    other_samples = sum(ctx.render_batch_dev(jobs).samples for _ in range(args.steps))
    barrier()
    other_rate = other_samples / (time.perf_counter() - t0) / 1e6
    ctx.set_tuning(render_mode=kept_mode)
    staged_jobs = [(k, c, f, _flagged(p, TS), film) for k, c, f, p, film in jobs]
    ctx.render_batch_dev(staged_jobs)
    staged = ctx.render_batch_dev(staged_jobs)
    if rank != 0:
        ctx.close()
        return 0
    stage_ms = dict(zip(STAGE_NAMES, staged.stage_ms))
    dom = max((k for k in STAGE_NAMES if k not in ("reset", "bin")), key=lambda k: stage_ms[k])
    tris = int(sum(len(it[0].indices) for it in items))
    # the same set with the device BVH builder (outside the timed region):
    # upload time and rendering rate over its trees
    ctx.set_bvh_builder(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.upload_set([it[0] for it in items])
    torch.cuda.synchronize()
    dev_upload_s = time.perf_counter() - t0
    _, dev_depth = ctx.bvh_stats()
    ctx.render_batch_dev(jobs)
    barrier()
    t0 = time.perf_counter()
    dev_samples = sum(ctx.render_batch_dev(jobs).samples for _ in range(args.steps))
    barrier()
    dev_rate = dev_samples / (time.perf_counter() - t0) / 1e6
    ctx.set_bvh_builder(False)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (64 seeded procedural scenes, no dataset)",
        "config": batch_config(world),
        "workload_detail": {"triangles": tris, "samples_per_step": int(stats[0].samples)},
        "value_is": "camera samples per second over the whole batch (one tr_render_batch_dev call per step)",
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 64 * 200, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(sum(launches_of(s) for s in stats)),
        "render_mode": "persistent kernel (the whole batch in one launch)" if kept_mode == TR_RENDER_MODE_PERSISTENT
        else "wavefront",
        "other_render_mode": {"mode": "persistent kernel (the whole batch in one launch)"
                              if other == TR_RENDER_MODE_PERSISTENT else "wavefront",
                              "msamples_per_s": round(other_rate, 1),
                              "note": "host-timed batch calls, not the headline"},
        "autotune": {"render_mode": tuning.render_mode,
                     "trav_refill_lanes": tuning.trav_refill_lanes, "trav_blocks_per_sm": tuning.trav_blocks_per_sm,
                     "shade_blocks_per_sm": tuning.shade_blocks_per_sm, "graph_iterations": tuning.graph_iterations,
                     "any_node_width": tuning.any_node_width, "ray_bin_bits": tuning.ray_bin_bits,
                     "treelet_nodes": tuning.treelet_nodes, "occluder_cache": tuning.occluder_cache,
                     "probe_ms": round(probe_ms, 2),
                     "tune_s": round(tune_s, 1)},
        "setup_s": {"generate": round(gen_s, 1), "upload_and_bvh": round(upload_s, 1)},
        "device_bvh": {"upload_and_bvh_s": round(dev_upload_s, 2), "msamples_per_s": round(dev_rate, 1),
                       "depth": dev_depth,
                       "note": "tr_ctx_set_bvh_builder(TR_BVH_DEVICE): trees built on the GPU (PLOC); "
                               "host-timed render calls; images agree with the reference trees' up to "
                               "equal-distance ties"},
        "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()}, "dominant_kernel": KERNEL_NAMES[dom],
        "clocks": clocks.summary(c0, c1),
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_traversal(args):
    """The traversal kernel test: 1M random triangles (leaf <= 4), 4M
    closest-hit rays and 4M shadow rays per step through tr_trace_*_dev;
    Mrays/s over both."""
    import torch
    from tracer_gb300.abi import RAY_DTYPE
    from tracer_gb300.native import GpuContext
    rank, world, local = ranks()
    dist = init_ranks(world)
    torch.cuda.set_device(local)
    n_tris, n_rays = 1 << 20, 1 << 22
    sc = scenes.traversal(n_tris)
    closest = scenes.traversal_rays(n_rays, shadow=False)
    shadow = scenes.traversal_rays(n_rays, shadow=True)
    ctx = GpuContext(local)
    # random short any-hit rays have no light to walk toward: the reference's
    # near-first order is this workload's faster one (an explicit --tuning wins)
    tuning = apply_tuning(ctx, args.tuning or "any_hit_order=0")
    t0 = time.perf_counter()
    ctx.upload(sc)
    upload_s = time.perf_counter() - t0
    dev = f"cuda:{local}"
    dc = torch.from_numpy(closest.view(np.uint8)).to(dev)
    ds = torch.from_numpy(shadow.view(np.uint8)).to(dev)
    prim = torch.empty(n_rays, dtype=torch.int32, device=dev)
    tout = torch.empty(n_rays, dtype=torch.float32, device=dev)
    hit = torch.empty(n_rays, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    torch.cuda.synchronize()

    def step():
        ctx.trace_closest_dev(dc.data_ptr(), n_rays, prim.data_ptr(), tout.data_ptr())
        ctx.trace_any_dev(ds.data_ptr(), n_rays, hit.data_ptr())

    def barrier():
        ctx.synchronize()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        step()
    barrier()
    c0 = clocks.mark()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ec = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    e0.record(stream)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ec[3 * k].record(stream)
        ctx.trace_closest_dev(dc.data_ptr(), n_rays, prim.data_ptr(), tout.data_ptr())
        ec[3 * k + 1].record(stream)
        ctx.trace_any_dev(ds.data_ptr(), n_rays, hit.data_ptr())
        ec[3 * k + 2].record(stream)
    e1.record(stream)
    barrier()
    c1 = clocks.mark()
    clocks.__exit__()
    ms = e0.elapsed_time(e1)
    closest_ms = sum(ec[3 * k].elapsed_time(ec[3 * k + 1]) for k in range(args.steps)) / args.steps
    any_ms = sum(ec[3 * k + 1].elapsed_time(ec[3 * k + 2]) for k in range(args.steps)) / args.steps
    ms = max_over_ranks(ms, dist, dev)
    value = world * 2 * n_rays * args.steps / (ms / 1e3) / 1e6
    # end to end: the host-buffer calls, rays in and results out every step
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.trace_closest(closest)
        ctx.trace_any(shadow)
    barrier()
    e2e = world * 2 * n_rays * args.steps / (time.perf_counter() - t0) / 1e6
    cb, cp = ctx.trace_count_dev(dc.data_ptr(), n_rays, False)
    ab, ap = ctx.trace_count_dev(ds.data_ptr(), n_rays, True)
    if rank != 0:
        ctx.close()
        return 0
    peak, peak_kind = measured_peak_hbm()
    bytes_c = 32 * cb + 48 * cp + 40 * n_rays
    bytes_a = 32 * ab + 48 * ap + 33 * n_rays
    dom_closest = closest_ms >= any_ms
    ach = (bytes_c / (closest_ms / 1e3) if dom_closest else bytes_a / (any_ms / 1e3)) / 1e9
    cpu_rate, cpu_threads, cpu_desc = None, None, None
    if not args.no_cpu_baseline and world == 1:
        import oracle
        cpu_threads = usable_cores()
        orc = oracle.Oracle(sc, "port", threads=cpu_threads)
        m = 1 << 18
        t0 = time.perf_counter()
        orc.trace_closest(closest[:m])
        orc.trace_any(shadow[:m])
        dt = time.perf_counter() - t0
        cpu_rate = 2 * m / dt / 1e6
        cpu_desc = f"the first {m} closest-hit and {m} shadow rays ({dt:.2f} s wall), CPU restatement of BVHAccel"
    line = {
        "metric": "Mrays/s (BVH traversal: closest hit + shadow any hit)", "value": value, "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded random triangles and rays, no dataset)",
        "config": traversal_config(world),
        "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 2 * 32 * n_rays,
                "d2h_bytes_per_step": n_rays * 8 + n_rays},
        "gpu_launches": 2 * args.steps,
        "per_kernel": {"closest_mrays_per_s": n_rays / closest_ms / 1e3, "any_mrays_per_s": n_rays / any_ms / 1e3,
                       "boxes_per_closest_ray": cb / n_rays, "prims_per_closest_ray": cp / n_rays,
                       "boxes_per_shadow_ray": ab / n_rays, "prims_per_shadow_ray": ap / n_rays},
        "roofline": {"bound": "hbm", "kernel": "k_trace_batch<false>" if dom_closest else "k_trace_batch<true>",
                     "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
                     "peak_source": f"{peak_kind} HBM copy bandwidth (hbm_gbs)",
                     "bytes_per_unit": (bytes_c if dom_closest else bytes_a) / n_rays},
        "setup_s": {"upload_and_bvh": round(upload_s, 2)},
        **({"tuning": tuning} if tuning else {}),
        "clocks": clocks.summary(c0, c1),
    }
    if cpu_rate is not None:
        line["cpu_baseline"] = {"value": cpu_rate, "unit": "Mrays/s", "cores": cpu_threads, "kind": "port",
                                "sample": cpu_desc}
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def _flagged(par, flags):
    p = TrRenderParams()
    ctypes.memmove(ctypes.byref(p), ctypes.byref(par), ctypes.sizeof(p))
    p.flags = flags
    return p


def frame_config(label, sc, par, gpus) -> dict:
    """The workload of a frame bench: identical in both arms' JSON lines."""
    nl = int(len(sc.light_prims))
    W, H = par.width, par.height
    return {"workload": label, "width": W, "height": H, "spp": par.spp, "max_depth": par.max_depth,
            "min_depth": par.min_depth, "lights": nl, "primitives": int(len(sc.prim_shape)),
            "parallelism": f"replicas x{gpus}",
            "l2": f"path state and queues ({W * H * (324 + 76 * max(nl, 1)) / 1e6:.0f} MB) exceed L2; "
                  "a 256 MiB buffer is written between timed steps"}


BATCH_LABEL = "batch_64_scenes_10k_2M_tris_mixed_res_spp_depth6"
TRAVERSAL_LABEL = "traversal_1M_tris_leaf4_4M_closest_4M_shadow_rays"


def batch_config(gpus) -> dict:
    return {"workload": BATCH_LABEL, "scenes": 64, "parallelism": f"replicas x{gpus}",
            "l2": "path state of all jobs exceeds L2; a 256 MiB buffer is written between timed steps"}


def traversal_config(gpus) -> dict:
    return {"workload": TRAVERSAL_LABEL, "triangles": 1 << 20, "rays_per_step": 2 << 22,
            "parallelism": f"replicas x{gpus}",
            "l2": "a 256 MiB buffer is written before each timed step (nodes + slots ~ 90 MB, rays 256 MB)"}


def launches_of(st) -> int:
    """Kernels one render launched: the persistent kernel's single launch
    (iterations 1), else k_init and 7 kernels per wavefront iteration."""
    return 1 if st.iterations == 1 else 1 + 7 * st.iterations


def apply_tuning(ctx, spec: str | None) -> dict:
    """--tuning key=value,...: tr_tuning fields set on the context."""
    if not spec:
        return {}
    kv = {k.strip(): int(v) for k, v in (p.split("=") for p in spec.split(",") if p)}
    ctx.set_tuning(**{("refill" if k == "trav_refill_lanes" else k): v for k, v in kv.items()})
    return kv


def run_ours(args):
    import torch
    from tracer_gb300.native import GpuContext

    rank, world, local = ranks()
    dist = init_ranks(world)
    torch.cuda.set_device(local)
    label, sc, cam, filt, par = workload(args.workload, args.size)
    ctx = GpuContext(local)
    ctx.upload(sc)
    tuning = apply_tuning(ctx, args.tuning)
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

    # The clock sampler starts before the warm-up: its first NVML query
    # stalls the device, which must not fall into the timed region.
    clocks = ClockSampler(local).__enter__()
    par.flags = 0
    for _ in range(args.warmup):
        # the flush runs in the warm-up too: its first launch loads torch's
        # kernel module, which must not happen inside the timed region
        with torch.cuda.stream(stream):
            flush.zero_()
        ctx.render_dev(cam, filt, par, film.data_ptr())
    stats = []
    barrier()
    c0 = clocks.mark()
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
    c1 = clocks.mark()
    clocks.__exit__()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, dist, f"cuda:{local}")
    samples = sum(s.samples for s in stats)
    value = world * samples / (ms / 1e3) / 1e6

    # end to end through the host-buffer C ABI call: per step the camera,
    # filter and parameters go in (the scene stays resident, as a reference
    # Scene outlives its renders) and the film comes back
    barrier()
    t0 = time.perf_counter()
    e2e_samples = 0
    for _ in range(args.steps):
        out, st = ctx.render(cam, filt, par)
        e2e_samples += st.samples
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    e2e = world * e2e_samples / e2e_s / 1e6
    h2d = ctypes.sizeof(TrCamera) + ctypes.sizeof(TrFilter) + ctypes.sizeof(TrRenderParams)

    # after the timed region: one step with CUDA events around every kernel,
    # one with the traversal counting boxes and primitives tested
    par.flags = TR_RENDER_TIME_STAGES
    ctx.render_dev(cam, filt, par, film.data_ptr())  # creates the event pool
    staged = ctx.render_dev(cam, filt, par, film.data_ptr())
    par.flags = TR_RENDER_COUNT_VISITS
    counted = ctx.render_dev(cam, filt, par, film.data_ptr())
    par.flags = 0

    if rank != 0:
        ctx.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # roofline of the dominant kernel, from the stage-timed step's CUDA events
    stage_ms = dict(zip(STAGE_NAMES, staged.stage_ms))
    iters = staged.iterations
    items = {"extend": staged.extend_rays, "shadow": staged.shadow_rays, "logic": staged.shade_items}
    kernels = [k for k in STAGE_NAMES if k not in ("reset", "bin") and stage_ms[k] > 0]
    dom = max(kernels, key=lambda k: stage_ms[k])
    per = {}
    if staged.extend_rays:
        per["extend"] = (counted.closest_boxes / counted.extend_rays, counted.closest_prims / counted.extend_rays)
    if staged.shadow_rays:
        per["shadow"] = (counted.any_boxes / counted.shadow_rays, counted.any_prims / counted.shadow_rays)
    bpr = kernel_bytes(dom, nl, *per.get(dom, (0.0, 0.0)))
    dom_items = items.get(dom)
    peak, peak_kind = measured_peak_hbm()
    roof = {"bound": "hbm", "kernel": KERNEL_NAMES[dom], "unit": "GB/s", "peak": peak,
            "peak_source": f"{peak_kind} HBM copy bandwidth (hbm_gbs)", "traffic": None,
            "launches": iters, "avg_launch_ms": stage_ms[dom] / max(iters, 1)}
    if dom_items:
        per_launch_bytes = bpr * dom_items / max(iters, 1)
        achieved = per_launch_bytes / (roof["avg_launch_ms"] / 1e3) / 1e9
        roof.update({"achieved": achieved, "frac": achieved / peak, "bytes_per_unit": bpr,
                     "units_per_launch": dom_items / max(iters, 1)})
        tr = traffic_per_unit(dom)
        if tr is not None:
            roof["traffic"] = tr["bytes_per_unit"] * dom_items / max(iters, 1)
            roof["traffic_source"] = tr["source"]
            roof.update(dram_bound(roof["traffic"], roof["avg_launch_ms"], peak))
    else:
        roof.update({"achieved": None, "frac": None})
    conv = None
    if not args.no_convergence and world == 1 and args.workload == "occluded_room" and not args.size:
        conv = convergence(ctx, args.workload)
    cpu_rate, cpu_threads, cpu_desc = (None, None, None)
    if not args.no_cpu_baseline and world == 1:
        cpu_rate, cpu_threads, cpu_desc = cpu_sample(sc, cam, filt, par)
    rays = staged.extend_rays + staged.shadow_rays
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene, no dataset)",
        "config": frame_config(label, sc, par, world),
        "render_mode": "persistent kernel (one launch per render)" if stats[0].iterations == 1 else "wavefront",
        **({"tuning": tuning} if tuning else {}),
        "value_is": "camera samples per second of the plain GPU path tracer (time-to-1% relMSE under "
                    "'convergence')",
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": W * H * 16},
        "gpu_launches": int(sum(launches_of(s) for s in stats)),
        "roofline": roof,
        "rays": {"extend": staged.extend_rays, "shadow": staged.shadow_rays,
                 "mrays_per_s": rays / (ms / args.steps / 1e3) / 1e6,
                 "boxes_per_extend_ray": per.get("extend", (None, None))[0],
                 "prims_per_extend_ray": per.get("extend", (None, None))[1],
                 "boxes_per_shadow_ray": per.get("shadow", (None, None))[0],
                 "prims_per_shadow_ray": per.get("shadow", (None, None))[1],
                 "shadow_rays_answered_by_occluder_cache": staged.occluder_hits},
        "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()},
        "clocks": clocks.summary(c0, c1),
    }
    if conv is not None:
        line["convergence"] = conv
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
    ap.add_argument("--workload", choices=list(WORKLOADS), default="occluded_room")
    ap.add_argument("--no-convergence", action="store_true", help="skip the time-to-1%% relMSE leg")
    ap.add_argument("--size", default=None, help="WxHxSPP override (profiling captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tuning", default=None, help="tr_tuning fields, e.g. render_mode=2,ray_bin_bits=0")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch(args)
    if args.workload == "traversal":
        return run_traversal(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
