"""bench.py on the host: the roofline helpers (what bounds a kernel, from its
measured DRAM bytes per launch; the committed per-item DRAM figures) and the
reference arm's JSON line, which needs no GPU."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_dram_bound_labels_latency_and_hbm(bench):
    # 1 GB in 1 ms is 1000 GB/s: 0.15 of a 6698 GB/s peak, a latency-bound walk
    r = bench.dram_bound(1e9, 1.0, 6698.0)
    assert r["bound"] == "latency"
    assert r["dram_gbs"] == pytest.approx(1000.0)
    assert r["dram_frac"] == pytest.approx(1000.0 / 6698.0)
    # 5 GB in 1 ms is 0.75 of the peak: bandwidth-bound
    r = bench.dram_bound(5e9, 1.0, 6698.0)
    assert r["bound"] == "hbm"
    assert r["dram_frac"] == pytest.approx(5000.0 / 6698.0)
    # the threshold is half the peak
    assert bench.dram_bound(0.5 * 6698e9 * 1e-3, 1.0, 6698.0)["bound"] == "hbm"
    assert bench.dram_bound(0.49 * 6698e9 * 1e-3, 1.0, 6698.0)["bound"] == "latency"


def test_committed_traffic_figures(bench):
    """The per-ray DRAM figures the bench scales to a launch are the ncu
    summaries' (read + write bytes per ray), and absent stages give None."""
    ext, sh = bench.traffic_per_unit("extend"), bench.traffic_per_unit("shadow")
    assert ext["bytes_per_unit"] == pytest.approx(209.7)
    assert sh["bytes_per_unit"] == pytest.approx(239.7)
    assert "ncu" in ext["source"] and "ncu" in sh["source"]
    assert bench.traffic_per_unit("material") is None


def _reference_arm(env_extra):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                           "cornell", "--size", "32x32x2", "--steps", "2", "--warmup", "1"],
                          env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)


def test_reference_arm_line():
    """The reference arm times the CPU restatement on the host cores and
    prints one JSON line carrying the keys the contract names."""
    r = _reference_arm({})
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["higher_is_better"] is True and d["unit"] == "Msamples/s"
    assert d["config"]["workload"].startswith("cornell_box_36tris_32x32_2spp")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 runs and prints; the others exit 0."""
    r = _reference_arm({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stdout + r.stderr
    assert not [x for x in r.stdout.splitlines() if x.startswith("{")]
