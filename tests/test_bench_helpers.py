"""bench.py's roofline helpers on the host: what bounds a kernel, from its
measured DRAM bytes per launch, and the committed per-item DRAM figures."""
import importlib.util
import os

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
