import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def gpu():
    """One GPU context for the session; the native library must load."""
    from tracer_gb300.native import GpuContext
    ctx = GpuContext(0)
    yield ctx
    ctx.close()


class tuned:
    """Context manager: the GPU context's launch tuning with some fields
    changed, restored afterwards (the `gpu` fixture is shared)."""

    FIELDS = ("trav_refill_lanes", "trav_blocks_per_sm", "shade_blocks_per_sm", "graph_iterations", "any_node_width",
              "ray_bin_bits", "treelet_nodes", "occluder_cache", "render_mode", "any_hit_order")

    def __init__(self, gpu, **fields):
        self.gpu, self.fields = gpu, fields

    def __enter__(self):
        self.old = {f: getattr(self.gpu.tuning(), f) for f in self.FIELDS}
        self._apply({**self.old, **self.fields})
        return self.gpu

    def __exit__(self, *exc):
        self._apply(self.old)

    def _apply(self, v):
        self.gpu.set_tuning(v["trav_refill_lanes"], v["trav_blocks_per_sm"], v["shade_blocks_per_sm"],
                            v["graph_iterations"], v["any_node_width"], v["ray_bin_bits"], v["treelet_nodes"],
                            v["occluder_cache"], v["render_mode"], v["any_hit_order"])
