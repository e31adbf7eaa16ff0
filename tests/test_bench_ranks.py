"""The multi-rank path of bench.py on CPU: two gloo ranks launched like
torchrun, each contributing its own timing; the reported time is the
slowest rank's and every rank sees it."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
rank, world, local = bench.ranks()
dist = bench.init_ranks(world)
assert dist is not None and dist.get_backend() == "gloo"
t = bench.max_over_ranks(10.0 + rank, dist, "cpu")
assert t == 10.0 + world - 1, t
dist.barrier()
dist.destroy_process_group()
print("rank", rank, "ok", t)
"""


def test_two_gloo_ranks_report_the_slowest_time(tmp_path):
    script = tmp_path / "child.py"
    script.write_text(CHILD.format(root=ROOT))
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT="29533", CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for r, (p, out) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, out
        assert f"rank {r} ok 11.0" in out


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.init_ranks(1) is None
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
