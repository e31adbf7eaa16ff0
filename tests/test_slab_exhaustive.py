"""The slab test's `tMax *= 1 + 0.0000001` (src/utility/geometry.hpp:848-859)
is float(double(x) * 1.0000001); the kernels evaluate it with one fused
multiply-add and a select (trg::slab_scale in tracer_gb300/csrc/tr_math.cuh). This compiles
that same function for the host and compares it with the double expression
on all 2^32 float bit patterns."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>
#include <atomic>
#include "tr_math.cuh"
static float ref(float x) { float t = x; t *= 1 + 0.0000001; return t; }
int main() {
  std::atomic<unsigned long long> bad{0};
  unsigned nt = std::thread::hardware_concurrency(); if (!nt) nt = 4;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) th.emplace_back([&, t] {
    unsigned long long b = 0;
    const unsigned long long lo = (1ull << 32) * t / nt, hi = (1ull << 32) * (t + 1) / nt;
    for (unsigned long long i = lo; i < hi; ++i) {
      unsigned u = (unsigned)i; float x; std::memcpy(&x, &u, 4);
      float a = ref(x), c = trg::slab_scale(x);
      unsigned ab, cb; std::memcpy(&ab, &a, 4); std::memcpy(&cb, &c, 4);
      if (ab != cb && !(a != a && c != c)) ++b;
    }
    bad += b; });
  for (auto& x : th) x.join();
  std::printf("%llu\n", (unsigned long long)bad.load());
  return bad.load() ? 1 : 0;
}
"""


def test_slab_scale_all_floats():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "slab.cpp")
        exe = os.path.join(d, "slab")
        open(src, "w").write(SRC)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
                        "-I", os.path.join(ROOT, "tracer_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, f"mismatches: {r.stdout}"
