"""Host build of tracer_gb300/csrc/exact32.cuh against the reference's double
expressions it replaces (normalize, cross, cos, Vector3 / float, the
shadow-ray length, the light pdf). The device build is checked the same way
by tests/test_gpu_exact32.py; this run uses the host's 1/sqrtf as the rsqrt
seed, so it exercises the certification on different approximations."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <thread>
#include <vector>
#include <atomic>
#include "exact32.cuh"
using namespace trg;
static unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull; z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull; return z ^ (z >> 31);
}
static float tf(unsigned long long& s) {
  s = mix64(s);
  unsigned cls = (unsigned)(s & 15u);
  float u = (float)((unsigned)(s >> 40)) * 5.9604645e-08f * 2.0f - 1.0f;
  switch (cls) {
    case 0: return 0.0f;
    case 1: return std::ldexp(u, (int)((s >> 8) & 63u) - 32);
    case 2: return (float)((int)((s >> 8) & 15u) - 8);
    case 3: return 1.0f - std::fabs(u) * 1e-6f;
    default: return u;
  }
}
static f3 tv(unsigned long long& s) { float a = tf(s), b = tf(s), c = tf(s); return mk3(a, b, c); }
static bool same(float a, float b) { unsigned x, y; std::memcpy(&x, &a, 4); std::memcpy(&y, &b, 4); return x == y || (a != a && b != b); }
static bool same3(f3 a, f3 b) { return same(a.x, b.x) && same(a.y, b.y) && same(a.z, b.z); }
int main(int argc, char** argv) {
  const unsigned long long n = std::strtoull(argv[1], 0, 10);
  std::atomic<unsigned long long> bad[6];
  for (auto& b : bad) b = 0;
  unsigned nt = std::thread::hardware_concurrency(); if (!nt) nt = 4;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) th.emplace_back([&, t] {
    unsigned long long lb[6] = {0};
    for (unsigned long long i = t; i < n; i += nt) {
      unsigned long long s = mix64(i * 0x632be59bd9b4e019ull + 7);
      f3 a = tv(s), b = tv(s);
      if ((s >> 60) == 0) b = a + scale(b, 1e-5f);
      if (!same3(cross_x(a, b), cross_d(a, b))) lb[0]++;
      f3 c = ((s >> 61) == 0) ? normalize_d(a) : a;
      if (!same3(normalize_x(c), normalize_d(c))) lb[1]++;
      if (!same(cos_x(a, b), cosv_d(a, b))) lb[2]++;
      float f = tf(s);
      if (!same3(div_x(a, f), divd(a, (double)f))) lb[3]++;
      float L = std::fabs(tf(s));
      if ((s >> 62) == 0) L = 3.6e-7f * (1.0f + tf(s) * 1e-3f);
      bool le; float d = dist_minus_eps(L, le);
      double dd = std::sqrt((double)L) - (double)kEps;
      if (!same(d, (float)dd) || le != (dd <= (double)kEps)) lb[4]++;
      float A = std::fabs(tf(s)) + 1e-3f, dt = tf(s), L2 = std::fabs(tf(s));
      if (!same(area_to_solid_pdf(A, dt, L2), (float)((double)A / std::fabs((double)dt / std::sqrt((double)L2))))) lb[5]++;
    }
    for (int k = 0; k < 6; ++k) bad[k] += lb[k]; });
  for (auto& x : th) x.join();
  unsigned long long tot = 0;
  for (int k = 0; k < 6; ++k) { std::printf("%llu ", (unsigned long long)bad[k].load()); tot += bad[k]; }
  std::printf("\n");
  return tot ? 1 : 0;
}
"""


def test_exact32_host():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "x.cpp")
        exe = os.path.join(d, "x")
        open(src, "w").write(SRC)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
                        "-I", os.path.join(ROOT, "tracer_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe, "20000000"], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, f"mismatches (cross normalize cos div dist pdf): {r.stdout}"
