"""Builds the native library libtracer_gb300.so in-tree (tracer_gb300/_build).

CUDA sources compile for sm_103a only, without multiply-add contraction
(--fmad=false on the device, -ffp-contract=off on the host): the hot path
reproduces the reference's float/double arithmetic operation by operation.
Translation units compile in parallel; the library links the CUDA runtime
statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtracer_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "--fmad=false", "-Xptxas", "-v",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{INCLUDE}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}"]

CU_SOURCES = ["context.cu", "render.cu", "mega.cu", "selftest.cu", "mlp.cu", "bvh_gpu.cu", "post.cu", "env_light.cu"]
CXX_SOURCES = ["bvh_build.cpp", "host_api.cpp", "image_out.cpp", "obj_load.cpp", "image_file.cpp", "image_formats.cpp"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tracer_gb300")
    return p


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + [os.path.join(INCLUDE, "tracer_gpu.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles every CUDA/C++ unit and links the shared library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(OUT, f.rsplit(".", 1)[0] + ".o")
        jobs.append(([nvcc(), *CU_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj], obj,
                     os.path.join(OUT, f.rsplit(".", 1)[0] + ".ptxas.log")))
    for f in CXX_SOURCES:
        obj = os.path.join(OUT, f.rsplit(".", 1)[0] + ".o")
        jobs.append((["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj], obj, None))

    def run(job):
        cmd, obj, log = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if log:
            with open(log, "w") as fh:
                fh.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(" ".join(cmd))
        return obj

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
