"""Builds the helios-gb300 core (libhx.so) and the CPU oracle in-tree.

The product library is compiled for sm_103a only, with --fmad=false so that
its float arithmetic rounds exactly like the oracle's (bit-exact integer
outputs).  Translation units compile in parallel; nothing is installed.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhx.so")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "-Xptxas", "-v" if os.environ.get("HX_PTXAS_V") else "-O3"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-Wall"]

CU_SOURCES = ["context.cu", "sort.cu", "bvh_build.cu", "scene.cu", "integrator.cu", "server.cu", "denoise.cu"]
CPP_SOURCES = ["procedural.cpp", "image_io.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(ROOT, "include", "hx.h"))
    jobs, objs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            if src.endswith(".cu"):
                jobs.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
            else:
                jobs.append([CXX] + CXX_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        logs.append(_run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


def build_driver():
    """Builds the headless C++ driver (helios_gb300/cpp/hx_render) against libhx.so."""
    src = os.path.join(HERE, "cpp", "hx_render.cpp")
    out = os.path.join(HERE, "cpp", "hx_render")
    deps = [src, os.path.join(ROOT, "include", "hx.h"), os.path.join(ROOT, "include", "helios_gb300.hpp"), LIB]
    if _stale(out, deps):
        _run([CXX, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", out, "-L", HERE, "-lhx",
              "-Wl,-rpath,$ORIGIN/.."])
    return out


def build_oracle():
    d = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", d])
    return os.path.join(d, "liboracle.so")


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_driver()
    build_oracle()
    print(LIB)
