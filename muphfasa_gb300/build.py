"""Builds libmph.so in-tree: hand-written CUDA for sm_103a plus the C++ host
configuration code, linked into one shared library with the C ABI of
include/mph.h.  Translation units compile in parallel; rebuilds are
incremental on file modification times.

Usage: python -m muphfasa_gb300.build [-v]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libmph.so")
DRIVER = os.path.join(BUILD, "mph_run")
BATCH_DRIVER = os.path.join(BUILD, "mph_batch_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler",
               "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC] + ARCH
# Translation units that must keep the reference's operation order.
EXACT_TUS = {"k_f64_exact.cu"}
HOST_TUS = ["host_config.cpp"]
DEVICE_TUS = ["k_f64_exact.cu", "k_fast_f64.cu", "k_fast_f32.cu", "k_fast_f16.cu", "k_fast_bf16.cu", "k_fast_f16c.cu", "k_fast_f16w.cu", "k_f64x.cu",
              "k_f64x_batch.cu", "ceiling.cu", "noalloc.cu", "monitor.cu", "nn.cu", "batch.cu", "sim.cu"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmph")
    return p


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".h", ".cuh")) and f != "driver_util.h"] + [os.path.join(INCLUDE, "mph.h")]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _headers())


def _compile(src_name: str, verbose: bool):
    src = os.path.join(CSRC, src_name)
    obj = os.path.join(BUILD, src_name + ".o")
    if not _stale(obj, src):
        return obj
    if src_name.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE, "-I", CSRC,
               "-c", src, "-o", obj + ".tmp"]
    else:
        cmd = [_nvcc()] + NVCC_COMMON + (["--fmad=false"] if src_name in EXACT_TUS else []) + [
            "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, file=sys.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    tus = DEVICE_TUS + HOST_TUS
    with cf.ThreadPoolExecutor(max_workers=min(12, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), tus))
    if not (os.path.exists(LIB) and all(os.path.getmtime(o) <= os.path.getmtime(LIB) for o in objs)):
        _link(objs)
    _driver()
    return LIB


def _driver():
    """The host drivers over libmph.so: mph_run (csrc/mph_run.cpp, one
    domain) and mph_batch_run (csrc/mph_batch_run.cpp, many domains)."""
    util = os.path.join(CSRC, "driver_util.h")
    for exe, src_name in ((DRIVER, "mph_run.cpp"), (BATCH_DRIVER, "mph_batch_run.cpp")):
        src = os.path.join(CSRC, src_name)
        deps = [src, util, LIB, os.path.join(INCLUDE, "mph.h")]
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(f) for f in deps):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", CSRC, src, "-o", exe + ".tmp", "-L", BUILD,
               "-lmph", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(exe + ".tmp", exe)


def _link(objs):
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [_nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
