"""Build recipe for librectv_gb300.so (sm_103a only).

Each translation unit is compiled by nvcc in parallel and linked into
``rectv_gpu_gb300/librectv_gb300.so`` next to this file.  Host code is compiled
without floating-point contraction so the angle plan (plan.cpp) reproduces the
device's sample-position arithmetic exactly.

Usage: ``python -m rectv_gpu_gb300.build`` or ``build()`` from Python.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_NAME = "librectv_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
BUILD_DIR = os.path.join(HERE, "_build")

SOURCES = ["plan.cpp", "usfft_kernels.cu", "gather_tc.cu", "scatter_tc.cu", "dir_kernels.cu", "fft_kernels.cu", "tv_kernels.cu", "io_kernels.cu", "rectv_host.cu", "engine.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _nvcc():
    return os.path.join(_cuda_home(), "bin", "nvcc")


def _compile(src, verbose):
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [_nvcc(), "-c", path, "-o", obj, "-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC,
           "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread"]
    if src.endswith(".cu"):
        cmd += ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
        if os.environ.get("RECTV_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    if verbose and (res.stdout or res.stderr):
        sys.stderr.write(res.stdout + res.stderr)
    return obj


def _newest_input():
    paths = [os.path.join(CSRC, s) for s in SOURCES]
    paths += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    paths += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def is_stale():
    return (not os.path.exists(LIB_PATH)) or os.path.getmtime(LIB_PATH) < _newest_input()


def build(force=False, verbose=False):
    """Compile and link the library if any source is newer than it."""
    if not force and not is_stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    libdir = os.path.join(_cuda_home(), "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(_cuda_home(), "lib")
    tmp = LIB_PATH + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH + [
        "-L", libdir, "-lcufft", "-lcudart", "-Xcompiler", "-pthread", "-Xlinker", "-rpath," + libdir]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
