"""Build recipe for the reference's own CUDA implementation ("plain FP32 form").

TEST INFRASTRUCTURE ONLY.  The library it makes, ``oracle/_ref/librectv_ref.so``,
is the reference's unmodified CUDA code (src/cuda/{rectv,admm,operators,
radonusfft}.cu with its headers in src/include/) plus two files of this
directory: ``ref_compat.h`` (force-included; maps the CUDA 12 form of
cudaMemPrefetchAsync that rectv.cu calls onto the CUDA 13 one) and
``ref_shim.cu`` (extern "C" entry points in place of the SWIG module).  Tests
and ``bench.py`` load it, in a process of its own (``oracle/ref_run.py``), to
pin the oracle and this project's GPU path against the reference's CUDA build
and to time that build.  The product (``rectv_gpu_gb300``) never uses it.

Where the reference's sources are present (the build container), they are
read where they lie and also copied into ``oracle/_ref/src/`` -- a build
directory that git ignores, so nothing of the reference enters the
repository's history -- because the GPU machine that runs the tests is an
aarch64 host without the reference's sources: there the recipe compiles the
copy.  Compiled objects never travel (they are built for the host they run
on).

Usage: ``python -m oracle.ref_build`` (prints the library path or the reason
it could not be built).
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = "/root/reference"
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "librectv_ref.so")
CU = ["rectv.cu", "admm.cu", "operators.cu", "radonusfft.cu"]
HDR = ["rectv.cuh", "radonusfft.cuh", "kernels_operators.cuh", "kernels_radonusfft.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _vendor():
    """Copy the reference's CUDA sources into the build directory when they
    are present on this machine."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src", "cuda")):
        return
    for sub, names in (("cuda", CU), ("include", HDR)):
        os.makedirs(os.path.join(SRC, sub), exist_ok=True)
        for nm in names:
            a = os.path.join(REF_ROOT, "src", sub, nm)
            b = os.path.join(SRC, sub, nm)
            if not os.path.exists(b) or os.path.getmtime(b) < os.path.getmtime(a):
                shutil.copy2(a, b)


def _sources():
    return [os.path.join(SRC, "cuda", c) for c in CU] + [os.path.join(HERE, "ref_shim.cu")]


def available():
    return all(os.path.exists(p) for p in _sources())


def _nvcc():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return os.path.join(cand, "bin", "nvcc"), cand
    nvcc = shutil.which("nvcc")
    if not nvcc:
        raise RuntimeError("nvcc not found")
    return nvcc, os.path.dirname(os.path.dirname(nvcc))


def is_stale():
    if not os.path.exists(LIB):
        return True
    deps = _sources() + [os.path.join(SRC, "include", h) for h in HDR] + [os.path.join(HERE, "ref_compat.h"),
                                                                         os.path.abspath(__file__)]
    return os.path.getmtime(LIB) < max(os.path.getmtime(p) for p in deps if os.path.exists(p))


def build(force=False):
    """Returns the library path, or None when the reference's sources are not
    available on this machine."""
    _vendor()
    if not available():
        return None
    if not force and not is_stale():
        return LIB
    nvcc, home = _nvcc()
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nvcc, "-c", src, "-o", obj, "-O3", "-I", os.path.join(SRC, "include"), "-include",
               os.path.join(HERE, "ref_compat.h"), "-Xcompiler", "-fPIC,-fopenmp", "-w"] + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=len(CU) + 1) as ex:
        objs = list(ex.map(compile_one, _sources()))
    libdir = os.path.join(home, "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(home, "lib")
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + [
        "-L", libdir, "-lcufft", "-lcublas", "-lcudart", "-Xcompiler", "-fopenmp", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv)
    print(p if p else "reference sources not available on this machine")
