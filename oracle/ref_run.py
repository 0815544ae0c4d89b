"""Runs the reference's own CUDA build (oracle/_ref/librectv_ref.so, made by
oracle/ref_build.py) in a child process.  TEST INFRASTRUCTURE ONLY.

The reference's class owns CUDA managed memory, runs OpenMP threads and its
free() resets the device (src/cuda/rectv.cu:87), so it never shares a
process with this project's library or with PyTorch: the parent writes the
inputs to a temporary .npz file, the child (``python -m oracle.ref_run``)
loads the library with ctypes, makes one ``rectv`` object
(rectv.cu:5-59) and calls ``run`` (rectv.cu:102-252) or ``check_adjoints``
(rectv.cu:255-290) exactly as the reference's Python wrapper does
(src/rectv_gpu/solver.py:45-93, minus its ``lambda0 *= lambda1``, which the
caller applies), and writes the outputs, the wall time of every call and the
per-iteration log values it printed (rectv.cu:238) back.
"""

import ctypes
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_ref", "librectv_ref.so")


def available():
    return os.path.exists(LIB)


def _child(inp, outp):
    d = dict(np.load(inp))
    mode = str(d["mode"])
    lib = ctypes.CDLL(LIB)
    lib.rectvref_create.restype = ctypes.c_void_p
    lib.rectvref_create.argtypes = [ctypes.c_int] * 6
    lib.rectvref_run.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_float] * 3 + [ctypes.c_int] * 2
    lib.rectvref_check_adjoints.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_float] * 2
    g = np.ascontiguousarray(d["g"], dtype=np.float32)
    theta = np.ascontiguousarray(d["theta"], dtype=np.float32)
    phi = np.ascontiguousarray(d["phi"], dtype=np.float32)
    nz, ntheta, n = g.shape
    m = phi.shape[0]
    nzp = int(d["nzp"])
    t0 = time.perf_counter()
    h = lib.rectvref_create(n, ntheta, m, nz, nzp, 1)
    t_create = time.perf_counter() - t0
    out = {"t_create": t_create}
    if mode == "run":
        f = np.zeros((nz, m, n, n), dtype=np.float32)
        times = []
        for niter in [int(x) for x in d["niters"]]:
            t0 = time.perf_counter()
            lib.rectvref_run(h, f.ctypes.data, g.ctypes.data, theta.ctypes.data, phi.ctypes.data,
                             float(d["center"]), float(d["lambda0"]), float(d["lambda1"]), niter, int(d["titer"]))
            times.append(time.perf_counter() - t0)
        out["f"] = f
        out["times"] = np.array(times)
    else:
        res = np.zeros(6, dtype=np.float64)
        lib.rectvref_check_adjoints(h, res.ctypes.data, g.ctypes.data, theta.ctypes.data, phi.ctypes.data,
                                    float(d["lambda1"]), float(d["center"]))
        out["res"] = res
    np.savez(outp, **out)
    sys.stderr.flush()
    # no free(): it would reset the device (rectv.cu:87); process exit releases everything
    os._exit(0)


def _call(inputs, timeout):
    if not available():
        raise RuntimeError("reference CUDA build not available (python -m oracle.ref_build)")
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "in.npz")
        outp = os.path.join(tmp, "out.npz")
        np.savez(inp, **inputs)
        r = subprocess.run([sys.executable, "-m", "oracle.ref_run", inp, outp], cwd=ROOT, capture_output=True,
                           text=True, timeout=timeout)
        if r.returncode != 0 or not os.path.exists(outp):
            raise RuntimeError("reference CUDA build failed (rc %d): %s" % (r.returncode, r.stderr[-2000:]))
        out = dict(np.load(outp))
    rdiff = [float(x) for x in re.findall(r"rdiff \|\|f\(k\+1\)-f\(k\)\|\|:([-+0-9.eEinfa]+)", r.stderr)]
    out["rdiff"] = np.array(rdiff)
    return out


def run(g, theta, phi, center, lambda0, lambda1, niter, titer, nzp, time_niters=None, timeout=3600):
    """rectv(n, ntheta, m, nz, nzp, 1).run(...) of the reference build.

    ``lambda0`` is passed to run() as given.  With ``time_niters`` (a list of
    iteration counts) run() is called once per entry, in order, on the same
    object, and the wall time of every call is returned; the result is the
    last call's.  Returns (f [nz, m, n, n] float32, dict with "times",
    "t_create" and "rdiff", the values the reference printed per iteration).
    """
    niters = list(time_niters) if time_niters else [niter]
    out = _call({"mode": np.array("run"), "g": np.asarray(g, np.float32), "theta": np.asarray(theta, np.float32),
                 "phi": np.asarray(phi, np.float32), "center": center, "lambda0": lambda0, "lambda1": lambda1,
                 "titer": titer, "nzp": nzp, "niters": np.array(niters)}, timeout)
    return out["f"], {"times": list(out["times"]), "t_create": float(out["t_create"]), "rdiff": list(out["rdiff"])}


def check_adjoints(g, theta, phi, lambda1, center, timeout=1800):
    """rectv(n, ntheta, m, nz, nz, 1).check_adjoints(...) of the reference build (res starts at zero)."""
    out = _call({"mode": np.array("adj"), "g": np.asarray(g, np.float32), "theta": np.asarray(theta, np.float32),
                 "phi": np.asarray(phi, np.float32), "center": center, "lambda0": 0.0, "lambda1": lambda1,
                 "titer": 0, "nzp": np.asarray(g).shape[0], "niters": np.array([0])}, timeout)
    return out["res"]


if __name__ == "__main__":
    _child(sys.argv[1], sys.argv[2])
