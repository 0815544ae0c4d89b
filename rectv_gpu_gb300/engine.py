"""Multi-problem engine: the batched form and the serving loop.

Python face of the C ABI ``rectv_engine_*`` (include/rectv_gb300.h).  A job is
one reconstruction (the arguments of ``rectv.run``, rectv.cu:102-252 of the
reference, with its own n, ntheta, m, nz, nzp).  Jobs are admitted in order of
arrival when their estimated device memory fits the HBM budget; an admitted
job's state stays resident on the GPU until its last iteration, its
iterations run on its own stream, and the kernels of all running jobs
overlap on the device.  Each job's result equals ``rectv.run`` on it alone.

Example::

    eng = Engine(budget_bytes=200e9)
    jid = eng.submit(g, theta, phi, nzp=8, niter=32, titer=4, arrival=0.0)
    eng.run()
    f = eng.result(jid)        # [nz, m, n, n] float32
    eng.info(jid)["latency"]   # completion - arrival, seconds
"""

import ctypes

import numpy as np

from . import _lib

NO_REUSE = 1
AUTOTUNE = 2
LARGEST_FIRST = 4
AGE_PRIORITY = 8
SHORTEST_FIRST = 16
STATUS = {0: "waiting", 1: "running", 2: "done", 3: "failed"}


def _pinned(shape, dtype=np.float32):
    """A host array in page-locked memory when torch is importable (the
    engine's copies then overlap with other jobs' kernels), else pageable."""
    try:
        import torch
        t = torch.empty(shape, dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
        return t.numpy(), t
    except Exception:
        return np.empty(shape, dtype=dtype), None


class Engine:
    def __init__(self, budget_bytes=0.0, max_resident=0, reuse=True, autotune=False, largest_first=False,
                 age_priority=True, pin=True, shortest_first=False):
        """budget_bytes <= 0: the free device memory minus 4 GiB; max_resident
        <= 0: no limit on running jobs; age_priority: each job's stream has a
        lower priority than the jobs running when it was admitted (the oldest
        runs first, newer jobs fill the SMs it leaves idle); shortest_first:
        among the jobs that have arrived, the one with the least work is
        admitted first (instead of the first to arrive)."""
        lib = _lib.load()
        flags = ((0 if reuse else NO_REUSE) | (AUTOTUNE if autotune else 0) | (LARGEST_FIRST if largest_first else 0)
                 | (AGE_PRIORITY if age_priority else 0) | (SHORTEST_FIRST if shortest_first else 0))
        h = ctypes.c_void_p()
        _lib.check(lib.rectv_engine_create(float(budget_bytes), int(max_resident), flags, ctypes.byref(h)))
        self._h = h
        self._pin = pin
        self._keep = {}

    def submit(self, g, theta, phi, nzp, niter, titer, center=None, lambda0=1e-3, lambda1=1.0, arrival=0.0,
               scale_lambda0=True, out=None, copy_input=None):
        """Queue one reconstruction; g [nz, ntheta, n] float32, theta [ntheta],
        phi [m, 2*ntheta].  lambda0 is multiplied by lambda1 as Solver.recon
        does (solver.py:76) unless scale_lambda0=False.  `out` (float32
        [nz, m, n, n], C-contiguous) receives the result, else a new array
        does; g is copied into page-locked memory unless copy_input=False (the
        caller's array is then used as is and must stay alive and unchanged
        until run() returns).  Returns the job id."""
        if copy_input is None:
            copy_input = self._pin
        g = np.ascontiguousarray(g, dtype=np.float32)
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        phi = np.ascontiguousarray(phi, dtype=np.float32)
        nz, ntheta, n = g.shape
        m = phi.shape[0]
        if theta.shape != (ntheta,) or phi.shape != (m, 2 * ntheta):
            raise ValueError("theta must be [ntheta] and phi [m, 2*ntheta]")
        if center is None:
            center = n / 2
        if scale_lambda0:
            lambda0 = lambda0 * lambda1
        gp, gt = g, None
        if copy_input:
            gp, gt = _pinned(g.shape)
            gp[...] = g
        ot = None
        if out is None:
            out, ot = _pinned((nz, m, n, n)) if self._pin else (np.empty((nz, m, n, n), dtype=np.float32), None)
        elif out.shape != (nz, m, n, n) or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 array [nz, m, n, n]")
        jid = ctypes.c_int()
        _lib.check(_lib.load().rectv_engine_submit(
            self._h, n, ntheta, m, nz, int(nzp), gp.ctypes.data, theta.ctypes.data, phi.ctypes.data, float(center),
            float(lambda0), float(lambda1), int(niter), int(titer), float(arrival), out.ctypes.data,
            ctypes.byref(jid)))
        self._keep[jid.value] = (gp, gt, theta, phi, out, ot)
        return jid.value

    def run(self):
        """Run every queued job to completion (arrival times count from now)."""
        _lib.check(_lib.load().rectv_engine_run(self._h))

    def result(self, jid):
        return self._keep[jid][4]

    def info(self, jid):
        times = (ctypes.c_double * 3)()
        byts = (ctypes.c_double * 2)()
        rr = (ctypes.c_double * 2)()
        tune = (ctypes.c_int * 2)()
        st = ctypes.c_int()
        _lib.check(_lib.load().rectv_engine_job_info(self._h, int(jid), times, byts, rr, tune, ctypes.byref(st)))
        buf = ctypes.create_string_buffer(1024)
        _lib.check(_lib.load().rectv_engine_job_error(self._h, int(jid), buf, 1024))
        return {"arrival": times[0], "admitted": times[1], "done": times[2], "latency": times[2] - times[0],
                "queued": times[1] - times[0], "est_bytes": byts[0], "bytes": byts[1], "rho": rr[0],
                "rdiff": rr[1], "zper": tune[0], "sc_grid": tune[1], "status": STATUS[st.value],
                "error": buf.value.decode()}

    def stats(self):
        s = (ctypes.c_double * 4)()
        _lib.check(_lib.load().rectv_engine_stats(self._h, s))
        return {"makespan": s[0], "peak_bytes": s[1], "budget": s[2], "peak_running": int(s[3])}

    def close(self):
        if self._h:
            _lib.load().rectv_engine_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
