"""Python class ``rectv``: the object the reference exposes through SWIG.

Mirrors src/cuda/rectv.i:9-28 of nikitinvv/rectv_gpu: constructor
``rectv(n, ntheta, m, nz, nzp, ngpus)``, read-only attributes ``n, ntheta, m,
nz``, and ``run``, ``check_adjoints``, ``free`` taking raw host addresses as
integers.  Backed by the C ABI of librectv_gb300.so (include/rectv_gb300.h).

Beyond the reference: the device-resident session (``setup_device``,
``iterate``, ``result_device``), per-iteration ``history()``, and the
reference's private operators (``op_*``) for testing.
"""

import ctypes

import numpy as np

from . import _lib


def _addr(x):
    return ctypes.c_void_p(int(x)) if x is not None else ctypes.c_void_p(0)


class rectv:
    """One reconstruction object on the current CUDA device (rectv.cuh:7-55)."""

    def __init__(self, n, ntheta, m, nz, nzp, ngpus):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.rectv_create(int(n), int(ntheta), int(m), int(nz), int(nzp), int(ngpus),
                                    ctypes.byref(h)))
        self._h = h
        dims = [ctypes.c_int() for _ in range(6)]
        _lib.check(lib.rectv_get_dims(h, *[ctypes.byref(d) for d in dims]))
        self._dims = tuple(d.value for d in dims)

    # -- read-only attributes (rectv.i:14-18) --
    @property
    def n(self):
        return self._dims[0]

    @property
    def ntheta(self):
        return self._dims[1]

    @property
    def m(self):
        return self._dims[2]

    @property
    def nz(self):
        return self._dims[3]

    @property
    def nzp(self):
        return self._dims[4]

    @property
    def ngpus(self):
        return self._dims[5]

    # -- reference methods (rectv.i:23-27) --
    def run(self, fres, g, theta, phi, center, lambda0, lambda1, niter, titer):
        """rectv::run (rectv.cu:102-252) on host addresses."""
        _lib.check(_lib.load().rectv_run(self._h, _addr(fres), _addr(g), _addr(theta), _addr(phi),
                                         float(center), float(lambda0), float(lambda1), int(niter),
                                         int(titer)))

    def check_adjoints(self, res, g, theta, phi, lambda1, center):
        """rectv::check_adjoints (rectv.cu:255-290); accumulates into res (float64[6])."""
        _lib.check(_lib.load().rectv_check_adjoints(self._h, _addr(res), _addr(g), _addr(theta),
                                                    _addr(phi), float(lambda1), float(center)))

    def free(self):
        """rectv::free (rectv.cu:63-91): idempotent; never resets the device."""
        if self._h:
            _lib.check(_lib.load().rectv_free(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().rectv_destroy(h)
            except Exception:
                pass
            self._h = None

    # -- extensions --
    def run_init(self, fres, g, theta, phi, finit, center, lambda0, lambda1, niter, titer):
        """run starting from the host array at address finit [nz][m][n][n]."""
        _lib.check(_lib.load().rectv_run_init(self._h, _addr(fres), _addr(g), _addr(theta), _addr(phi),
                                              _addr(finit), float(center), float(lambda0), float(lambda1),
                                              int(niter), int(titer)))

    def fbp_run(self, frec, g, theta, center):
        """Filtered backprojection into the host array at address frec [nz][n][n]."""
        _lib.check(_lib.load().rectv_fbp(self._h, _addr(frec), _addr(g), _addr(theta), float(center)))

    def set_verbose(self, verbose):
        _lib.check(_lib.load().rectv_set_verbose(self._h, int(bool(verbose))))

    def set_graphs(self, enable):
        _lib.check(_lib.load().rectv_set_graphs(self._h, int(bool(enable))))

    def setup_device(self, g_ptr, theta_ptr, phi_ptr, center, lambda0, lambda1, titer):
        _lib.check(_lib.load().rectv_setup_device(self._h, _addr(g_ptr), _addr(theta_ptr), _addr(phi_ptr),
                                                  float(center), float(lambda0), float(lambda1),
                                                  int(titer)))

    def iterate(self, niter):
        _lib.check(_lib.load().rectv_iterate(self._h, int(niter)))

    def result_device(self, f_ptr):
        _lib.check(_lib.load().rectv_get_result_device(self._h, _addr(f_ptr)))

    @property
    def stream(self):
        s = ctypes.c_void_p()
        _lib.check(_lib.load().rectv_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def synchronize(self):
        _lib.check(_lib.load().rectv_synchronize(self._h))

    def history(self):
        """Per outer iteration: rdiff=||f(k+1)-f(k)||^2, rho, r, s (rectv.cu:223-238)."""
        cnt = ctypes.c_int(0)
        _lib.check(_lib.load().rectv_get_history(self._h, None, None, None, None, ctypes.byref(cnt)))
        k = cnt.value
        out = {key: np.zeros(k) for key in ("rdiff", "rho", "r", "s")}
        if k:
            cnt = ctypes.c_int(k)
            _lib.check(_lib.load().rectv_get_history(
                self._h, out["rdiff"].ctypes.data, out["rho"].ctypes.data, out["r"].ctypes.data,
                out["s"].ctypes.data, ctypes.byref(cnt)))
        return out

    def op_set_geometry(self, theta_ptr, phi_ptr, center):
        _lib.check(_lib.load().rectv_op_set_geometry(self._h, _addr(theta_ptr), _addr(phi_ptr),
                                                     float(center)))

    def directions(self):
        """Number of ray directions whose rays share sample positions in the
        current geometry (0: every ray is interpolated on its own)."""
        nd, nr = ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(_lib.load().rectv_get_directions(self._h, ctypes.byref(nd), ctypes.byref(nr)))
        return nd.value

    def op_radonapr(self, g_ptr, f_ptr, nslices, tau=1.0):
        _lib.check(_lib.load().rectv_op_radonapr(self._h, _addr(g_ptr), _addr(f_ptr), int(nslices),
                                                 float(tau)))

    def op_radonapradj(self, f_ptr, g_ptr, nslices, tau=1.0):
        _lib.check(_lib.load().rectv_op_radonapradj(self._h, _addr(f_ptr), _addr(g_ptr), int(nslices),
                                                    float(tau)))

    def op_gradient(self, h2_ptr, fm_ptr, lambda1, flgl, flgr):
        _lib.check(_lib.load().rectv_op_gradient(self._h, _addr(h2_ptr), _addr(fm_ptr), float(lambda1),
                                                 int(flgl), int(flgr)))

    def op_divergent(self, fn_ptr, h2_ptr, lambda1, tau):
        _lib.check(_lib.load().rectv_op_divergent(self._h, _addr(fn_ptr), _addr(h2_ptr), float(lambda1),
                                                  float(tau)))

    def autotune(self, force=False):
        """Pick the launch shapes of the tensor-core USFFT kernels for this
        problem by timing them (after setup_device); returns (gather slices
        per block, scatter blocks or 0 for one per SM)."""
        z = ctypes.c_int()
        sg = ctypes.c_int()
        _lib.check(_lib.load().rectv_autotune(self._h, int(bool(force)), ctypes.byref(z), ctypes.byref(sg)))
        return z.value, sg.value

    def device_bytes(self):
        b = ctypes.c_double()
        _lib.check(_lib.load().rectv_get_device_bytes(self._h, ctypes.byref(b)))
        return b.value


def estimate_bytes(n, ntheta, m, nz, nzp):
    """Estimated device memory of a rectv object with these dimensions."""
    b = ctypes.c_double()
    _lib.check(_lib.load().rectv_estimate_bytes(int(n), int(ntheta), int(m), int(nz), int(nzp), ctypes.byref(b)))
    return b.value


def plan_directions(theta, n, tol_cells=0.0, min_group=0.0):
    """(directions, most rays in one direction) of a geometry, on the host.

    directions is the number of ray directions (theta modulo pi) whose rays
    would share sample positions, 0 when the geometry keeps the per-ray
    kernels; the defaults (0) are those of geometry set-up: 2e-3 grid cells,
    2.5 rays per direction.  No GPU is needed."""
    th = np.ascontiguousarray(theta, dtype=np.float32)
    nd, mr = ctypes.c_int(), ctypes.c_int()
    _lib.check(_lib.load().rectv_plan_directions(th.ctypes.data, int(n), int(th.size), float(tol_cells),
                                                 float(min_group), ctypes.byref(nd), ctypes.byref(mr)))
    return nd.value, mr.value
