"""Module for 4D tomography: ``Solver``, the reference's user-facing class.

Mirrors src/rectv_gpu/solver.py:11-93 of nikitinvv/rectv_gpu: same
constructor, context-manager behaviour, ``recon`` and ``adjoint_tests`` with
the same defaults and conventions (``lambda0 *= lambda1``, rotation centre
``n/2`` by default, result ``[nz, m, n, n]`` float32).  Arrays are converted to
C-contiguous float32 and their shapes checked before their addresses are
passed down (the reference passes them unchecked).

``Solver.from_scan`` adds the keyword form
``(N, Ntheta, M, Nrot, Nz, Nzp, ngpus=1, center, lambda0, lambda1)``: it
builds equally spaced angles over Nrot half-turns and the Fourier temporal
basis, and stores centre and regularisation defaults for ``reconstruct``.
"""

import numpy as np

from .rectv import rectv


def getp(a):
    """Address of an array's data (solver.py:7-8)."""
    return a.__array_interface__["data"][0]


def takephi(ntheta, m):
    """Fourier temporal basis [m, 2*ntheta] float32, interleaved (re, im):
    phi_i(k) = exp(2 pi i (k - ntheta/2)(i - m/2)/ntheta)/sqrt(ntheta)
    (the basis of the reference's test and examples, tests/test_adjoint.py:23-27)."""
    x, y = np.meshgrid(np.arange(-ntheta // 2, ntheta // 2), np.arange(-m // 2, m // 2))
    phi = np.zeros([m, 2 * ntheta], dtype="float32")
    phi[:, ::2] = np.cos(2 * np.pi * x * y / ntheta) / np.sqrt(ntheta)
    phi[:, 1::2] = np.sin(2 * np.pi * x * y / ntheta) / np.sqrt(ntheta)
    return phi


def _f32(a, shape, name):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != tuple(shape):
        raise ValueError("%s must have shape %s, got %s" % (name, tuple(shape), a.shape))
    return a


class Solver(rectv):
    """Base class for the time-resolved tomography solver (solver.py:11-30).

    Attributes
    ----------
    ntheta : int
        The number of projections.
    n, nz : int
        The pixel width and height of the projection.
    m : int
        The number of time samples / temporal basis functions.
    nzp : int
        The number of slices processed together (one ADMM chunk).
    ngpus : int
        Number of GPUs (clamped to nz//nzp; this build runs on one device).
    """

    def __init__(self, n, ntheta, m, nz, nzp, ngpus=1):
        super().__init__(n, ntheta, m, nz, nzp, ngpus)
        self.theta = None
        self.phi = None
        self.rot_center = None
        self.lambda0 = 1e-3
        self.lambda1 = 1.0

    def __enter__(self):
        """Return self at start of a with-block."""
        return self

    def __exit__(self, type, value, traceback):
        """Free GPU memory due at interruptions or with-block exit."""
        self.free()

    def recon(self, data, theta, phi, rot_center=None, lambda0=1e-3, lambda1=1, niter=1, titer=1, *,
              init=None):
        """Reconstruct with the time-resolved method (solver.py:45-84).

        data : float [nz, ntheta, n] projections; theta : float [ntheta];
        phi : float [m, 2*ntheta] temporal basis; rot_center defaults to n/2;
        lambda0, lambda1 regularisation; niter outer ADMM iterations, titer
        inner iterations.  Returns float32 [nz, m, n, n].

        init (keyword, extension): None starts from zero like the reference;
        'fbp' starts from the filtered backprojection of every slice (the same
        image at every time sample); an array [nz, m, n, n] starts from it.
        """
        # equivalent problem: lambda0 is applied as lambda0*lambda1 (solver.py:76)
        lambda0 *= lambda1
        if rot_center is None:
            rot_center = self.n / 2
        data = _f32(data, (self.nz, self.ntheta, self.n), "data")
        theta = _f32(theta, (self.ntheta,), "theta")
        phi = _f32(phi, (self.m, 2 * self.ntheta), "phi")
        rtv = np.zeros([self.nz, self.m, self.n, self.n], dtype="float32")
        if init is None:
            self.run(getp(rtv), getp(data), getp(theta), getp(phi), rot_center, lambda0, lambda1,
                     niter, titer)
            return rtv
        if isinstance(init, str):
            if init != "fbp":
                raise ValueError("init must be None, 'fbp' or an array")
            f0 = self.fbp(data, theta, rot_center)
            init = np.ascontiguousarray(np.broadcast_to(f0[:, None], rtv.shape))
        init = _f32(init, rtv.shape, "init")
        self.run_init(getp(rtv), getp(data), getp(theta), getp(phi), getp(init), rot_center, lambda0,
                      lambda1, niter, titer)
        return rtv

    def fbp(self, data, theta, rot_center=None):
        """Filtered backprojection of every slice (static object): float32
        [nz, n, n], with the reference's ramp filter and circular mask
        (applyfilter, circ: kernels_radonusfft.cuh:146-189)."""
        if rot_center is None:
            rot_center = self.n / 2
        data = _f32(data, (self.nz, self.ntheta, self.n), "data")
        theta = _f32(theta, (self.ntheta,), "theta")
        out = np.zeros([self.nz, self.n, self.n], dtype="float32")
        self.fbp_run(getp(out), getp(data), getp(theta), rot_center)
        return out

    def adjoint_tests(self, data, theta, phi, lambda1, rot_center=None):
        """Adjoint test values (solver.py:86-93); see rectv_check_adjoints."""
        if rot_center is None:
            rot_center = self.n / 2
        data = _f32(data, (self.nz, self.ntheta, self.n), "data")
        theta = _f32(theta, (self.ntheta,), "theta")
        phi = _f32(phi, (self.m, 2 * self.ntheta), "phi")
        res = np.zeros([6])
        self.check_adjoints(getp(res), getp(data), getp(theta), getp(phi), lambda1, rot_center)
        return res

    # -- keyword form of the constructor --
    @classmethod
    def from_scan(cls, N, Ntheta, M, Nrot, Nz, Nzp, ngpus=1, center=None, lambda0=1e-3, lambda1=1.0):
        """Solver for a continuous scan of Nrot half-turns with Ntheta equally
        spaced angles, M Fourier temporal basis functions, rotation centre
        ``center`` (default N/2) and regularisation defaults."""
        s = cls(N, Ntheta, M, Nz, Nzp, ngpus)
        s.theta = np.linspace(0, Nrot * np.pi, Ntheta, endpoint=False).astype("float32")
        s.phi = takephi(Ntheta, M)
        s.rot_center = N / 2 if center is None else center
        s.lambda0 = lambda0
        s.lambda1 = lambda1
        return s

    def reconstruct(self, data, niter=1, titer=4):
        """``recon`` with the angles, basis, centre and lambdas stored by from_scan."""
        if self.theta is None:
            raise ValueError("reconstruct() needs a Solver built with from_scan()")
        return self.recon(data, self.theta, self.phi, rot_center=self.rot_center,
                          lambda0=self.lambda0, lambda1=self.lambda1, niter=niter, titer=titer)
