"""FP64 NumPy/SciPy oracle of the rectv_gpu reconstruction hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
The product path (``rectv_gpu_gb300``) never calls it and fails loudly when its
CUDA library is missing.

It restates, step by step and in float64, what the reference computes
(nikitinvv/rectv_gpu; citations are ``file:line`` inside that project):

* USFFT Radon transform ``radonusfft::fwdR`` / ``adjR``
  (src/cuda/radonusfft.cu:5-135, kernels in src/include/kernels_radonusfft.cuh:4-215)
* temporal-basis operators ``rectv::radonapr`` / ``radonapradj``
  (src/cuda/operators.cu:6-58, kernels src/include/kernels_operators.cuh:75-149)
* 4D gradient / divergence ``rectv::gradient`` / ``divergent``
  (src/cuda/operators.cu:60-71, kernels src/include/kernels_operators.cuh:4-73)
* linearised ADMM ``rectv::solver_admm`` (src/cuda/admm.cu:5-122)
* outer loop with z-chunks, 1-slice halo from the previous iterate and the rho rule
  ``rectv::run`` (src/cuda/rectv.cu:102-252)
* ``rectv::check_adjoints`` (src/cuda/rectv.cu:255-290)
* the Python wrapper's conventions ``Solver.recon`` (src/rectv_gpu/solver.py:45-93)

The structure deliberately follows the reference (one fwdR/adjR per basis
function, explicit fftshift modulations, padded grid with wrap halo) so that the
GPU implementation, which reorganises the arithmetic, is checked against an
independent, literal restatement.

Pinning: the USFFT restatement is checked against the reference's own test
(tests/test_adjoint.py:132-158, adjoint identities), against analytic Radon
projections of a Gaussian blob (known answer, independent of the code), and the
GPU build is checked against this oracle.  The reference's CUDA build cannot run
in this environment, so no golden vectors from the reference binary exist.
"""

import numpy as np
import scipy.sparse as sp

# kernels_radonusfft.cuh:1 -- the USFFT kernels use this truncated constant.
PI_USFFT = 3.1415926535
# kernels_operators.cuh:2
PI_OPS = np.pi


# ---------------------------------------------------------------------------
# USFFT parameters and geometry
# ---------------------------------------------------------------------------

def usfft_params(n):
    """Gaussian width ``mu`` and interpolation radius ``r`` (radonusfft.cu:10-11).

    ``mu`` is a float member in the reference, so it is rounded to float32.
    ``r`` evaluates to 4 for every detector width.
    """
    eps = np.float32(1e-3)
    mu = np.float32(-np.log(np.float64(eps)) / (2.0 * n * n))
    r = int(np.ceil(2.0 * n / PI_USFFT *
                    np.sqrt(-float(mu) * np.log(float(eps)) + (float(mu) * n) ** 2 / 4.0)))
    return float(mu), r


def takexy(theta, n):
    """Polar frequency points (kernels_radonusfft.cuh:66-79).

    Returns x, y of shape [ntheta, n]; x uses sin, y uses cos; values >= 0.5
    are clamped to 0.5-1e-5 (only the k=0 sample can reach 0.5, and that
    sample is zeroed by the gather).
    """
    th = np.asarray(theta, dtype=np.float64)
    q = (np.arange(n) - n // 2) / float(n)
    x = q[None, :] * np.sin(th)[:, None]
    y = q[None, :] * np.cos(th)[:, None]
    x = np.where(x >= 0.5, 0.5 - 1e-5, x)
    y = np.where(y >= 0.5, 0.5 - 1e-5, y)
    return x, y


def takeshift(c, n):
    """Centre phase ramp exp(i 2 pi c (k-n/2)/n) (kernels_radonusfft.cuh:191-198)."""
    k = np.arange(n, dtype=np.float64)
    return np.exp(1j * 2 * PI_USFFT * c * (k - n / 2.0) / n)


def gather_matrix(theta, n):
    """Sparse interpolation matrix of ``gather`` (kernels_radonusfft.cuh:81-144).

    Rows: polar points (theta index major, detector index minor), n*ntheta.
    Columns: cells of the padded grid (2n+2r)^2 in row-major [y][x] order.
    Entries: w / n with w = PI/mu exp(-PI^2/mu (w0^2+w1^2)); the rows of the
    k=0 samples are empty (the reference zeroes them).
    The forward gather is ``G @ fde``, the adjoint scatter is ``G.T @ g``.
    """
    mu, r = usfft_params(n)
    x, y = takexy(theta, n)
    ntheta = x.shape[0]
    pw = 2 * n + 2 * r
    x0 = x.ravel()
    y0 = y.ravel()
    fx = np.floor(2 * n * x0).astype(np.int64)
    fy = np.floor(2 * n * y0).astype(np.int64)
    npts = x0.size
    rows = np.repeat(np.arange(npts, dtype=np.int64), (2 * r + 1) ** 2)
    i1, i0 = np.meshgrid(np.arange(2 * r + 1), np.arange(2 * r + 1), indexing="ij")
    i1 = i1.ravel()
    i0 = i0.ravel()
    ell0 = fx[:, None] - r + i0[None, :]
    ell1 = fy[:, None] - r + i1[None, :]
    w0 = ell0 / float(2 * n) - x0[:, None]
    w1 = ell1 / float(2 * n) - y0[:, None]
    w = PI_USFFT / mu * np.exp(-PI_USFFT * PI_USFFT / mu * (w0 * w0 + w1 * w1)) / n
    # zero the tx==0 samples
    k = np.tile(np.arange(n), ntheta)
    w[k == 0, :] = 0.0
    cols = (n + r + ell0) + pw * (n + r + ell1)
    G = sp.csr_matrix((w.ravel(), (rows, cols.ravel())), shape=(npts, pw * pw))
    G.eliminate_zeros()
    return G


class USFFT:
    """Literal restatement of class ``radonusfft`` (radonusfft.cu:5-135)."""

    def __init__(self, n, theta, center):
        self.n = n
        self.theta = np.asarray(theta, dtype=np.float32)
        self.ntheta = self.theta.size
        self.mu, self.r = usfft_params(n)
        self.G = gather_matrix(self.theta, n)
        # set_center (radonusfft.cu:70-75)
        self.shiftfwd = takeshift(-(center - n / 2.0), n)
        self.shiftadj = takeshift(center - n / 2.0, n)
        k = np.arange(n)
        kk = k - n // 2
        phi1 = np.exp(-self.mu * kk * kk)
        # divphi (kernels_radonusfft.cuh:4-24): 1/phi/(4n^2)
        self.deapod = 1.0 / (phi1[:, None] * phi1[None, :]) / (4.0 * n * n)
        pw = 2 * n + 2 * self.r
        X = np.arange(pw)
        # fftshift with flg=1 over the padded grid: (-1)^(x+y) (kernels_radonusfft.cuh:26-38)
        self.mod2 = ((-1.0) ** X)[None, :] * ((-1.0) ** X)[:, None]
        # 1D fftshift: (1-2((tx+1)%2)) = (-1)^(tx+1)
        self.mod1 = -((-1.0) ** k)
        self.scale = 1.0 / np.sqrt(float(n) * float(self.ntheta))

    def _wrap_fwd(self, fde):
        # kernels_radonusfft.cuh:40-64, direction TOMO_FWD: halo <- periodic interior
        n, r = self.n, self.r
        P = 2 * n
        idx = (np.arange(2 * n + 2 * r) - r + P) % P + r
        return fde[:, idx][:, :, idx]

    def _wrap_adj(self, fde):
        # TOMO_ADJ: every halo cell is added into its periodic image in the
        # interior (atomicAdd in the reference); halo values are never read again.
        n, r = self.n, self.r
        P = 2 * n
        pw = 2 * n + 2 * r
        idx = (np.arange(pw) - r + P) % P + r
        tgt = (idx[:, None] * pw + idx[None, :]).ravel()
        out = np.empty_like(fde)
        for z in range(fde.shape[0]):
            v = fde[z].ravel()
            re = np.bincount(tgt, weights=v.real, minlength=pw * pw)
            im = np.bincount(tgt, weights=v.imag, minlength=pw * pw)
            out[z] = (re + 1j * im).reshape(pw, pw)
        return out

    def fwd(self, f):
        """fwdR: complex f[nz, n, n] -> complex g[nz, ntheta, n] (radonusfft.cu:77-104)."""
        n, r = self.n, self.r
        nz = f.shape[0]
        pw = 2 * n + 2 * r
        fde = np.zeros((nz, pw, pw), dtype=np.complex128)
        # divphi FWD
        fde[:, n // 2 + r:n // 2 + r + n, n // 2 + r:n // 2 + r + n] = f * self.deapod[None]
        fde *= self.mod2[None]
        inner = fde[:, r:r + 2 * n, r:r + 2 * n]
        fde[:, r:r + 2 * n, r:r + 2 * n] = np.fft.fft2(inner)  # CUFFT_FORWARD
        fde *= self.mod2[None]
        fde = self._wrap_fwd(fde)
        g = (self.G @ fde.reshape(nz, -1).T).T.reshape(nz, self.ntheta, n)
        g = g * self.shiftfwd[None, None, :]
        g = g * self.mod1
        g = np.fft.ifft(g, axis=-1) * n  # CUFFT_INVERSE (unnormalised)
        g = g * self.mod1
        return g * self.scale

    def adj(self, g):
        """adjR: complex g[nz, ntheta, n] -> complex f[nz, n, n] (radonusfft.cu:106-135)."""
        n, r = self.n, self.r
        nz = g.shape[0]
        pw = 2 * n + 2 * r
        g = g * self.mod1
        g = np.fft.fft(g, axis=-1)  # CUFFT_FORWARD
        g = g * self.mod1
        g = g * self.shiftadj[None, None, :]
        fde = (self.G.T @ g.reshape(nz, -1).T).T.reshape(nz, pw, pw)
        fde = self._wrap_adj(fde)
        fde *= self.mod2[None]
        inner = fde[:, r:r + 2 * n, r:r + 2 * n]
        fde[:, r:r + 2 * n, r:r + 2 * n] = np.fft.ifft2(inner) * (2 * n) ** 2  # CUFFT_INVERSE
        fde *= self.mod2[None]
        f = fde[:, n // 2 + r:n // 2 + r + n, n // 2 + r:n // 2 + r + n] * self.deapod[None]
        return f * self.scale


# ---------------------------------------------------------------------------
# Temporal basis
# ---------------------------------------------------------------------------

def takephi(ntheta, m):
    """Fourier temporal basis used by the reference's test and examples
    (tests/test_adjoint.py:23-27, examples/foam/foam_example.py:17-23):
    float32 [m, 2*ntheta], interleaved (re, im)."""
    x, y = np.meshgrid(np.arange(-ntheta // 2, ntheta // 2), np.arange(-m // 2, m // 2))
    phi = np.zeros([m, 2 * ntheta], dtype="float32")
    phi[:, ::2] = np.cos(2 * np.pi * x * y / ntheta) / np.sqrt(ntheta)
    phi[:, 1::2] = np.sin(2 * np.pi * x * y / ntheta) / np.sqrt(ntheta)
    return phi


def phi_complex(phi):
    phi = np.asarray(phi, dtype=np.float64)
    return phi[:, 0::2] + 1j * phi[:, 1::2]


class Operators:
    """``radonapr``/``radonapradj``/``gradient``/``divergent`` for one chunk of nzp slices."""

    def __init__(self, n, ntheta, m, theta, phi, center):
        self.n, self.ntheta, self.m = n, ntheta, m
        self.R = USFFT(n, theta, center)
        self.phi = phi_complex(phi)  # [m, ntheta]
        # decphi/recphi sample the basis at theta index j*ntheta/m (kernels_operators.cuh:113-114)
        self.tj = (np.arange(m) * ntheta) // m
        # mulphi factor 1/sqrt(M)*Ntheta (kernels_operators.cuh:145-146)
        self.cphi = ntheta / np.sqrt(m)

    def radonapr(self, f, tau=1.0):
        """g = tau*Re(sum_i phi_i(theta) ntheta/sqrt(m) R[sum_j f_j conj(phi_i(t_j))])
        (operators.cu:6-32).  f: [nzp, m, n, n] real -> g [nzp, ntheta, n]."""
        g = np.zeros((f.shape[0], self.ntheta, self.n))
        for i in range(self.m):
            # decphi (kernels_operators.cuh:99-116)
            c = np.einsum("zjyx,j->zyx", f.astype(np.complex128), np.conj(self.phi[i, self.tj]))
            gt = self.R.fwd(c)
            # mulphi c=+1 (kernels_operators.cuh:135-149)
            gt = gt * self.cphi * self.phi[i][None, :, None]
            g += tau * gt.real  # addreal
        return g

    def radonapradj(self, g, tau=1.0):
        """f_incr = tau*Re(sum_i phi_i(t_j) R^*[conj(phi_i(theta)) ntheta/sqrt(m) g])
        (operators.cu:34-58).  g: [nzp, ntheta, n] -> [nzp, m, n, n]."""
        acc = np.zeros((g.shape[0], self.m, self.n, self.n), dtype=np.complex128)
        for i in range(self.m):
            gt = g.astype(np.complex128) * self.cphi * np.conj(self.phi[i])[None, :, None]
            c = self.R.adj(gt)
            acc += c[:, None, :, :] * self.phi[i, self.tj][None, :, None, None]  # recphi
        return tau * acc.real


def extendf(fm, flgl, flgr):
    """extendf (kernels_operators.cuh:4-20).  fm: chunk with halo, shape [nzp+2, m, n, n]
    (slab 0 and nzp+1 are the halo slabs).  Returns fe [nzp+2, m+2, n+2, n+2]."""
    nzp = fm.shape[0] - 2
    m, n = fm.shape[1], fm.shape[2]
    ix = np.clip(np.arange(n + 2) - 1, 0, n - 1)
    it = np.clip(np.arange(m + 2) - 1, 0, m - 1)
    iz = np.clip(np.arange(nzp + 2) - 1, -flgl, nzp - 1 + flgr) + 1  # +1: halo slab offset
    return fm[iz][:, it][:, :, ix][:, :, :, ix]


def grad_scale(lambda1):
    """Forward differences are divided by 2/cbrt(2)/(lambda1/2) (kernels_operators.cuh:40-43)."""
    return 1.0 / (2.0 * np.cbrt(2.0) * (lambda1 / 2.0))


def gradient(fm, lambda1, flgl, flgr):
    """gradf (kernels_operators.cuh:22-44) on extendf's grid.

    Returns h [nzp+1, m+1, n+1, n+1, 4] (components x, y, lambda1*t, z)."""
    fe = extendf(fm, flgl, flgr)
    s = grad_scale(lambda1)
    b = fe[:-1, :-1, :-1, :-1]
    h = np.empty(b.shape + (4,))
    h[..., 0] = (fe[:-1, :-1, :-1, 1:] - b) * s
    h[..., 1] = (fe[:-1, :-1, 1:, :-1] - b) * s
    h[..., 2] = (fe[:-1, 1:, :-1, :-1] - b) * s * lambda1
    h[..., 3] = (fe[1:, :-1, :-1, :-1] - b) * s
    return h


def divergent(h, lambda1, tau):
    """div (kernels_operators.cuh:46-73): increment tau*(h[i-1]-h[i])/(4 cbrt2 lambda1/2).

    h: [nzp+1, m+1, n+1, n+1, 4] -> increment [nzp, m, n, n].  This equals
    tau/2 times the transpose of ``gradient`` on the grid points it reads."""
    s = 1.0 / (4.0 * np.cbrt(2.0) * (lambda1 / 2.0))
    c = h[1:, 1:, 1:, 1:]
    out = (h[1:, 1:, 1:, :-1, 0] - c[..., 0]) * s
    out = out + (h[1:, 1:, :-1, 1:, 1] - c[..., 1]) * s
    out = out + (h[1:, :-1, 1:, 1:, 2] - c[..., 2]) * s * lambda1
    out = out + (h[:-1, 1:, 1:, 1:, 3] - c[..., 3]) * s
    return tau * out


def solve_reg(h2, mu, lambda0, rho):
    """solve_reg_ker (admm.cu:40-72): isotropic soft threshold of h2+mu/rho."""
    psi = h2 + mu / rho
    za = np.sqrt(np.sum(psi * psi, axis=-1, keepdims=True))
    thr = lambda0 / rho
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where(za <= thr, 0.0, psi - thr * psi / za)
    return out


# ---------------------------------------------------------------------------
# ADMM driver
# ---------------------------------------------------------------------------

def solver_admm(ops, fm, g, psi, mu, lambda0, lambda1, rho, flgl, flgr, titer):
    """rectv::solver_admm (admm.cu:74-122) on one chunk.

    fm: [nzp+2, m, n, n] chunk with halo slabs (modified in place on the
    interior); g: [nzp, ntheta, n]; psi, mu: [nzp+1, m+1, n+1, n+1, 4]
    (modified in place).  Returns (||h2-psi||, ||G fm0 - G fm||) as float64."""
    inner = slice(1, fm.shape[0] - 1)
    h2stored = gradient(fm, lambda1, flgl, flgr)
    for _ in range(titer):
        h2 = gradient(fm, lambda1, flgl, flgr)
        h1 = ops.radonapr(fm[inner], 1.0)
        h2 = rho * (h2 - psi) + mu
        h1 = h1 - g
        fm[inner] += divergent(h2, lambda1, -0.5)
        fm[inner] += ops.radonapradj(h1, -0.5)
    h2 = gradient(fm, lambda1, flgl, flgr)
    psi[...] = solve_reg(h2, mu, lambda0, rho)
    mu[...] = mu + rho * h2 - rho * psi
    h2stored = h2stored - h2
    h2 = h2 - psi
    return np.sqrt(np.sum(h2 * h2)), np.sqrt(np.sum(h2stored * h2stored))


def run(data, theta, phi, center, lambda0, lambda1, niter, titer, nzp, return_history=False,
        callback=None, init=None):
    """rectv::run (rectv.cu:102-252) with the wrapper's conventions applied by the caller.

    ``lambda0`` here is the value passed to ``run`` (Solver.recon multiplies
    the user's lambda0 by lambda1 first, solver.py:76).
    data: [nz, ntheta, n] float32; returns f [nz, m, n, n] (float64).
    Slices beyond (nz//nzp)*nzp are never touched (zero), as in the reference.
    """
    data = np.asarray(data, dtype=np.float64)
    nz, ntheta, n = data.shape
    phi = np.asarray(phi)
    m = phi.shape[0]
    nchunks = nz // nzp
    ops = Operators(n, ntheta, m, theta, phi, center)
    f = np.zeros((nz, m, n, n))
    if init is not None:  # extension: warm start instead of rectv.cu:119-120's zero
        nzc = nchunks * nzp
        f[:nzc] = np.asarray(init, dtype=np.float64)[:nzc]
    fn = np.zeros((nz, m, n, n))
    gp = (nzp + 1, m + 1, n + 1, n + 1, 4)
    psi = [np.zeros(gp) for _ in range(nchunks)]
    mu = [np.zeros(gp) for _ in range(nchunks)]
    rho = 0.5
    history = []
    for it in range(niter):
        nd = []
        for iz in range(nchunks):
            z0 = iz * nzp
            flgl = int(iz != 0)
            flgr = int(iz != nchunks - 1)
            fm = np.zeros((nzp + 2, m, n, n))
            fm[1:nzp + 1] = f[z0:z0 + nzp]
            if flgl:
                fm[0] = f[z0 - 1]
            if flgr:
                fm[nzp + 1] = f[z0 + nzp]
            nd.append(solver_admm(ops, fm, data[z0:z0 + nzp], psi[iz], mu[iz],
                                  lambda0, lambda1, rho, flgl, flgr, titer))
            fn[z0:z0 + nzp] = fm[1:nzp + 1]
        # rho rule (rectv.cu:223-232)
        r = sum(a * a for a, _ in nd)
        s = sum(rho * rho * b * b for _, b in nd)
        if r > 10 * s:
            rho *= 2
        elif s > 10 * r:
            rho *= 0.5
        norm = float(np.sum((fn - f) ** 2))  # rectv.cu:235-238
        history.append({"iter": it, "rdiff": norm, "rho": rho, "r": r, "s": s})
        f, fn = fn, f
        if callback is not None:
            callback(it, f)
    if return_history:
        return f, history
    return f


def check_adjoints(data, theta, phi, lambda1, center):
    """rectv::check_adjoints (rectv.cu:255-290) for one chunk (nz == nzp).

    Returns the six sums exactly as the reference defines them, including
    res[4], which sums the squares of only the first (n+1)^2(m+1)(nz+1)
    floats of the float4 gradient array (rectv.cu:283-287)."""
    data = np.asarray(data, dtype=np.float64)
    nz, ntheta, n = data.shape
    m = np.asarray(phi).shape[0]
    ops = Operators(n, ntheta, m, theta, phi, center)
    f = ops.radonapradj(data, 1.0)
    h1 = ops.radonapr(f, 1.0)
    res = np.zeros(6)
    res[0] = np.sum(f * f)
    res[1] = np.sum(data * h1)
    res[2] = np.sum(h1 * h1)
    fm = np.zeros((nz + 2, m, n, n))
    fm[1:nz + 1] = f
    h2 = gradient(fm, lambda1, 0, 0)
    fn = divergent(h2, lambda1, 1.0)
    res[3] = np.sum(f * fn)
    npts = (n + 1) * (n + 1) * (m + 1) * (nz + 1)
    res[4] = np.sum(h2.ravel()[:npts] ** 2)
    res[5] = np.sum(fn * fn)
    return res


# ---------------------------------------------------------------------------
# Data ingest (the step before the path)
# ---------------------------------------------------------------------------

def preprocess(data, dark, flat):
    """Flat/dark normalisation, -log and projection -> sinogram transpose of
    the reference's tao example (examples/tao/tao.py:41), in float64."""
    data = np.asarray(data, dtype=np.float64)
    dm = np.mean(np.asarray(dark, dtype=np.float64), axis=0)
    fm = np.mean(np.asarray(flat, dtype=np.float64), axis=0)
    with np.errstate(invalid="ignore", divide="ignore"):
        return -np.log((data - dm) / (1e-3 + fm - dm)).swapaxes(0, 1)


# ---------------------------------------------------------------------------
# Filtered backprojection with the reference's unused filter and mask
# ---------------------------------------------------------------------------

def fbp(data, theta, center):
    """circ(pi/4 * adjR(applyfilter(g))) per slice: adjR (radonusfft.cu:
    106-135) with applyfilter (kernels_radonusfft.cuh:173-189) applied to the
    centred row spectrum right after the row FFT's fftshift, and circ with
    r = 0 (kernels_radonusfft.cuh:146-159).  data [nz, ntheta, n] ->
    [nz, n, n] float64."""
    data = np.asarray(data, dtype=np.float64)
    nz, ntheta, n = data.shape
    R = USFFT(n, theta, center)
    k = np.arange(n)
    rho = (k - n // 2) / float(n)
    with np.errstate(invalid="ignore", divide="ignore"):
        w = np.where(rho == 0, 0.0, np.abs(rho) * n * 4 * np.sin(rho) / rho)
    g = data.astype(np.complex128) * R.mod1
    g = np.fft.fft(g, axis=-1) * R.mod1 * w
    g = np.fft.ifft(g * R.mod1, axis=-1) * R.mod1  # back to s; adj transforms again
    f = R.adj(g).real * (PI_USFFT / 4)
    x = (np.arange(n) - n // 2) / float(n)
    mask = (4 * x[None, :] ** 2 + 4 * x[:, None] ** 2) < 1
    return f * mask[None]
