"""FP64 PyTorch transcription of the NumPy oracle (oracle/rectv_oracle.py).

TEST INFRASTRUCTURE ONLY.  Like the NumPy oracle this module is the checker:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s accuracy and
CPU-baseline legs may import it.  The product path (``rectv_gpu_gb300``) never
calls it.

It computes the same float64 arithmetic as the NumPy restatement, step by step
(one fwdR/adjR per basis function, explicit fftshift modulations, the gather
as a sparse matrix with the reference's index formula), with torch tensors so
that it runs on a GPU in float64 for problem sizes where the NumPy oracle
would take hours (n = 512 ... 1024 with thousands of angles).  The
transcription is checked against the NumPy oracle to 1e-12 on the CPU
(tests/test_oracle_torch.py).  Citations are ``file:line`` inside the
reference project (nikitinvv/rectv_gpu):

* ``radonusfft::fwdR`` / ``adjR`` (src/cuda/radonusfft.cu:77-135; kernels
  divphi, fftshift, wrap, gather, shift, mulr in
  src/include/kernels_radonusfft.cuh:4-215)
* ``rectv::radonapr`` / ``radonapradj`` (src/cuda/operators.cu:6-58; decphi,
  recphi, mulphi, addreal in src/include/kernels_operators.cuh:75-149)
* ``rectv::gradient`` / ``divergent`` (src/cuda/operators.cu:60-71;
  extendf, gradf, div in src/include/kernels_operators.cuh:4-73)
* ``rectv::solver_admm`` (src/cuda/admm.cu:74-122, solve_reg_ker admm.cu:40-72)
* ``rectv::run`` (src/cuda/rectv.cu:102-252): chunks with a one-slice z-halo
  from the previous iterate, the rho rule (rectv.cu:223-232)

One difference in form, not in value: the reference (and the NumPy oracle)
copies the periodic interior of the 2n x 2n spectrum into a halo of width r
before the gather (wrap, TOMO_FWD) and folds the halo back after the scatter
(wrap, TOMO_ADJ).  Here the gather matrix indexes the periodic grid directly
(column (n + l) mod 2n for stencil offset l), which is the same linear map.
"""

import warnings

import numpy as np
import torch

from oracle import rectv_oracle as orc

PI_USFFT = orc.PI_USFFT
F64 = torch.float64
C128 = torch.complex128

warnings.filterwarnings("ignore", message="Sparse CSR tensor support is in beta")
warnings.filterwarnings("ignore", message="Sparse invariant checks are implicitly disabled")


def _t(a, device, dtype=F64):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=device)


def gather_csr(theta, n, device, chunk=1 << 22):
    """Gather matrix of kernels_radonusfft.cuh:81-144 on the periodic 2n x 2n
    grid, as CSR (rows: polar samples theta-major, 81 taps each; the rows of
    the k = 0 samples hold zeros) and its transpose, both float64.

    Positions come from orc.takexy (float64 sin/cos of the float32 angles,
    x clamped below 0.5), the stencil origin floor(2n x) - 4, weights
    pi/mu exp(-pi^2/mu (w0^2 + w1^2)) / n."""
    mu, r = orc.usfft_params(n)
    P = 2 * n
    taps = 2 * r + 1
    x, y = orc.takexy(theta, n)
    x = _t(x.ravel(), device)
    y = _t(y.ravel(), device)
    npts = x.numel()
    kk = torch.arange(npts, device=device) % n
    d = torch.arange(taps, device=device)
    cols_all, vals_all = [], []
    for s in range(0, npts, chunk):
        xs, ys = x[s:s + chunk], y[s:s + chunk]
        fx = torch.floor(2 * n * xs).to(torch.int64)
        fy = torch.floor(2 * n * ys).to(torch.int64)
        ell0 = fx[:, None, None] - r + d[None, None, :]   # x offset (inner)
        ell1 = fy[:, None, None] - r + d[None, :, None]   # y offset (outer)
        w0 = ell0.to(F64) / float(2 * n) - xs[:, None, None]
        w1 = ell1.to(F64) / float(2 * n) - ys[:, None, None]
        w = PI_USFFT / mu * torch.exp(-PI_USFFT * PI_USFFT / mu * (w0 * w0 + w1 * w1)) / n
        w = w * (kk[s:s + chunk] != 0).to(F64)[:, None, None]
        cols = torch.remainder(n + ell0, P) + P * torch.remainder(n + ell1, P)
        cols = cols.reshape(-1, taps * taps)
        w = w.reshape(-1, taps * taps)
        cols, order = torch.sort(cols, dim=1)
        cols_all.append(cols)
        vals_all.append(torch.gather(w, 1, order))
    cols = torch.cat(cols_all).reshape(-1)
    vals = torch.cat(vals_all).reshape(-1)
    nnz = vals.numel()
    itype = torch.int32 if nnz < 2 ** 31 - 1 else torch.int64
    crow = torch.arange(0, nnz + 1, taps * taps, device=device, dtype=itype)
    G = torch.sparse_csr_tensor(crow, cols.to(itype), vals, size=(npts, P * P), check_invariants=False)
    rows = torch.arange(npts, device=device, dtype=torch.int64).repeat_interleave(taps * taps)
    coo = torch.sparse_coo_tensor(torch.stack([cols, rows]), vals, size=(P * P, npts)).coalesce()
    del rows, cols, vals
    GT = coo.to_sparse_csr()
    if itype == torch.int32:
        GT = torch.sparse_csr_tensor(GT.crow_indices().to(itype), GT.col_indices().to(itype), GT.values(),
                                     size=GT.shape, check_invariants=False)
    return G, GT


def _spmm(A, z):
    """A (real CSR) @ z for complex z [ncols_of_A, batch] -> complex [nrows, batch]."""
    zr = torch.view_as_real(z).reshape(z.shape[0], -1)
    out = torch.sparse.mm(A, zr)
    return torch.view_as_complex(out.reshape(out.shape[0], -1, 2).contiguous())


class USFFT:
    """radonusfft (radonusfft.cu:5-135) in float64 on `device`."""

    def __init__(self, n, theta, center, device="cpu"):
        self.n = n
        self.device = torch.device(device)
        self.theta = np.asarray(theta, dtype=np.float32)
        self.ntheta = self.theta.size
        self.mu, self.r = orc.usfft_params(n)
        P = 2 * n
        self.P = P
        self.G, self.GT = gather_csr(self.theta, n, self.device)
        # set_center (radonusfft.cu:70-75)
        self.shiftfwd = _t(orc.takeshift(-(center - n / 2.0), n), self.device, C128)
        self.shiftadj = _t(orc.takeshift(center - n / 2.0, n), self.device, C128)
        kk = np.arange(n) - n // 2
        phi1 = np.exp(-self.mu * kk * kk)
        # divphi (kernels_radonusfft.cuh:4-24): 1/phi/(4n^2)
        self.deapod = _t(1.0 / (phi1[:, None] * phi1[None, :]) / (4.0 * n * n), self.device)
        # fftshift flg=1 over the padded grid, X = inner index + r (kernels_radonusfft.cuh:26-38)
        X = np.arange(P) + self.r
        self.mod2 = _t(((-1.0) ** X)[None, :] * ((-1.0) ** X)[:, None], self.device)
        # 1D fftshift (-1)^(k+1)
        self.mod1 = _t(-((-1.0) ** np.arange(n)), self.device)
        self.scale = 1.0 / np.sqrt(float(n) * float(self.ntheta))

    def fwd(self, f):
        """fwdR: complex f [b, n, n] -> complex g [b, ntheta, n] (radonusfft.cu:77-104)."""
        n, P = self.n, self.P
        b = f.shape[0]
        fde = torch.zeros((b, P, P), dtype=C128, device=self.device)
        fde[:, n // 2:n // 2 + n, n // 2:n // 2 + n] = f * self.deapod
        fde *= self.mod2
        fde = torch.fft.fft2(fde)
        fde *= self.mod2
        z = fde.permute(1, 2, 0).reshape(P * P, b)
        del fde
        g = _spmm(self.G, z).reshape(self.ntheta, n, b).permute(2, 0, 1)
        g = g * self.shiftfwd * self.mod1
        g = torch.fft.ifft(g, dim=-1) * n
        g = g * self.mod1
        return g * self.scale

    def adj(self, g):
        """adjR: complex g [b, ntheta, n] -> complex f [b, n, n] (radonusfft.cu:106-135)."""
        n, P = self.n, self.P
        b = g.shape[0]
        g = g * self.mod1
        g = torch.fft.fft(g, dim=-1)
        g = g * self.mod1 * self.shiftadj
        z = g.permute(1, 2, 0).reshape(self.ntheta * n, b)
        fde = _spmm(self.GT, z).reshape(P, P, b).permute(2, 0, 1)
        fde = fde * self.mod2
        fde = torch.fft.ifft2(fde) * float(P * P)
        fde *= self.mod2
        f = fde[:, n // 2:n // 2 + n, n // 2:n // 2 + n] * self.deapod
        return f * self.scale


class Operators:
    """radonapr / radonapradj (operators.cu:6-58) for nzp slices, float64 on `device`."""

    def __init__(self, n, ntheta, m, theta, phi, center, device="cpu", basis_batch=None):
        self.n, self.ntheta, self.m = n, ntheta, m
        self.device = torch.device(device)
        self.R = USFFT(n, theta, center, device)
        self.phi = _t(orc.phi_complex(phi), self.device, C128)   # [m, ntheta]
        self.tj = torch.as_tensor((np.arange(m) * ntheta) // m, device=self.device)
        self.phit = self.phi[:, self.tj]                            # phi_i(t_j) [i, j]
        self.cphi = ntheta / np.sqrt(m)
        self.bb = basis_batch or m   # basis functions per batched fwdR/adjR call

    def radonapr(self, f, tau=1.0):
        """g = tau Re sum_i phi_i(theta) ntheta/sqrt(m) R[sum_j f_j conj(phi_i(t_j))]."""
        nzp = f.shape[0]
        g = torch.zeros((nzp, self.ntheta, self.n), dtype=F64, device=self.device)
        fc = f.to(C128)
        for i0 in range(0, self.m, self.bb):
            ib = slice(i0, min(self.m, i0 + self.bb))
            # decphi (kernels_operators.cuh:99-116), a batch of basis functions
            c = torch.einsum("zjyx,ij->izyx", fc, torch.conj(self.phit[ib]))
            nb = c.shape[0]
            gt = self.R.fwd(c.reshape(nb * nzp, self.n, self.n)).reshape(nb, nzp, self.ntheta, self.n)
            # mulphi c=+1 (kernels_operators.cuh:135-149), addreal (kernels_operators.cuh:75-84)
            gt = gt * self.cphi * self.phi[ib][:, None, :, None]
            g += tau * gt.real.sum(dim=0)
        return g

    def radonapradj(self, g, tau=1.0):
        """tau Re sum_i phi_i(t_j) R^*[conj(phi_i(theta)) ntheta/sqrt(m) g]."""
        nzp = g.shape[0]
        acc = torch.zeros((nzp, self.m, self.n, self.n), dtype=C128, device=self.device)
        gc = g.to(C128)
        for i0 in range(0, self.m, self.bb):
            ib = slice(i0, min(self.m, i0 + self.bb))
            gt = gc[None] * self.cphi * torch.conj(self.phi[ib])[:, None, :, None]
            nb = gt.shape[0]
            c = self.R.adj(gt.reshape(nb * nzp, self.ntheta, self.n)).reshape(nb, nzp, self.n, self.n)
            # recphi (kernels_operators.cuh:118-133)
            acc += torch.einsum("izyx,ij->zjyx", c, self.phit[ib])
        return tau * acc.real


def extendf(fm, flgl, flgr):
    """extendf (kernels_operators.cuh:4-20): fm [nzp+2, m, n, n] -> fe [nzp+2, m+2, n+2, n+2]."""
    nzp = fm.shape[0] - 2
    m, n = fm.shape[1], fm.shape[2]
    dev = fm.device
    ix = torch.clamp(torch.arange(n + 2, device=dev) - 1, 0, n - 1)
    it = torch.clamp(torch.arange(m + 2, device=dev) - 1, 0, m - 1)
    iz = torch.clamp(torch.arange(nzp + 2, device=dev) - 1, -flgl, nzp - 1 + flgr) + 1
    return fm[iz][:, it][:, :, ix][:, :, :, ix]


def gradient(fm, lambda1, flgl, flgr):
    """gradf (kernels_operators.cuh:22-44): h [nzp+1, m+1, n+1, n+1, 4]."""
    fe = extendf(fm, flgl, flgr)
    s = orc.grad_scale(lambda1)
    b = fe[:-1, :-1, :-1, :-1]
    return torch.stack([(fe[:-1, :-1, :-1, 1:] - b) * s,
                        (fe[:-1, :-1, 1:, :-1] - b) * s,
                        (fe[:-1, 1:, :-1, :-1] - b) * s * lambda1,
                        (fe[1:, :-1, :-1, :-1] - b) * s], dim=-1)


def divergent(h, lambda1, tau):
    """div (kernels_operators.cuh:46-73): h -> increment [nzp, m, n, n]."""
    s = 1.0 / (4.0 * np.cbrt(2.0) * (lambda1 / 2.0))
    c = h[1:, 1:, 1:, 1:]
    out = (h[1:, 1:, 1:, :-1, 0] - c[..., 0]) * s
    out = out + (h[1:, 1:, :-1, 1:, 1] - c[..., 1]) * s
    out = out + (h[1:, :-1, 1:, 1:, 2] - c[..., 2]) * s * lambda1
    out = out + (h[:-1, 1:, 1:, 1:, 3] - c[..., 3]) * s
    return tau * out


def solve_reg(h2, mu, lambda0, rho):
    """solve_reg_ker (admm.cu:40-72)."""
    psi = h2 + mu / rho
    za = torch.sqrt(torch.sum(psi * psi, dim=-1, keepdim=True))
    thr = lambda0 / rho
    shrunk = psi - thr * psi / torch.where(za > 0, za, torch.ones_like(za))
    return torch.where(za <= thr, torch.zeros_like(psi), shrunk)


def solver_admm(ops, fm, g, psi, mu, lambda0, lambda1, rho, flgl, flgr, titer):
    """rectv::solver_admm (admm.cu:74-122) on one chunk; fm, psi, mu updated in place."""
    inner = slice(1, fm.shape[0] - 1)
    h2stored = gradient(fm, lambda1, flgl, flgr)
    for _ in range(titer):
        h2 = gradient(fm, lambda1, flgl, flgr)
        h1 = ops.radonapr(fm[inner], 1.0)
        h2 = rho * (h2 - psi) + mu
        h1 = h1 - g
        fm[inner] += divergent(h2, lambda1, -0.5)
        del h2
        fm[inner] += ops.radonapradj(h1, -0.5)
    h2 = gradient(fm, lambda1, flgl, flgr)
    psi.copy_(solve_reg(h2, mu, lambda0, rho))
    mu.copy_(mu + rho * h2 - rho * psi)
    h2stored = h2stored - h2
    h2 = h2 - psi
    return float(torch.sqrt(torch.sum(h2 * h2))), float(torch.sqrt(torch.sum(h2stored * h2stored)))


def run(data, theta, phi, center, lambda0, lambda1, niter, titer, nzp, device="cpu", return_history=False,
        callback=None, rho_sequence=None, basis_batch=None):
    """rectv::run (rectv.cu:102-252), as orc.run, in float64 on `device`.

    rho_sequence: optional rho after each outer iteration to follow instead
    of the rule's own choice (the rule's choice is still recorded as
    "rho_rule"), so that a reconstruction can be compared iteration by
    iteration with another one's rho sequence.  callback(it, f) sees the
    iterate (a float64 tensor on `device`) after every outer iteration.
    Returns f [nz, m, n, n] as a float64 NumPy array."""
    dev = torch.device(device)
    data = torch.as_tensor(np.asarray(data), dtype=F64, device=dev)
    nz, ntheta, n = data.shape
    m = np.asarray(phi).shape[0]
    nchunks = nz // nzp
    ops = Operators(n, ntheta, m, theta, phi, center, dev, basis_batch)
    f = torch.zeros((nz, m, n, n), dtype=F64, device=dev)
    fn = torch.zeros_like(f)
    gp = (nzp + 1, m + 1, n + 1, n + 1, 4)
    psi = [torch.zeros(gp, dtype=F64, device=dev) for _ in range(nchunks)]
    mu = [torch.zeros(gp, dtype=F64, device=dev) for _ in range(nchunks)]
    rho = 0.5
    history = []
    for it in range(niter):
        nd = []
        for iz in range(nchunks):
            z0 = iz * nzp
            flgl = int(iz != 0)
            flgr = int(iz != nchunks - 1)
            fm = torch.zeros((nzp + 2, m, n, n), dtype=F64, device=dev)
            fm[1:nzp + 1] = f[z0:z0 + nzp]
            if flgl:
                fm[0] = f[z0 - 1]
            if flgr:
                fm[nzp + 1] = f[z0 + nzp]
            nd.append(solver_admm(ops, fm, data[z0:z0 + nzp], psi[iz], mu[iz], lambda0, lambda1, rho, flgl, flgr,
                                  titer))
            fn[z0:z0 + nzp] = fm[1:nzp + 1]
            del fm
        r = sum(a * a for a, _ in nd)
        s = sum(rho * rho * b * b for _, b in nd)
        rule = rho
        if r > 10 * s:
            rule = rho * 2
        elif s > 10 * r:
            rule = rho * 0.5
        rho = float(rho_sequence[it]) if rho_sequence is not None else rule
        norm = float(torch.sum((fn - f) ** 2))
        history.append({"iter": it, "rdiff": norm, "rho": rho, "rho_rule": rule, "r": r, "s": s})
        f, fn = fn, f
        if callback is not None:
            callback(it, f)
    out = f.cpu().numpy()
    if return_history:
        return out, history
    return out
