"""GPU tests of the filtered backprojection (the reference's unused
applyfilter/circ kernels and adjR filter flag) and of the warm start."""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import scan_angles

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Solver(lib_built, torch_cuda):
    from rectv_gpu_gb300 import Solver
    return Solver


@pytest.mark.parametrize("case", [(64, 180, 4, 2, 0.0), (48, 100, 3, 3, 2.5), (36, 64, 5, 1, -1.0)])
def test_fbp_matches_oracle(Solver, case):
    n, ntheta, nz, nzp, dc = case
    theta = scan_angles(ntheta, 2)
    g = np.random.default_rng(3).standard_normal((nz, ntheta, n)).astype(np.float32)
    ref = orc.fbp(g, theta, n / 2 + dc)
    with Solver(n, ntheta, 4, nz, nzp, 1) as s:
        got = s.fbp(g, theta, rot_center=n / 2 + dc)
    assert got.shape == (nz, n, n)
    assert rel(got, ref) < 2e-5


def test_fbp_reconstructs_a_static_object(Solver):
    """FBP(R u) ~ u for a smooth zero-mean object (the filter's w(0)=0 drops the mean)."""
    n, ntheta = 128, 720
    theta = scan_angles(ntheta, 4)
    xx = np.arange(n) - n // 2
    img = np.exp(-((xx[None, :] - 10) ** 2 + (xx[:, None] + 6) ** 2) / (2 * 8.0 ** 2))
    img -= img.mean()
    U = orc.USFFT(n, theta, n / 2)
    g = U.fwd(img[None].astype(complex)).real.astype(np.float32)
    with Solver(n, ntheta, 2, 1, 1, 1) as s:
        rec = s.fbp(g, theta)[0]
    mask = (4 * (xx[None, :] / n) ** 2 + 4 * (xx[:, None] / n) ** 2) < 1
    assert rel(rec * mask, img * mask) < 0.1


def test_warm_start_matches_oracle(Solver):
    n, ntheta, m, nz, nzp = 32, 64, 4, 4, 2
    theta = scan_angles(ntheta, 4)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(4)
    g = rng.random((nz, ntheta, n)).astype(np.float32)
    init = rng.random((nz, m, n, n)).astype(np.float32)
    ref = orc.run(g, theta, phi, n / 2, 1e-3 * 2.0, 2.0, 2, 2, nzp, init=init)
    with Solver(n, ntheta, m, nz, nzp, 1) as s:
        s.set_verbose(False)
        got = s.recon(g, theta, phi, lambda0=1e-3, lambda1=2.0, niter=2, titer=2, init=init)
        fb = s.recon(g, theta, phi, lambda0=1e-3, lambda1=2.0, niter=1, titer=1, init="fbp")
    assert rel(got, ref) < 1e-4
    assert np.isfinite(fb).all() and np.linalg.norm(fb) > 0
