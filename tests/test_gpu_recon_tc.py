"""Reconstruction parity of the production path against the FP64 oracle.

With more than 8 time samples the solver mixes the time samples on the
tensor cores (k_gather_tc, k_scatter_tc, 3xTF32 with FP32 accumulation); with
2n a power of two in [256, 2048] the padded-grid 2D FFTs are the hand-written
ones (k_fft_rows_fwd, k_fft_cols, k_fft_rows_inv); with n a power of two in
[256, 1024] the inner residual runs through k_resid_rows; the TV steps are
k_graddiv in its w-mode (titer > 1) and k_shrink.  These are the kernels of
the benchmark workload, so the reconstructions below run all of them for
several outer iterations and compare with the FP64 restatement of
rectv::run (rectv.cu:102-252, admm.cu:74-122) on the same seeded inputs, with
the same rho sequence.

Tolerance: 1e-4 relative L2 for the reconstruction (the metric's bar).
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

pytestmark = pytest.mark.gpu

REC_TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(autouse=True)
def per_ray_path(monkeypatch):
    """These cases revisit their directions; keep them on the per-ray tensor-core kernels."""
    monkeypatch.setenv("RECTV_DIRS", "0")


@pytest.fixture(scope="module")
def Solver(lib_built, torch_cuda):
    from rectv_gpu_gb300 import Solver
    return Solver


def _problem(n, ntheta, m, nz, nrot, seed=0):
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=seed)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    g = add_noise(ops.radonapr(u.astype(np.float64)), 0.01, seed)
    return theta, phi, g


@pytest.mark.parametrize("case", [
    # n, ntheta, m, nz, nzp, nrot, niter, titer
    (64, 128, 16, 4, 2, 4, 6, 4),    # tensor-core gather and scatter, cuFFT padded grid, two chunks
    (128, 192, 16, 2, 2, 4, 4, 4),   # + hand-written padded-grid FFTs (2n = 256)
    (64, 96, 12, 3, 1, 2, 4, 3),     # 12 time samples (zero-padded to 16 on the tensor cores), three chunks
])
def test_tc_recon_matches_oracle(Solver, case):
    n, ntheta, m, nz, nzp, nrot, niter, titer = case
    lam0, lam1 = 1e-3, 4.0
    theta, phi, g = _problem(n, ntheta, m, nz, nrot)
    ref, hist = orc.run(g, theta, phi, n / 2, lam0 * lam1, lam1, niter, titer, nzp, return_history=True)
    with Solver(n, ntheta, m, nz, nzp, 1) as slv:
        slv.set_verbose(False)
        got = slv.recon(g, theta, phi, lambda0=lam0, lambda1=lam1, niter=niter, titer=titer)
        h = slv.history()
    err = rel(got, ref)
    assert err < REC_TOL, err
    assert np.allclose(h["rho"], [x["rho"] for x in hist])
    np.testing.assert_allclose(h["rdiff"], [x["rdiff"] for x in hist], rtol=1e-3)
