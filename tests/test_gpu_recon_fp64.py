"""Reconstructions of the production path against the FP64 oracle at sizes
where the NumPy oracle would take hours: the FP64 PyTorch transcription of the
oracle (oracle/rectv_oracle_torch.py, checked against the NumPy oracle to
1e-12 in tests/test_oracle_torch.py) runs on the GPU in float64.

* n=256 (2n = 512): every kernel of the benchmark workload (tensor-core
  gather and scatter, hand-written padded-grid FFTs, fused residual rows,
  k_graddiv w-mode, k_shrink), two chunks with the z-halo, 8 outer iterations;
* config 2 of the benchmark plan: N=512, Nz=32, Nzp=8, Ntheta=1440 over 8
  half-turns, M=16, 64 ADMM iterations (titer=4), the seeded 10-ellipsoid
  phantom forward-projected in FP64 plus 1% Gaussian noise.

Tolerance: 1e-4 relative L2 against the FP64 reconstruction at every outer
iteration, and the same rho sequence (the rule's decisions).
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

pytestmark = pytest.mark.gpu

REC_TOL = 1e-4


@pytest.fixture(scope="module")
def env(lib_built, torch_cuda):
    from oracle import rectv_oracle_torch as ort
    from rectv_gpu_gb300 import rectv
    return torch_cuda, ort, rectv


def _compare(torch, ort, rectv, g, theta, phi, n, m, nz, nzp, niter, titer, lam0=1e-3, lam1=4.0):
    """Runs the GPU reconstruction (device session API) in lockstep with the
    FP64 oracle on the GPU; returns the relative error of the GPU iterate
    after every outer iteration, the GPU history and the FP64 history."""
    ntheta = theta.size
    dev = torch.device("cuda")
    obj = rectv(n, ntheta, m, nz, nzp, 1)
    obj.set_verbose(False)
    dg = torch.from_numpy(np.ascontiguousarray(g, dtype=np.float32)).to(dev)
    dth = torch.from_numpy(theta).to(dev)
    dph = torch.from_numpy(phi).to(dev)
    out = torch.empty((nz, m, n, n), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    obj.setup_device(dg.data_ptr(), dth.data_ptr(), dph.data_ptr(), n / 2, lam0 * lam1, lam1, titer)
    errs = []

    def step(it, f):
        obj.iterate(1)
        obj.result_device(out.data_ptr())
        obj.synchronize()
        a = out.to(torch.float64)
        errs.append(float(torch.linalg.vector_norm(a - f) / torch.linalg.vector_norm(f)))

    try:
        _, h64 = ort.run(g, theta, phi, n / 2, lam0 * lam1, lam1, niter, titer, nzp, device="cuda",
                         return_history=True, callback=step)
        hist = obj.history()
    finally:
        obj.free()
    return errs, hist, h64


def test_production_kernels_match_fp64(env):
    torch, ort, rectv = env
    n, ntheta, m, nz, nzp, nrot, niter, titer = 256, 360, 16, 4, 2, 8, 8, 4
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=4)
    ops = ort.Operators(n, ntheta, m, theta, phi, n / 2, device="cuda")
    g = add_noise(ops.radonapr(torch.from_numpy(u.astype(np.float64)).cuda()).cpu().numpy(), 0.01, 4)
    errs, hist, h64 = _compare(torch, ort, rectv, g, theta, phi, n, m, nz, nzp, niter, titer)
    assert max(errs) < REC_TOL, errs
    assert list(hist["rho"]) == [x["rho"] for x in h64]


def test_config2_matches_fp64(env):
    torch, ort, rectv = env
    n, ntheta, m, nz, nzp, nrot, niter, titer = 512, 1440, 16, 32, 8, 8, 64, 4
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=0)
    ops = ort.Operators(n, ntheta, m, theta, phi, n / 2, device="cuda")
    g = np.concatenate([ops.radonapr(torch.from_numpy(u[z:z + 8].astype(np.float64)).cuda()).cpu().numpy()
                        for z in range(0, nz, 8)])
    del ops
    g = add_noise(g, 0.01, 0)
    errs, hist, h64 = _compare(torch, ort, rectv, g, theta, phi, n, m, nz, nzp, niter, titer)
    print("config 2: relative error vs FP64 per iteration: first %.2e, max %.2e, last %.2e"
          % (errs[0], max(errs), errs[-1]))
    assert max(errs) < REC_TOL, errs
    assert list(hist["rho"]) == [x["rho"] for x in h64]
