"""GPU test of rectv_shrink_noalloc, the allocation-free entry point.

Callers that cannot let a library allocate device memory (their own pool owns
the device budget, or their loop must not stall on cudaMalloc/cudaFree) use
it to run the ADMM shrink step on their own buffers.  This test checks, through
the C ABI, that two calls in a row reproduce what rectv_iterate reports for two
outer iterations: the residual sums r, s/rho^2 and ||u(k+1)-u(k)||^2 of its
history.  The file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def test_shrink_noalloc_matches_iterate(lib_built, torch_cuda):
    torch = torch_cuda
    from rectv_gpu_gb300 import _lib, rectv, takephi
    from rectv_gpu_gb300.phantom import scan_angles

    n, ntheta, m, nz, nzp, titer = 32, 64, 4, 4, 2, 2
    lam1 = 4.0
    lam0 = 1e-3 * lam1
    nchunks = nz // nzp
    theta = scan_angles(ntheta, 4)
    phi = takephi(ntheta, m)
    rng = np.random.default_rng(7)
    g = rng.random((nz, ntheta, n)).astype(np.float32)
    dev = torch.device("cuda", 0)
    d_g, d_th, d_ph = (torch.from_numpy(a).to(dev) for a in (g, theta, phi))

    obj = rectv(n, ntheta, m, nz, nzp, 1)
    obj.set_verbose(False)
    torch.cuda.synchronize()
    obj.setup_device(d_g.data_ptr(), d_th.data_ptr(), d_ph.data_ptr(), n / 2, lam0, lam1, titer)
    u = [torch.zeros((nz, m, n, n), dtype=torch.float32, device=dev) for _ in range(3)]
    for k in (1, 2):
        obj.iterate(1)
        obj.result_device(u[k].data_ptr())
        obj.synchronize()
    hist = obj.history()
    obj.free()

    gp = (n + 1) * (n + 1) * (m + 1) * (nzp + 1)
    psi = torch.zeros(4 * nchunks * gp, dtype=torch.float32, device=dev)
    mu = torch.zeros(4 * nchunks * gp, dtype=torch.float32, device=dev)
    sums = torch.zeros(3, dtype=torch.float64, device=dev)
    lib = _lib.load()
    rho = 0.5  # rho of the first outer iteration (rectv.cu:125)
    for k in (1, 2):
        torch.cuda.synchronize()
        _lib.check(lib.rectv_shrink_noalloc(
            ctypes.c_void_p(u[k].data_ptr()), ctypes.c_void_p(u[k - 1].data_ptr()),
            ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(mu.data_ptr()), n, m, nzp, nchunks,
            rho, lam0, lam1, ctypes.c_void_p(sums.data_ptr()), None))
        torch.cuda.synchronize()
        r_sum, s_sum, conv = sums.cpu().numpy()
        i = k - 1
        np.testing.assert_allclose(r_sum, hist["r"][i], rtol=RTOL)
        np.testing.assert_allclose(s_sum * rho * rho, hist["s"][i], rtol=RTOL)
        np.testing.assert_allclose(conv, hist["rdiff"][i], rtol=RTOL)
        assert conv > 0 and r_sum > 0
        rho = float(hist["rho"][i])  # rho after the update, used by the next iteration


def test_shrink_noalloc_rejects_oversize(lib_built, torch_cuda):
    from rectv_gpu_gb300 import _lib
    lib = _lib.load()
    dummy = ctypes.c_void_p(1)
    rc = lib.rectv_shrink_noalloc(dummy, dummy, dummy, dummy, 2048, 16, 16, 4, 0.5, 1e-3, 4.0, dummy, None)
    assert rc == 1
    assert "at most 65536" in lib.rectv_last_error().decode()
