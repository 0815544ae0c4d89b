"""GPU parity of the full reconstruction (rectv::run through Solver.recon) and
of rectv::check_adjoints against the FP64 oracle.

Tolerance: reconstructions within 1e-4 relative L2 of the FP64 oracle on the
same seeded inputs.
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

pytestmark = pytest.mark.gpu

REC_TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


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
    # n, ntheta, m, nz, nzp, nrot, niter, titer, lambda0, lambda1
    (32, 64, 4, 4, 2, 4, 3, 2, 1e-3, 4.0),
    (32, 48, 8, 3, 1, 2, 2, 3, 1e-2, 1.0),
    (24, 40, 4, 5, 2, 4, 2, 1, 1e-3, 8.0),   # ragged: slice 4 is outside every chunk
    (32, 64, 4, 2, 2, 4, 2, 0, 1e-3, 4.0),   # titer = 0
])
def test_recon_matches_oracle(Solver, case):
    n, ntheta, m, nz, nzp, nrot, niter, titer, lam0, lam1 = case
    theta, phi, g = _problem(n, ntheta, m, nz, nrot)
    ref, hist = orc.run(g, theta, phi, n / 2, lam0 * lam1, lam1, niter, titer, nzp, return_history=True)
    with Solver(n, ntheta, m, nz, nzp, 1) as slv:
        slv.set_verbose(False)
        got = slv.recon(g, theta, phi, lambda0=lam0, lambda1=lam1, niter=niter, titer=titer)
        h = slv.history()
    assert got.shape == (nz, m, n, n) and got.dtype == np.float32
    if np.linalg.norm(ref) > 0:
        assert rel(got, ref) < REC_TOL, rel(got, ref)
    nzc = (nz // nzp) * nzp
    assert np.all(got[nzc:] == 0)
    assert np.allclose(h["rho"], [x["rho"] for x in hist])
    np.testing.assert_allclose(h["rdiff"], [x["rdiff"] for x in hist], rtol=1e-3, atol=1e-12)


def test_check_adjoints_matches_oracle(Solver):
    n, ntheta, m, nz, lam1 = 48, 96, 8, 1, 8.0
    theta = np.linspace(0, 8 * np.pi, ntheta).astype(np.float32)  # as tests/test_adjoint.py:35
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(0)
    data = rng.random((nz, ntheta, n)).astype(np.float32)
    ref = orc.check_adjoints(data, theta, phi, lam1, n / 2)
    with Solver(n, ntheta, m, nz, nz, 1) as slv:
        got = slv.adjoint_tests(data, theta, phi, lam1)
    np.testing.assert_allclose(got, ref, rtol=2e-5)
    # the reference test's assertions (tests/test_adjoint.py:155-156)
    np.testing.assert_allclose(got[0], got[1], rtol=1e-1)
    np.testing.assert_allclose(got[1], got[2], rtol=1)


def test_reference_test_config_matches_golden(Solver):
    """The reference's own test (tests/test_adjoint.py: n=504, ntheta=2400,
    m=16, nz=1, lambda1=8, seed 0) on the GPU: its four assertions, and the
    six values within 2e-5 of the FP64 oracle's golden values."""
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "refconfig_adjoint.json")) as f:
        gold = np.array(json.load(f)["res"])
    n, ntheta, m, nz, lam1 = 504, 2400, 16, 1, 8.0
    np.random.seed(0)
    data = np.random.random([nz, ntheta, n]).astype("float32")
    theta = np.linspace(0, 8 * np.pi, ntheta).astype("float32")
    with Solver(n, ntheta, m, nz, nz, 1) as slv:
        res = slv.adjoint_tests(data, theta, orc.takephi(ntheta, m), lam1)
    np.testing.assert_allclose(res, gold, rtol=2e-5)
    np.testing.assert_allclose(res[0], res[1], rtol=1e-1)
    np.testing.assert_allclose(res[1], res[2], rtol=1)
    np.testing.assert_allclose(res[3], res[4], rtol=1e-1)
    np.testing.assert_allclose(res[4], res[5], rtol=1)


def test_config1_recon_matches_golden(Solver):
    """Config 1 (N=64, Nz=8, Nzp=8, Ntheta=256, Nrot=4, M=8, 32 ADMM
    iterations, titer=4) against the FP64 oracle's reconstruction."""
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_golden
    gold = np.load(os.path.join(here, "golden", "c1_recon.npz"))
    theta, phi, g = make_golden.c1_inputs()
    c = make_golden.C1
    with Solver(c["n"], c["ntheta"], c["m"], c["nz"], c["nzp"], 1) as slv:
        slv.set_verbose(False)
        got = slv.recon(g, theta, phi, lambda0=c["lambda0"], lambda1=c["lambda1"], niter=c["niter"],
                        titer=c["titer"])
        h = slv.history()
    assert rel(got, gold["f"].astype(np.float64)) < REC_TOL
    np.testing.assert_allclose(h["rho"], gold["rho"])


@pytest.mark.parametrize("case", [
    (256, 360, 8, 2, 2, 2, 3),
    (1024, 720, 16, 2, 1, 2, 2),   # the benchmark's grid, two chunks
    (512, 361, 12, 1, 1, 2, 2),    # odd number of rows (a row pair with one row), one slice (a slice pair with one slice)
])
def test_recon_padded_fft_and_fused_rows_match_cufft_path(Solver, monkeypatch, case):
    """With 2n a power of two (n = 256, and n = 1024 as in the benchmark) the
    reconstruction runs the hand-written padded-grid FFTs and the fused
    residual-row kernel (inverse row FFT, residual and the adjoint's row
    transform in one pass); RECTV_CUFFT=1 runs the same iterations through
    cuFFT and the separate passes.  Both must agree to FP32 rounding
    accumulated over the iterations, and give the same rho sequence."""
    n, ntheta, m, nz, nzp, niter, titer = case
    lam0, lam1 = 1e-3, 4.0
    theta = scan_angles(ntheta, 4)
    phi = orc.takephi(ntheta, m)
    g = np.random.default_rng(3).standard_normal((nz, ntheta, n)).astype(np.float32)
    out = {}
    for mode in ("own", "cufft"):
        if mode == "cufft":
            monkeypatch.setenv("RECTV_CUFFT", "1")
        else:
            monkeypatch.delenv("RECTV_CUFFT", raising=False)
        with Solver(n, ntheta, m, nz, nzp, 1) as slv:
            slv.set_verbose(False)
            out[mode] = (slv.recon(g, theta, phi, lambda0=lam0, lambda1=lam1, niter=niter, titer=titer),
                         slv.history())
    assert rel(out["own"][0], out["cufft"][0].astype(np.float64)) < 2e-5
    assert np.allclose(out["own"][1]["rho"], out["cufft"][1]["rho"])
    np.testing.assert_allclose(out["own"][1]["rdiff"], out["cufft"][1]["rdiff"], rtol=1e-4)
