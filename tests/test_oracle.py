"""CPU tests of the FP64 oracle: pins it against known answers and the
reference's own test, and checks the algebra the GPU path relies on."""

import json
import os

import numpy as np
import pytest

from oracle import rectv_oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))


def test_usfft_radius_is_four():
    # radonusfft.cu:11 gives 4 for every width the kernels may see
    for n in (2, 8, 64, 255, 504, 1024, 4096):
        assert orc.usfft_params(n)[1] == 4


def test_usfft_adjoint_identity():
    rng = np.random.default_rng(0)
    n, ntheta = 32, 64
    theta = np.linspace(0, 4 * np.pi, ntheta, endpoint=False).astype(np.float32)
    U = orc.USFFT(n, theta, n / 2 + 1.5)
    f = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
    g = rng.standard_normal((2, ntheta, n)) + 1j * rng.standard_normal((2, ntheta, n))
    a = np.vdot(g, U.fwd(f))
    b = np.vdot(U.adj(g), f)
    assert abs(a - b) / abs(a) < 1e-12


@pytest.mark.parametrize("center_off", [0.0, 3.0, -5.0])
@pytest.mark.parametrize("blob", [(0.0, 0.0), (5.0, -3.0), (-7.0, 4.0)])
def test_usfft_known_answer_gaussian(center_off, blob):
    """Radon transform of a Gaussian blob is a Gaussian in s = x sin(theta) +
    y cos(theta) (+ rotation-axis offset); the USFFT (eps = 1e-3) reproduces it
    scaled by 1/sqrt(n ntheta)."""
    n, ntheta, sig = 64, 16, 4.0
    theta = np.linspace(0, np.pi, ntheta, endpoint=False).astype(np.float32)
    U = orc.USFFT(n, theta, n / 2 + center_off)
    xx = np.arange(n) - n // 2
    xc, yc = blob
    img = np.exp(-((xx[None, :] - xc) ** 2 + (xx[:, None] - yc) ** 2) / (2 * sig ** 2))
    p = U.fwd(img[None].astype(complex))[0]
    th = theta.astype(np.float64)
    sc = xc * np.sin(th) + yc * np.cos(th) + center_off
    s = np.arange(n) - n // 2
    ana = sig * np.sqrt(2 * np.pi) * np.exp(-(s[None, :] - sc[:, None]) ** 2 / (2 * sig ** 2))
    ana /= np.sqrt(n * ntheta)
    assert np.linalg.norm(p.real - ana) / np.linalg.norm(ana) < 1e-4
    assert np.abs(p.imag).max() < 1e-4 * np.abs(ana).max()


def test_radonapr_adjoint_identity():
    rng = np.random.default_rng(1)
    n, ntheta, m = 32, 64, 4
    theta = np.linspace(0, 4 * np.pi, ntheta, endpoint=False).astype(np.float32)
    ops = orc.Operators(n, ntheta, m, theta, orc.takephi(ntheta, m), n / 2)
    f = rng.standard_normal((2, m, n, n))
    g = rng.standard_normal((2, ntheta, n))
    a = np.sum(g * ops.radonapr(f))
    b = np.sum(ops.radonapradj(g) * f)
    assert abs(a - b) / abs(a) < 1e-12


def _reformulated_radonapr(ops, f):
    """R_apr computed the way the GPU does: one real 2D FFT per time sample,
    one gather of all samples, K'(theta, j) mixing, one row FFT."""
    R = ops.R
    n, r, ntheta, m = R.n, R.r, ops.ntheta, ops.m
    kmat = ops.cphi * np.einsum("it,ij->tj", ops.phi, np.conj(ops.phi[:, ops.tj]))
    nz = f.shape[0]
    out = np.zeros((nz, ntheta, n))
    for z in range(nz):
        acc = np.zeros((ntheta, n), dtype=complex)
        for j in range(m):
            pw = 2 * n + 2 * r
            fde = np.zeros((pw, pw), dtype=complex)
            fde[n // 2 + r:n // 2 + r + n, n // 2 + r:n // 2 + r + n] = f[z, j] * R.deapod
            fde *= R.mod2
            fde[r:r + 2 * n, r:r + 2 * n] = np.fft.fft2(fde[r:r + 2 * n, r:r + 2 * n])
            fde *= R.mod2
            fde = R._wrap_fwd(fde[None])[0]
            gj = (R.G @ fde.ravel()).reshape(ntheta, n)
            acc += kmat[:, j][:, None] * gj
        acc *= R.shiftfwd[None, :] * R.mod1
        y = np.fft.ifft(acc, axis=-1) * n * R.mod1 * R.scale
        out[z] = y.real
    return out


def test_gpu_formulation_equals_reference_structure():
    rng = np.random.default_rng(2)
    n, ntheta, m = 24, 40, 5
    theta = np.linspace(0, 6 * np.pi, ntheta, endpoint=False).astype(np.float32)
    phi = (rng.standard_normal((m, 2 * ntheta)) / np.sqrt(ntheta)).astype(np.float32)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2 + 2.0)
    f = rng.standard_normal((2, m, n, n))
    a = ops.radonapr(f)
    b = _reformulated_radonapr(ops, f)
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-12


def test_divergence_is_half_gradient_transpose():
    """div = 1/2 G^T on the grid points div reads (kernels_operators.cuh:40-43
    divide by 2 cbrt2 lambda1/2, :69-72 by 4 cbrt2 lambda1/2)."""
    rng = np.random.default_rng(3)
    n, m, nzp, lam1 = 10, 4, 3, 4.0
    for flgl, flgr in ((0, 0), (1, 1)):
        fm = rng.standard_normal((nzp + 2, m, n, n))
        h = orc.gradient(fm, lam1, flgl, flgr)
        d = orc.divergent(h, lam1, 1.0)
        mask = np.zeros(h.shape, dtype=bool)
        mask[1:, 1:, 1:, :, 0] = True
        mask[1:, 1:, :, 1:, 1] = True
        mask[1:, :, 1:, 1:, 2] = True
        mask[:, 1:, 1:, 1:, 3] = True
        # only the chunk interior is updated; the halo term cancels for flg=0
        if flgl == 0 and flgr == 0:
            lhs = np.sum(fm[1:nzp + 1] * d)
            rhs = 0.5 * np.sum((h * mask) ** 2)
            assert abs(lhs - rhs) / rhs < 1e-12
        assert d.shape == (nzp, m, n, n)


def test_reference_test_assertions_small():
    """tests/test_adjoint.py:132-158 of the reference on a smaller geometry."""
    n, ntheta, m, nz, lam1 = 48, 240, 16, 1, 8.0
    np.random.seed(0)
    data = np.random.random([nz, ntheta, n]).astype("float32")
    theta = np.linspace(0, 8 * np.pi, ntheta).astype("float32")
    res = orc.check_adjoints(data, theta, orc.takephi(ntheta, m), lam1, n / 2)
    np.testing.assert_allclose(res[0], res[1], rtol=1e-10)  # exact adjoint in FP64
    np.testing.assert_allclose(res[1], res[2], rtol=1)


def test_golden_refconfig_adjoint():
    """Oracle values on the reference test's exact configuration
    (n=504, ntheta=2400, m=16, lambda1=8) pass all four of its assertions
    (tests/test_adjoint.py:155-158), the R one exactly."""
    with open(os.path.join(HERE, "golden", "refconfig_adjoint.json")) as f:
        res = np.array(json.load(f)["res"])
    np.testing.assert_allclose(res[0], res[1], rtol=1e-10)
    np.testing.assert_allclose(res[0], res[1], rtol=1e-1)
    np.testing.assert_allclose(res[1], res[2], rtol=1)
    np.testing.assert_allclose(res[3], res[4], rtol=1e-1)
    np.testing.assert_allclose(res[4], res[5], rtol=1)


def test_admm_reduces_data_misfit():
    n, ntheta, m, nz, nzp = 16, 32, 2, 2, 1
    theta = np.linspace(0, 2 * np.pi, ntheta, endpoint=False).astype(np.float32)
    phi = orc.takephi(ntheta, m)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    u = np.zeros((nz, m, n, n))
    u[:, :, 5:11, 4:12] = 1.0
    g = ops.radonapr(u)
    f, hist = orc.run(g, theta, phi, n / 2, 1e-4, 1.0, 6, 3, nzp, return_history=True)
    r0 = np.linalg.norm(g)
    r1 = np.linalg.norm(ops.radonapr(f) - g)
    assert r1 < 0.5 * r0
    assert all(h["rho"] > 0 for h in hist)


# ---------------------------------------------------------------------------
# Pins against the reference's own CUDA build: fixtures made by
# tests/golden/make_ref_golden.py, which runs the reference's src/cuda/*.cu
# (compiled unchanged for sm_103a by oracle/ref_build.py) on a GB300.
# ---------------------------------------------------------------------------
REF_PIN = 1e-5  # the reference computes in FP32 with __sinf/__cosf sample positions


def _golden(name):
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name)


def test_oracle_matches_reference_build_config1():
    """Config 1 (32 ADMM iterations): the oracle's FP64 reconstruction
    (committed) against the reference build's."""
    ref = np.load(_golden("ref_c1_recon.npz"))
    f64 = np.load(_golden("c1_recon.npz"))
    err = np.linalg.norm(f64["f"].astype(np.float64) - ref["f"]) / np.linalg.norm(f64["f"].astype(np.float64))
    assert err < REF_PIN, err
    np.testing.assert_allclose(ref["rdiff"], f64["rdiff"], rtol=1e-4)


def test_oracle_matches_reference_build_16_time_samples():
    import sys
    sys.path.insert(0, os.path.dirname(_golden("x")))
    import make_ref_golden
    c = make_ref_golden.M16
    theta, phi, g = make_ref_golden.m16_inputs()
    f, hist = orc.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"], c["titer"],
                      c["nzp"], return_history=True)
    ref = np.load(_golden("ref_m16_recon.npz"))
    err = np.linalg.norm(f - ref["f"]) / np.linalg.norm(f)
    assert err < REF_PIN, err
    np.testing.assert_allclose(ref["rdiff"], [x["rdiff"] for x in hist], rtol=1e-4)


def test_oracle_check_adjoints_matches_reference_build():
    """The reference test's own configuration (n=504, ntheta=2400, m=16)."""
    import json
    with open(_golden("ref_refconfig_adjoint.json")) as fh:
        ref = np.array(json.load(fh)["res"])
    with open(_golden("refconfig_adjoint.json")) as fh:
        f64 = np.array(json.load(fh)["res"])
    np.testing.assert_allclose(f64, ref, rtol=REF_PIN)
