"""GPU parity of the direction path (dir_kernels.cu) through the C ABI.

Scans over several half-turns revisit every direction: rays theta,
theta + pi, ... sample the same frequency points, so the USFFT interpolates
once per position and forms each ray by its time weights.  Rays are grouped
when their sample positions agree within 2e-3 grid cells; the operators must
still match the FP64 oracle (which interpolates every ray at its own angle)
within the operator bar 2e-5, agree with the per-ray tensor-core kernels,
keep the adjoint identity to 1e-5, and give reconstructions within 1e-4 of
the oracle with the same rho sequence.
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

pytestmark = pytest.mark.gpu

OP_TOL = 2e-5
REC_TOL = 1e-4


def rel(a, b):
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def env(lib_built, torch_cuda):
    from rectv_gpu_gb300 import rectv
    return torch_cuda, rectv


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ops(torch, rectv, n, ntheta, m, nz, theta, phi, center, f, g, tau):
    """GPU radonapr(f) and f + tau radonapradj(g); the direction count."""
    obj = rectv(n, ntheta, m, nz, nz, 1)
    dth, dph, df, dg = dev(torch, theta), dev(torch, phi), dev(torch, f), dev(torch, g)
    out = torch.zeros((nz, ntheta, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
    ndir = obj.directions()
    obj.op_radonapr(out.data_ptr(), df.data_ptr(), nz, 1.0)
    obj.op_radonapradj(df.data_ptr(), dg.data_ptr(), nz, tau)
    fw, ad = out.cpu().numpy(), df.cpu().numpy()
    obj.free()
    return fw, ad, ndir


def test_directions_detected(env, monkeypatch):
    torch, rectv = env
    n, ntheta, m = 64, 256, 8
    phi = orc.takephi(ntheta, m)
    f = np.zeros((1, m, n, n), np.float32)
    g = np.zeros((1, ntheta, n), np.float32)
    monkeypatch.delenv("RECTV_DIRS", raising=False)
    assert _ops(torch, rectv, n, ntheta, m, 1, scan_angles(ntheta, 8), phi, n / 2, f, g, 1.0)[2] == 32
    # the reference test's angles (linspace with the end point) do not repeat
    th = np.linspace(0, 8 * np.pi, ntheta).astype(np.float32)
    assert _ops(torch, rectv, n, ntheta, m, 1, th, phi, n / 2, f, g, 1.0)[2] == 0
    monkeypatch.setenv("RECTV_DIRS", "0")
    assert _ops(torch, rectv, n, ntheta, m, 1, scan_angles(ntheta, 8), phi, n / 2, f, g, 1.0)[2] == 0


CASES = [
    # n, ntheta, m, nz, nrot, center offset, phi kind
    (64, 256, 8, 2, 8, 0.0, "fourier"),
    (128, 360, 16, 2, 8, 1.5, "fourier"),   # off-centre axis
    (96, 240, 12, 1, 4, 0.0, "random"),     # 12 time samples (zero-padded to 16)
    (32, 64, 20, 1, 4, 0.0, "random"),      # two groups of time samples
    (40, 60, 8, 2, 2, -1.0, "fourier"),     # 2n not a multiple of 16
    (48, 90, 16, 2, 8, 0.0, "fourier"),     # two rays per direction (RECTV_DIRS=1)
    (256, 720, 16, 1, 8, 0.0, "fourier"),   # hand-written padded-grid FFT size
    (64, 512, 16, 2, 32, 0.5, "random"),    # 32 rays per direction: four mixing rounds
    (64, 240, 16, 2, 12, 0.0, "fourier"),   # 12 rays per direction: a partial mixing round
]


@pytest.mark.parametrize("case", CASES)
def test_dir_operators_match_oracle(env, monkeypatch, case):
    torch, rectv = env
    n, ntheta, m, nz, nrot, dc, kind = case
    monkeypatch.setenv("RECTV_DIRS", "1")
    center = n / 2 + dc
    theta = scan_angles(ntheta, nrot)
    rng = np.random.default_rng(n + m)
    phi = orc.takephi(ntheta, m) if kind == "fourier" else \
        (rng.standard_normal((m, 2 * ntheta)) / np.sqrt(ntheta)).astype(np.float32)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    tau = -0.5
    ops = orc.Operators(n, ntheta, m, theta, phi, center)
    ref_f = ops.radonapr(f.astype(np.float64), 1.0)
    ref_a = ops.radonapradj(g.astype(np.float64), tau)
    fw, ad, ndir = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, center, f, g, tau)
    assert 0 < ndir < ntheta
    assert rel(fw, ref_f) < OP_TOL, rel(fw, ref_f)
    assert rel(ad - f, ref_a) < OP_TOL, rel(ad - f, ref_a)


def test_dir_path_equals_per_ray_path(env, monkeypatch):
    torch, rectv = env
    n, ntheta, m, nz = 128, 360, 16, 2
    theta = scan_angles(ntheta, 8)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(7)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    monkeypatch.setenv("RECTV_DIRS", "0")
    f0, a0, nd0 = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, n / 2, f, g, 1.0)
    monkeypatch.setenv("RECTV_DIRS", "1")
    f1, a1, nd1 = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, n / 2, f, g, 1.0)
    assert nd0 == 0 and nd1 == 45
    assert rel(f1, f0) < 1e-5, rel(f1, f0)
    assert rel(a1 - f, a0 - f) < 1e-5, rel(a1 - f, a0 - f)


def test_dir_adjoint_identity(env, monkeypatch):
    torch, rectv = env
    monkeypatch.delenv("RECTV_DIRS", raising=False)
    n, ntheta, m, nz = 256, 480, 16, 2
    theta = scan_angles(ntheta, 8)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    fw, ad, ndir = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, n / 2, f, g, 1.0)
    assert ndir == 60
    a = float(np.sum(fw.astype(np.float64) * g))
    b = float(np.sum((ad - f).astype(np.float64) * f))
    assert abs(a - b) / abs(a) < 1e-5


def test_dir_deterministic(env, monkeypatch):
    torch, rectv = env
    monkeypatch.delenv("RECTV_DIRS", raising=False)
    n, ntheta, m, nz = 64, 256, 16, 2
    theta = scan_angles(ntheta, 8)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(5)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    r1 = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, n / 2, f, g, 1.0)
    r2 = _ops(torch, rectv, n, ntheta, m, nz, theta, phi, n / 2, f, g, 1.0)
    assert np.array_equal(r1[0], r2[0]) and np.array_equal(r1[1], r2[1])


@pytest.mark.parametrize("case", [
    # n, ntheta, m, nz, nzp, nrot, niter, titer
    (64, 128, 16, 4, 2, 4, 6, 4),     # two chunks, cuFFT padded grid
    (128, 192, 16, 2, 2, 4, 4, 4),    # hand-written padded-grid FFTs (2n = 256)
    (64, 96, 8, 3, 1, 2, 4, 3),       # 8 time samples, three chunks
])
def test_dir_recon_matches_oracle(lib_built, torch_cuda, monkeypatch, case):
    from rectv_gpu_gb300 import Solver
    monkeypatch.setenv("RECTV_DIRS", "1")
    n, ntheta, m, nz, nzp, nrot, niter, titer = case
    lam0, lam1 = 1e-3, 4.0
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=0)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    g = add_noise(ops.radonapr(u.astype(np.float64)), 0.01, 0)
    ref, hist = orc.run(g, theta, phi, n / 2, lam0 * lam1, lam1, niter, titer, nzp, return_history=True)
    with Solver(n, ntheta, m, nz, nzp, 1) as slv:
        slv.set_verbose(False)
        got = slv.recon(g, theta, phi, lambda0=lam0, lambda1=lam1, niter=niter, titer=titer)
        h = slv.history()
    err = rel(got, ref)
    assert err < REC_TOL, err
    assert np.allclose(h["rho"], [x["rho"] for x in hist])
