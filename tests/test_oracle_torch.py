"""The FP64 PyTorch transcription of the oracle (oracle/rectv_oracle_torch.py)
against the NumPy oracle, on the CPU: operators and reconstructions agree to
1e-12 relative (both are float64 restatements of the same steps), and the
config-1 reconstruction reproduces the committed golden values."""

import os

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

torch = pytest.importorskip("torch")
ort = pytest.importorskip("oracle.rectv_oracle_torch")

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("case", [
    # n, ntheta, m, nz, nrot, centre offset
    (64, 256, 8, 2, 4, 0.0),    # config 1's geometry
    (48, 90, 16, 1, 8, -1.5),
    (40, 60, 5, 2, 2, 2.0),
])
def test_operators_match_numpy(case):
    n, ntheta, m, nz, nrot, dc = case
    theta = scan_angles(ntheta, nrot)
    rng = np.random.default_rng(1)
    phi = orc.takephi(ntheta, m) if m % 2 == 0 else (rng.standard_normal((m, 2 * ntheta)) / 8).astype(np.float32)
    u = rng.standard_normal((nz, m, n, n))
    g = rng.standard_normal((nz, ntheta, n))
    a = orc.Operators(n, ntheta, m, theta, phi, n / 2 + dc)
    b = ort.Operators(n, ntheta, m, theta, phi, n / 2 + dc, basis_batch=3)
    assert rel(b.radonapr(torch.from_numpy(u)).numpy(), a.radonapr(u)) < 1e-12
    assert rel(b.radonapradj(torch.from_numpy(g), 0.5).numpy(), a.radonapradj(g, 0.5)) < 1e-12
    fm = rng.standard_normal((nz + 2, m, n, n))
    for fl, fr in ((0, 0), (1, 0), (0, 1), (1, 1)):
        h = orc.gradient(fm, 4.0, fl, fr)
        assert np.array_equal(ort.gradient(torch.from_numpy(fm), 4.0, fl, fr).numpy(), h)
        assert np.array_equal(ort.divergent(torch.from_numpy(h), 4.0, -0.5).numpy(), orc.divergent(h, 4.0, -0.5))


def test_recon_matches_numpy():
    n, ntheta, m, nz, nzp, nrot = 32, 64, 16, 4, 2, 4
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=2)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    g = add_noise(ops.radonapr(u.astype(np.float64)), 0.01, 2)
    ref, hr = orc.run(g, theta, phi, n / 2, 4e-3, 4.0, 4, 3, nzp, return_history=True)
    got, hg = ort.run(g, theta, phi, n / 2, 4e-3, 4.0, 4, 3, nzp, return_history=True)
    assert rel(got, ref) < 1e-12
    assert [x["rho"] for x in hg] == [x["rho"] for x in hr]
    np.testing.assert_allclose([x["rdiff"] for x in hg], [x["rdiff"] for x in hr], rtol=1e-12)
    # a forced rho sequence that the rule would not choose
    forced = [0.5, 1.0, 0.25, 0.25]
    _, hf = ort.run(g, theta, phi, n / 2, 4e-3, 4.0, 4, 3, nzp, return_history=True, rho_sequence=forced)
    assert [x["rho"] for x in hf] == forced


def test_config1_matches_golden():
    """Config 1 (N=64, Nz=8, Nzp=8, Ntheta=256, Nrot=4, M=8, 32 iterations,
    titer=4) against the NumPy oracle's committed reconstruction (stored as
    float32, so the bar is float32 rounding)."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    gold = np.load(os.path.join(HERE, "golden", "c1_recon.npz"))
    theta, phi, g = make_golden.c1_inputs()
    c = make_golden.C1
    f, h = ort.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"], c["titer"],
                   c["nzp"], return_history=True)
    assert rel(f, gold["f"].astype(np.float64)) < 1e-7
    np.testing.assert_array_equal([x["rho"] for x in h], gold["rho"])
    np.testing.assert_allclose([x["rdiff"] for x in h], gold["rdiff"], rtol=1e-10)
