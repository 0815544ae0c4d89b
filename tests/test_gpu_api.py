"""GPU tests of the drop-in API's behaviour: determinism, CUDA-graph replay,
the device-resident session, input validation, error reporting, and
full-size, size-independent properties of the operators."""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def mods(lib_built, torch_cuda):
    import rectv_gpu_gb300 as r
    from rectv_gpu_gb300 import _lib
    return torch_cuda, r, _lib


def _small_problem(n=32, ntheta=64, m=4, nz=4, nrot=4, seed=0):
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=seed)
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    return theta, phi, add_noise(ops.radonapr(u.astype(np.float64)), 0.01, seed)


def test_deterministic_and_graphs_equal_eager(mods):
    torch, r, _ = mods
    theta, phi, g = _small_problem()
    outs = []
    for graphs in (True, True, False):
        with r.Solver(32, 64, 4, 4, 2, 1) as s:
            s.set_verbose(False)
            s.set_graphs(graphs)
            outs.append(s.recon(g, theta, phi, lambda0=1e-3, lambda1=4.0, niter=4, titer=3))
    assert np.array_equal(outs[0], outs[1])  # run to run
    assert np.array_equal(outs[0], outs[2])  # graph replay == eager launches


def test_device_session_equals_host_run(mods):
    torch, r, _ = mods
    theta, phi, g = _small_problem()
    n, ntheta, m, nz, nzp = 32, 64, 4, 4, 2
    with r.Solver(n, ntheta, m, nz, nzp, 1) as s:
        s.set_verbose(False)
        host = s.recon(g, theta, phi, lambda0=1e-3, lambda1=4.0, niter=3, titer=2)
        dg, dth, dph = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (g, theta, phi))
        out = torch.zeros((nz, m, n, n), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        s.setup_device(dg.data_ptr(), dth.data_ptr(), dph.data_ptr(), n / 2, 1e-3 * 4.0, 4.0, 2)
        s.iterate(1)
        s.iterate(2)  # resumable: 1 + 2 iterations == 3
        s.result_device(out.data_ptr())
        s.synchronize()
        h = s.history()
    assert np.array_equal(out.cpu().numpy(), host)
    assert len(h["rdiff"]) == 3


def test_input_validation_and_errors(mods):
    torch, r, lib = mods
    theta, phi, g = _small_problem()
    s = r.Solver(32, 64, 4, 4, 2, 1)
    assert (s.n, s.ntheta, s.m, s.nz) == (32, 64, 4, 4)
    with pytest.raises(AttributeError):
        s.n = 5  # read-only, as in the SWIG class (rectv.i:14-18)
    with pytest.raises(ValueError):
        s.recon(g[:, :, :16], theta, phi)
    with pytest.raises(ValueError):
        s.recon(g, theta[:10], phi)
    with pytest.raises(lib.RectvError):
        s.adjoint_tests(g, theta, phi, 4.0)  # nz != nzp
    s.free()
    s.free()  # idempotent (rectv.cu:65)
    with pytest.raises(lib.RectvError):
        s.recon(g, theta, phi)
    with pytest.raises(lib.RectvError):
        r.Solver(32, 64, 4, 2, 4, 1)  # nzp > nz
    # ngpus is clamped to nz // nzp (rectv.cu:9)
    with r.Solver(32, 64, 4, 4, 2, 8) as s2:
        assert s2.ngpus == 2


@pytest.mark.parametrize("case", [
    # n, ntheta, m, nz, nzp, center offset: 2n not a multiple of 16, off-centre axis
    (36, 50, 4, 3, 3, 1.5),
    (40, 72, 3, 4, 2, -2.0),
])
def test_recon_partial_tiles_and_offcentre(mods, case):
    torch, r, _ = mods
    n, ntheta, m, nz, nzp, dc = case
    theta = scan_angles(ntheta, 4)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(5)
    g = rng.random((nz, ntheta, n)).astype(np.float32)
    ref = orc.run(g, theta, phi, n / 2 + dc, 1e-3 * 2.0, 2.0, 2, 2, nzp)
    with r.Solver(n, ntheta, m, nz, nzp, 1) as s:
        s.set_verbose(False)
        got = s.recon(g, theta, phi, rot_center=n / 2 + dc, lambda0=1e-3, lambda1=2.0, niter=2, titer=2)
    assert rel(got, ref) < 1e-4


def test_from_scan_keyword_constructor(mods):
    torch, r, _ = mods
    n, ntheta, m, nz, nzp = 32, 64, 4, 2, 2
    s = r.Solver.from_scan(n, ntheta, m, 4, nz, nzp, lambda0=1e-3, lambda1=4.0)
    s.set_verbose(False)
    g = np.random.default_rng(0).random((nz, ntheta, n)).astype(np.float32)
    a = s.reconstruct(g, niter=2, titer=2)
    b = s.recon(g, scan_angles(ntheta, 4), r.takephi(ntheta, m), lambda0=1e-3, lambda1=4.0, niter=2, titer=2)
    s.free()
    assert np.array_equal(a, b)


def test_full_size_gaussian_blob_known_answer(mods):
    """N=1024, 2880 angles over 8 half-turns, one time sample constant in
    time: R_apr of a Gaussian blob is the analytic projection (the USFFT's
    eps = 1e-3 accuracy), independent of the oracle."""
    torch, r, _ = mods
    n, ntheta, m = 1024, 2880, 1
    theta = scan_angles(ntheta, 8)
    phi = np.zeros((1, 2 * ntheta), np.float32)
    phi[0, 0::2] = 1.0 / np.sqrt(ntheta)  # constant basis: K' = ntheta/sqrt(m) * 1/ntheta = 1
    xx = np.arange(n) - n // 2
    sig, xc, yc = 20.0, 130.0, -75.0
    img = np.exp(-((xx[None, :] - xc) ** 2 + (xx[:, None] - yc) ** 2) / (2 * sig ** 2)).astype(np.float32)
    obj = r.rectv(n, ntheta, m, 1, 1, 1)
    d_u = torch.from_numpy(img[None, None]).cuda()
    d_g = torch.zeros((1, ntheta, n), dtype=torch.float32, device="cuda")
    dth, dph = torch.from_numpy(theta).cuda(), torch.from_numpy(phi).cuda()
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), n / 2)
    obj.op_radonapr(d_g.data_ptr(), d_u.data_ptr(), 1, 1.0)
    p = d_g.cpu().numpy()[0].astype(np.float64)
    obj.free()
    th = theta.astype(np.float64)
    sc = xc * np.sin(th) + yc * np.cos(th)
    s = np.arange(n) - n // 2
    ana = sig * np.sqrt(2 * np.pi) * np.exp(-(s[None, :] - sc[:, None]) ** 2 / (2 * sig ** 2)) / np.sqrt(n * ntheta)
    assert rel(p, ana) < 1e-3


def test_full_size_adjoint_identity(mods):
    """<R_apr u, g> = <u, R_apr* g> at N=1024, Ntheta=2880, M=16 (one slice)."""
    torch, r, _ = mods
    n, ntheta, m = 1024, 2880, 16
    theta = scan_angles(ntheta, 8)
    phi = orc.takephi(ntheta, m)
    gen = torch.Generator(device="cuda").manual_seed(0)
    u = torch.randn((1, m, n, n), generator=gen, device="cuda")
    g = torch.randn((1, ntheta, n), generator=gen, device="cuda")
    ru = torch.zeros_like(g)
    ag = torch.zeros_like(u)
    obj = r.rectv(n, ntheta, m, 1, 1, 1)
    dth, dph = torch.from_numpy(theta).cuda(), torch.from_numpy(phi).cuda()
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), n / 2)
    obj.op_radonapr(ru.data_ptr(), u.data_ptr(), 1, 1.0)
    obj.op_radonapradj(ag.data_ptr(), g.data_ptr(), 1, 1.0)
    a = float((ru.double() * g.double()).sum())
    b = float((ag.double() * u.double()).sum())
    obj.free()
    assert abs(a - b) / abs(a) < 1e-5


def test_geometry_cache_across_runs(lib_built, torch_cuda):
    """rectv_run keeps the angle plan, K' and the captured graphs when theta,
    phi and the centre repeat: a second run is bit-identical to the first, a
    run with another centre rebuilds them and matches a fresh object, and
    the result still matches the oracle."""
    from rectv_gpu_gb300 import Solver
    from oracle import rectv_oracle as orc
    n, ntheta, m, nz, nzp = 32, 64, 4, 4, 2
    theta = np.linspace(0, 4 * np.pi, ntheta, endpoint=False).astype(np.float32)
    phi = orc.takephi(ntheta, m)
    g = np.random.default_rng(9).random((nz, ntheta, n)).astype(np.float32)
    with Solver(n, ntheta, m, nz, nzp, 1) as s:
        s.set_verbose(False)
        a = s.recon(g, theta, phi, lambda0=1e-3, lambda1=2.0, niter=3, titer=2)
        b = s.recon(g, theta, phi, lambda0=1e-3, lambda1=2.0, niter=3, titer=2)
        c = s.recon(g, theta, phi, rot_center=n / 2 + 1.5, lambda0=1e-3, lambda1=2.0, niter=3, titer=2)
    assert np.array_equal(a, b)
    with Solver(n, ntheta, m, nz, nzp, 1) as s2:
        s2.set_verbose(False)
        c2 = s2.recon(g, theta, phi, rot_center=n / 2 + 1.5, lambda0=1e-3, lambda1=2.0, niter=3, titer=2)
    assert np.array_equal(c, c2)
    ref = orc.run(g, theta, phi, n / 2, 1e-3 * 2.0, 2.0, 3, 2, nzp)
    assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-4


def test_bounded_wait_expires_promptly_and_is_reported(mods):
    """A wait that runs out (an mbarrier that nothing arrives on, nothing in
    flight) ends the kernel promptly, later waits of the same thread give up
    after the short limit instead of a full one each, the expiry is reported
    by rectv_synchronize, and the CUDA context stays usable."""
    import time
    torch, r, lib = mods
    s = r.rectv(32, 64, 4, 2, 2, 1)
    try:
        s.synchronize()
        t0 = time.perf_counter()
        # 2e6 cycles (~1 ms) for the first wait, then 1000 short waits (~0.1 ms each)
        lib.check(lib.load().rectv_selftest_wait(s._h, 2000000, 1000))
        with pytest.raises(lib.RectvError) as e:
            s.synchronize()
        elapsed = time.perf_counter() - t0
        assert e.value.code == 4  # RECTV_ERR_STATE
        assert elapsed < 2.0, elapsed
    finally:
        s.free()
    x = torch.arange(10, device="cuda", dtype=torch.float32)
    assert float(x.sum()) == 45.0
