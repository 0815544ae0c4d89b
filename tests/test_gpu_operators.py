"""GPU parity of the reference's operators (radonapr, radonapradj, gradient,
divergent) against the FP64 oracle, through the C ABI.

Tolerances: operators are FP32 on the GPU; relative L2 error against the FP64
oracle must be below 2e-5, and the GPU adjoint identity
<R u, g> = <u, R* g> must hold to 1e-5 relative.
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc

pytestmark = pytest.mark.gpu

OP_TOL = 2e-5


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def env(lib_built, torch_cuda):
    from rectv_gpu_gb300 import rectv
    return torch_cuda, rectv


@pytest.fixture(params=["per_ray", "auto"])
def usfft_path(request, monkeypatch):
    """Both USFFT paths: per-ray kernels, and the default choice (rays of a
    repeated direction share positions where they average 2.5 or more)."""
    if request.param == "per_ray":
        monkeypatch.setenv("RECTV_DIRS", "0")
    else:
        monkeypatch.delenv("RECTV_DIRS", raising=False)
    return request.param


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CASES = [
    # n, ntheta, m, nz, nzp, nrot, center_offset
    (32, 64, 4, 2, 2, 4, 0.0),
    (64, 128, 8, 3, 3, 4, 2.5),
    (48, 90, 16, 2, 1, 8, -1.0),
    (40, 60, 5, 2, 2, 2, 0.0),     # m not a power of two, 2n not a multiple of 16
    (64, 100, 1, 1, 1, 1, 0.0),
    (32, 64, 20, 1, 1, 4, 0.0),    # m > 16: two passes over time-sample groups
    (128, 360, 16, 2, 2, 8, 1.5),  # tensor-core gather, several ray chunks per item
    (96, 240, 12, 1, 1, 4, 0.0),   # tensor-core gather with zero-padded time samples
]


def _geometry(n, ntheta, m, nrot, seed):
    theta = np.linspace(0, nrot * np.pi, ntheta, endpoint=False).astype(np.float32)
    rng = np.random.default_rng(seed)
    if m <= 16 and seed % 2 == 0:
        phi = orc.takephi(ntheta, m)
    else:
        phi = (rng.standard_normal((m, 2 * ntheta)) / np.sqrt(ntheta)).astype(np.float32)
    return theta, phi


@pytest.mark.parametrize("case", CASES)
def test_radonapr_matches_oracle(env, usfft_path, case):
    torch, rectv = env
    n, ntheta, m, nz, nzp, nrot, dc = case
    center = n / 2 + dc
    theta, phi = _geometry(n, ntheta, m, nrot, n + m)
    rng = np.random.default_rng(1)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    ops = orc.Operators(n, ntheta, m, theta, phi, center)
    ref = ops.radonapr(f.astype(np.float64), 1.0)
    obj = rectv(n, ntheta, m, nz, nzp, 1)
    dth, dph, df = dev(torch, theta), dev(torch, phi), dev(torch, f)
    dg = torch.zeros((nz, ntheta, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
    obj.op_radonapr(dg.data_ptr(), df.data_ptr(), nz, 1.0)
    got = dg.cpu().numpy()
    obj.free()
    assert rel(got, ref) < OP_TOL, rel(got, ref)


@pytest.mark.parametrize("case", CASES)
def test_radonapradj_matches_oracle(env, usfft_path, case):
    torch, rectv = env
    n, ntheta, m, nz, nzp, nrot, dc = case
    center = n / 2 + dc
    theta, phi = _geometry(n, ntheta, m, nrot, n + m)
    rng = np.random.default_rng(2)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    f0 = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    tau = -0.5
    ops = orc.Operators(n, ntheta, m, theta, phi, center)
    ref = f0.astype(np.float64) + ops.radonapradj(g.astype(np.float64), tau)
    obj = rectv(n, ntheta, m, nz, nzp, 1)
    dth, dph, dg, df = dev(torch, theta), dev(torch, phi), dev(torch, g), dev(torch, f0)
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
    obj.op_radonapradj(df.data_ptr(), dg.data_ptr(), nz, tau)
    got = df.cpu().numpy()
    obj.free()
    inc_ref = ref - f0
    assert rel(got - f0, inc_ref) < OP_TOL, rel(got - f0, inc_ref)


def test_gpu_adjoint_identity(env):
    torch, rectv = env
    n, ntheta, m, nz = 64, 180, 8, 2
    theta = np.linspace(0, 8 * np.pi, ntheta, endpoint=False).astype(np.float32)
    phi = orc.takephi(ntheta, m)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    obj = rectv(n, ntheta, m, nz, nz, 1)
    dth, dph, df, dg = dev(torch, theta), dev(torch, phi), dev(torch, f), dev(torch, g)
    rf = torch.zeros_like(dg)
    ag = torch.zeros_like(df)
    torch.cuda.synchronize()
    obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), n / 2)
    obj.op_radonapr(rf.data_ptr(), df.data_ptr(), nz, 1.0)
    obj.op_radonapradj(ag.data_ptr(), dg.data_ptr(), nz, 1.0)
    a = float(np.sum(rf.cpu().numpy().astype(np.float64) * g))
    b = float(np.sum(ag.cpu().numpy().astype(np.float64) * f))
    obj.free()
    assert abs(a - b) / abs(a) < 1e-5


@pytest.mark.parametrize("flg", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gradient_divergent_match_oracle(env, flg):
    torch, rectv = env
    n, m, nzp, lam1 = 24, 5, 3, 4.0
    flgl, flgr = flg
    rng = np.random.default_rng(4)
    fm = rng.standard_normal((nzp + 2, m, n, n)).astype(np.float32)
    obj = rectv(n, 8, m, nzp, nzp, 1)
    dfm = dev(torch, fm)
    dh = torch.zeros((nzp + 1, m + 1, n + 1, n + 1, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    obj.op_gradient(dh.data_ptr(), dfm.data_ptr(), lam1, flgl, flgr)
    h = dh.cpu().numpy()
    href = orc.gradient(fm.astype(np.float64), lam1, flgl, flgr)
    assert rel(h, href) < 1e-6
    fn0 = rng.standard_normal((nzp, m, n, n)).astype(np.float32)
    dfn = dev(torch, fn0)
    torch.cuda.synchronize()
    obj.op_divergent(dfn.data_ptr(), dh.data_ptr(), lam1, -0.5)
    got = dfn.cpu().numpy() - fn0
    ref = orc.divergent(h.astype(np.float64), lam1, -0.5)
    obj.free()
    assert rel(got, ref) < 1e-5


@pytest.mark.parametrize("case", [(128, 360, 16, 2, 8, 1.5), (64, 180, 24, 1, 4, 0.0), (80, 200, 9, 1, 2, -2.0)])
def test_gather_paths_agree(env, case, monkeypatch):
    """The tensor-core gather (ray-wise time-sample mixing on tcgen05 with a
    three-term TF32/BF16 split) and the direct FP32 gather give the same
    forward operator: both within OP_TOL of the oracle, and within 5e-6 of
    each other."""
    torch, rectv = env
    n, ntheta, m, nz, nrot, dc = case
    center = n / 2 + dc
    theta, phi = _geometry(n, ntheta, m, nrot, 7)
    f = np.random.default_rng(2).standard_normal((nz, m, n, n)).astype(np.float32)
    ref = orc.Operators(n, ntheta, m, theta, phi, center).radonapr(f.astype(np.float64), 1.0)
    dth, dph, df = dev(torch, theta), dev(torch, phi), dev(torch, f)
    out = {}
    for mode in ("direct", "tc", "auto"):
        monkeypatch.setenv("RECTV_GATHER", mode)
        obj = rectv(n, ntheta, m, nz, nz, 1)
        dg = torch.zeros((nz, ntheta, n), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
        obj.op_radonapr(dg.data_ptr(), df.data_ptr(), nz, 1.0)
        out[mode] = dg.cpu().numpy()
        obj.free()
    for mode, got in out.items():
        assert rel(got, ref) < OP_TOL, (mode, rel(got, ref))
    assert rel(out["tc"], out["direct"].astype(np.float64)) < 5e-6
    assert rel(out["auto"], out["direct"].astype(np.float64)) < 5e-6


@pytest.mark.parametrize("case", [(128, 360, 16, 2, 8, 1.5), (64, 180, 24, 1, 4, 0.0), (80, 200, 9, 1, 2, -2.0),
                                  (72, 150, 16, 1, 2, 1.0)])
def test_scatter_paths_agree(env, case, monkeypatch):
    """The tensor-core scatter (ray-wise grids, then the time samples as a
    3xTF32 GEMM over rays on tcgen05) and the direct FP32 scatter give the same
    adjoint operator: both within OP_TOL of the oracle, within 5e-6 of each
    other, and the tensor-core path is reproducible bit for bit (n = 72: the
    Nyquist column falls inside a tile)."""
    torch, rectv = env
    n, ntheta, m, nz, nrot, dc = case
    center = n / 2 + dc
    theta, phi = _geometry(n, ntheta, m, nrot, 11)
    g = np.random.default_rng(5).standard_normal((nz, ntheta, n)).astype(np.float32)
    ref = orc.Operators(n, ntheta, m, theta, phi, center).radonapradj(g.astype(np.float64), 1.0)
    dth, dph, dg = dev(torch, theta), dev(torch, phi), dev(torch, g)
    out = {}
    for mode in ("direct", "tc", "tc2"):
        monkeypatch.setenv("RECTV_SCATTER", "tc" if mode == "tc2" else mode)
        obj = rectv(n, ntheta, m, nz, nz, 1)
        df = torch.zeros((nz, m, n, n), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
        obj.op_radonapradj(df.data_ptr(), dg.data_ptr(), nz, 1.0)
        out[mode] = df.cpu().numpy()
        obj.free()
    for mode, got in out.items():
        assert rel(got, ref) < OP_TOL, (mode, rel(got, ref))
    assert rel(out["tc"], out["direct"].astype(np.float64)) < 5e-6
    assert np.array_equal(out["tc"], out["tc2"])


@pytest.mark.parametrize("case", [(128, 180, 16, 2, 4, 1.5), (512, 360, 16, 1, 8, -3.0)])
def test_pad_fft_paths_agree(env, case, monkeypatch):
    """The hand-written padded-grid FFTs (row pairs and columns that skip the
    zero padding, deapodisation and crop fused in) and the cuFFT path
    (RECTV_CUFFT=1: deapodise/pad, cuFFT R2C / C2R, crop) give the same forward
    and adjoint operators to FP32 rounding; at n = 128 both are also checked
    against the oracle."""
    torch, rectv = env
    n, ntheta, m, nz, nrot, dc = case
    center = n / 2 + dc
    theta, phi = _geometry(n, ntheta, m, nrot, 3)
    rng = np.random.default_rng(9)
    f = rng.standard_normal((nz, m, n, n)).astype(np.float32)
    g = rng.standard_normal((nz, ntheta, n)).astype(np.float32)
    dth, dph, df, dg = dev(torch, theta), dev(torch, phi), dev(torch, f), dev(torch, g)
    fwd, adj = {}, {}
    for mode in ("pad", "cufft"):
        if mode == "cufft":
            monkeypatch.setenv("RECTV_CUFFT", "1")
        else:
            monkeypatch.delenv("RECTV_CUFFT", raising=False)
        obj = rectv(n, ntheta, m, nz, nz, 1)
        og = torch.zeros((nz, ntheta, n), dtype=torch.float32, device="cuda")
        of = torch.zeros((nz, m, n, n), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        obj.op_set_geometry(dth.data_ptr(), dph.data_ptr(), center)
        obj.op_radonapr(og.data_ptr(), df.data_ptr(), nz, 1.0)
        obj.op_radonapradj(of.data_ptr(), dg.data_ptr(), nz, 1.0)
        fwd[mode], adj[mode] = og.cpu().numpy(), of.cpu().numpy()
        obj.free()
    assert rel(fwd["pad"], fwd["cufft"].astype(np.float64)) < 2e-6
    assert rel(adj["pad"], adj["cufft"].astype(np.float64)) < 2e-6
    if n <= 128:
        ops = orc.Operators(n, ntheta, m, theta, phi, center)
        assert rel(fwd["pad"], ops.radonapr(f.astype(np.float64), 1.0)) < OP_TOL
        assert rel(adj["pad"], ops.radonapradj(g.astype(np.float64), 1.0)) < OP_TOL
