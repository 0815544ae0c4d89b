"""The multi-problem engine (batched form and serving loop) and the launch-
shape autotuner on the GPU.

* Every job's result in a mix of problems of different sizes -- arriving at
  different times, admitted by a device-memory budget that makes some wait,
  running concurrently -- equals its result alone (rectv.run, the drop-in
  call), within 1e-5 relative (the kernels are deterministic, so equality is
  expected).
* A job larger than the budget fails with a message; the others complete.
* Autotuned launch shapes leave the reconstruction unchanged.
"""

import numpy as np
import pytest

from oracle import rectv_oracle as orc
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles
from rectv_gpu_gb300.rectv import estimate_bytes

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def env(lib_built, torch_cuda):
    import rectv_gpu_gb300 as r
    from rectv_gpu_gb300 import _lib, engine
    return r, engine, _lib


def _problem(n, ntheta, m, nz, nrot, seed):
    theta = scan_angles(ntheta, nrot)
    phi = orc.takephi(ntheta, m)
    u = phantom4d(n, nz, m, ntheta, seed=seed)
    g = np.random.default_rng(seed).standard_normal((nz, ntheta, n)).astype(np.float32) * 0.01
    ops = orc.Operators(n, ntheta, m, theta, phi, n / 2)
    g = g + add_noise(ops.radonapr(u.astype(np.float64)), 0.01, seed)
    return theta, phi, g.astype(np.float32)


JOBS = [
    # n, ntheta, m, nz, nzp, nrot, niter, titer, arrival (s)
    (128, 180, 16, 4, 2, 4, 4, 3, 0.0),
    (64, 128, 8, 3, 3, 4, 6, 2, 0.0),
    (32, 64, 4, 4, 2, 4, 5, 3, 0.02),
    (256, 240, 16, 2, 2, 8, 3, 4, 0.05),
    (128, 180, 16, 4, 2, 4, 2, 3, 0.05),   # same dimensions as job 0: reuses its handle
    (64, 96, 12, 2, 1, 2, 4, 2, 0.1),
]


def test_mix_equals_alone(env):
    r, engine, _ = env
    probs = [_problem(*j[:4], j[5], seed=i) for i, j in enumerate(JOBS)]
    est = [estimate_bytes(j[0], j[1], j[2], j[3], j[4]) for j in JOBS]
    budget = sorted(est)[-1] + sorted(est)[-2] * 1.01  # at most about two of the largest at once
    with engine.Engine(budget_bytes=budget) as eng:
        ids = []
        for (n, ntheta, m, nz, nzp, nrot, niter, titer, arr), (theta, phi, g) in zip(JOBS, probs):
            ids.append(eng.submit(g, theta, phi, nzp=nzp, niter=niter, titer=titer, lambda0=1e-3, lambda1=4.0,
                                  arrival=arr))
        eng.run()
        infos = [eng.info(i) for i in ids]
        outs = [eng.result(i).copy() for i in ids]
        st = eng.stats()
    assert all(x["status"] == "done" for x in infos), infos
    assert st["peak_running"] >= 2, st
    assert st["peak_bytes"] <= budget * 1.05, st
    for (n, ntheta, m, nz, nzp, nrot, niter, titer, arr), (theta, phi, g), f, inf in zip(JOBS, probs, outs, infos):
        assert inf["admitted"] >= arr - 1e-6 and inf["done"] >= inf["admitted"]
        with r.Solver(n, ntheta, m, nz, nzp, 1) as slv:
            slv.set_verbose(False)
            alone = slv.recon(g, theta, phi, lambda0=1e-3, lambda1=4.0, niter=niter, titer=titer)
            h = slv.history()
        assert rel(f, alone) < TOL, (n, m, rel(f, alone))
        assert inf["rho"] == h["rho"][-1]


def test_job_over_budget_fails_others_complete(env):
    r, engine, lib = env
    theta, phi, g = _problem(32, 64, 4, 2, 4, seed=1)
    theta2, phi2, g2 = _problem(128, 180, 16, 4, 4, seed=2)
    with engine.Engine(budget_bytes=1.5 * estimate_bytes(32, 64, 4, 2, 2)) as eng:
        a = eng.submit(g, theta, phi, nzp=2, niter=2, titer=2)
        b = eng.submit(g2, theta2, phi2, nzp=2, niter=2, titer=2)
        eng.run()
        ia, ib = eng.info(a), eng.info(b)
    assert ia["status"] == "done"
    assert ib["status"] == "failed" and "budget" in ib["error"]


def test_autotune_keeps_results(env):
    r, _, _ = env
    import torch
    n, ntheta, m, nz, nzp = 256, 360, 16, 4, 2
    theta, phi, g = _problem(n, ntheta, m, nz, 8, seed=3)
    dev = torch.device("cuda")
    dg, dth, dph = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (g, theta, phi))
    outs = []
    shapes = None
    for tune in (False, True):
        obj = r.rectv(n, ntheta, m, nz, nzp, 1)
        obj.set_verbose(False)
        torch.cuda.synchronize()
        obj.setup_device(dg.data_ptr(), dth.data_ptr(), dph.data_ptr(), n / 2, 4e-3, 4.0, 3)
        if tune:
            shapes = obj.autotune(force=True)
            obj.setup_device(dg.data_ptr(), dth.data_ptr(), dph.data_ptr(), n / 2, 4e-3, 4.0, 3)
        obj.iterate(3)
        out = torch.empty((nz, m, n, n), dtype=torch.float32, device=dev)
        obj.result_device(out.data_ptr())
        obj.synchronize()
        outs.append(out.cpu().numpy())
        obj.free()
    assert shapes[0] in (8, 16, 32, 64) and shapes[1] >= 0
    assert np.array_equal(outs[0], outs[1])


def test_shortest_first_admission_order(env):
    """With one job at a time and every job waiting from the start, the
    shortest-first policy admits them in order of estimated work (bytes x
    iterations); arrival order admits them as submitted."""
    r, engine, _ = env
    sizes = [(128, 180, 16, 4, 2, 4, 3), (32, 64, 4, 4, 2, 4, 3), (64, 128, 8, 3, 3, 4, 3)]
    probs = [_problem(n, nt, m, nz, nrot, seed=i) for i, (n, nt, m, nz, nzp, nrot, it) in enumerate(sizes)]
    work = [estimate_bytes(n, nt, m, nz, nzp) * it for (n, nt, m, nz, nzp, nrot, it) in sizes]
    for sjf in (False, True):
        with engine.Engine(max_resident=1, shortest_first=sjf) as eng:
            ids = [eng.submit(g, th, ph, nzp=s[4], niter=s[6], titer=2, arrival=0.0)
                   for s, (th, ph, g) in zip(sizes, probs)]
            eng.run()
            infos = [eng.info(i) for i in ids]
        assert all(x["status"] == "done" for x in infos), infos
        order = list(np.argsort([x["admitted"] for x in infos]))
        assert order == (list(np.argsort(work)) if sjf else [0, 1, 2]), (sjf, order, work)
