"""The reference's own CUDA build ("plain FP32 form") as a parity pin.

oracle/ref_build.py compiles the reference's src/cuda/*.cu unchanged for
sm_103a (plus a compatibility overload of cudaMemPrefetchAsync for CUDA 13
and an extern "C" shim in place of SWIG); oracle/ref_run.py runs it in a
child process.  These tests run it on seeded inputs and compare:

* its reconstruction with this project's GPU reconstruction and with the
  FP64 oracle (config 1, and 16 time samples on the tensor-core path);
* its check_adjoints sums on the reference test's own configuration with the
  GPU's and the oracle's.

Tolerances: 1e-4 relative L2 between reconstructions (the metric's bar);
check_adjoints sums 1e-4 relative.  The reference evaluates its polar
sample positions with the fast intrinsics __sinf/__cosf
(kernels_radonusfft.cuh:73-74) at angles up to 8 pi, this project and the
oracle with accurate sines; the bars include that difference.
"""

import os
import sys

import numpy as np
import pytest

from oracle import rectv_oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REC_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def ref(lib_built, torch_cuda):
    from oracle import ref_build, ref_run
    try:
        path = ref_build.build()
    except RuntimeError as e:
        pytest.fail("the reference's CUDA sources are present but do not build: %s" % e)
    if path is None:
        pytest.skip("reference CUDA sources not present on this machine (python -m oracle.ref_build)")
    sys.path.insert(0, os.path.join(HERE, "golden"))
    return ref_run


@pytest.fixture(scope="module")
def Solver(lib_built, torch_cuda):
    from rectv_gpu_gb300 import Solver
    return Solver


def _ours(Solver, g, theta, phi, c):
    with Solver(c["n"], c["ntheta"], c["m"], c["nz"], c["nzp"], 1) as slv:
        slv.set_verbose(False)
        f = slv.recon(g, theta, phi, lambda0=c["lambda0"], lambda1=c["lambda1"], niter=c["niter"], titer=c["titer"])
        return f, slv.history()


@pytest.mark.parametrize("which", ["c1", "m16"])
def test_reconstruction_matches_reference_build(ref, Solver, which):
    import make_golden
    import make_ref_golden
    if which == "c1":
        c, inputs = make_golden.C1, make_golden.c1_inputs
    else:
        c, inputs = make_ref_golden.M16, make_ref_golden.m16_inputs
    theta, phi, g = inputs()
    f_ref, info = ref.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"],
                          c["titer"], c["nzp"])
    f_ours, h = _ours(Solver, g, theta, phi, c)
    if which == "c1":  # the committed FP64 reconstruction of config 1
        f64 = np.load(os.path.join(HERE, "golden", "c1_recon.npz"))["f"]
    else:
        f64 = orc.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"],
                      c["titer"], c["nzp"])
    e_ref64, e_ours64, e_ours_ref = rel(f_ref, f64), rel(f_ours, f64), rel(f_ours, f_ref)
    print("%s: reference build vs FP64 %.2e, ours vs FP64 %.2e, ours vs reference build %.2e"
          % (which, e_ref64, e_ours64, e_ours_ref))
    assert e_ref64 < REC_TOL
    assert e_ours_ref < REC_TOL
    np.testing.assert_allclose(h["rdiff"], info["rdiff"], rtol=1e-3)


def test_check_adjoints_matches_reference_build(ref, Solver):
    import make_golden
    data, theta, phi, lambda1 = make_golden.refconfig_inputs()
    n = data.shape[2]
    res_ref = ref.check_adjoints(data, theta, phi, lambda1, n / 2)
    with Solver(n, theta.size, phi.shape[0], 1, 1, 1) as slv:
        res_ours = slv.adjoint_tests(data, theta, phi, lambda1)
    import json
    with open(os.path.join(HERE, "golden", "refconfig_adjoint.json")) as f:
        res64 = np.array(json.load(f)["res"])
    print("check_adjoints: reference build", res_ref, "ours", res_ours, "FP64", res64)
    np.testing.assert_allclose(res_ref, res64, rtol=1e-4)
    np.testing.assert_allclose(res_ours, res_ref, rtol=1e-4)
