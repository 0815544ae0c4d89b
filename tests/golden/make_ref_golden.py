"""Generate golden fixtures from the reference's own CUDA build.

Needs a GPU and the reference build (``python -m oracle.ref_build``, which
compiles the reference's src/cuda/*.cu unchanged for sm_103a); it runs the
reference through oracle/ref_run.py in a child process.  Outputs:

  ref_refconfig_adjoint.json  rectv::check_adjoints on the reference test's
                              own inputs (tests/test_adjoint.py:15-35 of the
                              reference: n=504, ntheta=2400, m=16, nz=nzp=1,
                              lambda1=8, np.random.seed(0) uniform data,
                              theta = linspace(0, 8 pi, ntheta) with the
                              endpoint, centre n/2).
  ref_c1_recon.npz            rectv::run on config 1 (N=64, Nz=8, Nzp=8,
                              Ntheta=256, Nrot=4, M=8, lambda0=1e-3*lambda1,
                              lambda1=4, 32 iterations, titer=4, seed 0):
                              the reconstruction and the printed rdiff.
  ref_m16_recon.npz           rectv::run with 16 time samples (N=32, Nz=4,
                              Nzp=2, Ntheta=64, Nrot=4, 8 iterations,
                              titer=3, seed 1).

Run from the repository root: ``python tests/golden/make_ref_golden.py``.
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import ref_build, ref_run  # noqa: E402
from oracle import rectv_oracle as orc  # noqa: E402
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles  # noqa: E402
import make_golden  # noqa: E402

M16 = dict(n=32, ntheta=64, m=16, nz=4, nzp=2, nrot=4, lambda0=1e-3, lambda1=4.0, niter=8, titer=3, seed=1)


def m16_inputs():
    c = M16
    theta = scan_angles(c["ntheta"], c["nrot"])
    phi = orc.takephi(c["ntheta"], c["m"])
    u = phantom4d(c["n"], c["nz"], c["m"], c["ntheta"], seed=c["seed"])
    ops = orc.Operators(c["n"], c["ntheta"], c["m"], theta, phi, c["n"] / 2)
    g = add_noise(ops.radonapr(u.astype(np.float64)), 0.01, c["seed"])
    return theta, phi, g


def main():
    if ref_build.build() is None:
        raise SystemExit("reference sources not available")
    data, theta, phi, lambda1 = make_golden.refconfig_inputs()
    n = data.shape[2]
    res = ref_run.check_adjoints(data, theta, phi, lambda1, n / 2)
    with open(os.path.join(HERE, "ref_refconfig_adjoint.json"), "w") as f:
        json.dump({"res": [float(x) for x in res], "n": 504, "ntheta": 2400, "m": 16, "nz": 1, "lambda1": lambda1,
                   "source": "reference CUDA build, rectv::check_adjoints"}, f, indent=1)
    print("refconfig", res)
    for name, c, inputs in (("ref_c1_recon.npz", make_golden.C1, make_golden.c1_inputs),
                            ("ref_m16_recon.npz", M16, m16_inputs)):
        theta, phi, g = inputs()
        f, info = ref_run.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"],
                              c["titer"], c["nzp"])
        np.savez_compressed(os.path.join(HERE, name), f=f, rdiff=np.array(info["rdiff"]))
        print(name, f.shape, info["times"], info["rdiff"][-3:])


if __name__ == "__main__":
    main()
