"""Generate the golden fixtures of tests/golden/ with the FP64 oracle.

  refconfig_adjoint.json  check_adjoints on the reference test's own
                          configuration (tests/test_adjoint.py:15-35 of the
                          reference: n=504, ntheta=2400, m=16, nz=nzp=1,
                          lambda1=8, np.random.seed(0) uniform data, theta =
                          linspace(0, 8 pi, ntheta) with the endpoint).
  c1_recon.npz            the reconstruction of config 1 (N=64, Nz=8,
                          Nzp=8, Ntheta=256, Nrot=4, M=8, lambda0=1e-3,
                          lambda1=4, 32 ADMM iterations, titer=4, seed 0)
                          with the per-iteration rdiff and rho.

Run from the repository root: ``python tests/golden/make_golden.py``.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import rectv_oracle as orc  # noqa: E402
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles  # noqa: E402

C1 = dict(n=64, ntheta=256, m=8, nz=8, nzp=8, nrot=4, lambda0=1e-3, lambda1=4.0, niter=32, titer=4,
          seed=0)


def refconfig_inputs():
    n, ntheta, m, nz, lambda1 = 504, 2400, 16, 1, 8.0
    np.random.seed(0)
    data = np.random.random([nz, ntheta, n]).astype("float32")
    theta = np.linspace(0, 8 * np.pi, ntheta).astype("float32")
    phi = orc.takephi(ntheta, m)
    return data, theta, phi, lambda1


def c1_inputs():
    c = C1
    theta = scan_angles(c["ntheta"], c["nrot"])
    phi = orc.takephi(c["ntheta"], c["m"])
    u = phantom4d(c["n"], c["nz"], c["m"], c["ntheta"], seed=c["seed"])
    ops = orc.Operators(c["n"], c["ntheta"], c["m"], theta, phi, c["n"] / 2)
    g = add_noise(ops.radonapr(u.astype(np.float64)), 0.01, c["seed"])
    return theta, phi, g


def main():
    t = time.time()
    data, theta, phi, lambda1 = refconfig_inputs()
    n = data.shape[2]
    res = orc.check_adjoints(data, theta, phi, lambda1, n / 2)
    with open(os.path.join(HERE, "refconfig_adjoint.json"), "w") as f:
        json.dump({"res": [float(x) for x in res], "n": 504, "ntheta": 2400, "m": 16, "nz": 1,
                   "lambda1": lambda1}, f, indent=1)
    print("refconfig", res, time.time() - t)

    t = time.time()
    theta, phi, g = c1_inputs()
    c = C1
    f, hist = orc.run(g, theta, phi, c["n"] / 2, c["lambda0"] * c["lambda1"], c["lambda1"], c["niter"],
                      c["titer"], c["nzp"], return_history=True)
    np.savez_compressed(os.path.join(HERE, "c1_recon.npz"), f=f.astype(np.float32),
                        rdiff=np.array([h["rdiff"] for h in hist]),
                        rho=np.array([h["rho"] for h in hist]))
    print("c1", time.time() - t)


if __name__ == "__main__":
    main()
