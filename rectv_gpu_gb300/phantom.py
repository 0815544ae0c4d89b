"""Synthetic 4D (x, y, z, t) phantom: moving ellipsoids sampled at the m time
instants of the temporal model.

The reconstruction models the object at the m instants t_j = j*ntheta/m
(in projection-index units, decphi/recphi in kernels_operators.cuh:99-133 of
the reference), so the phantom is sampled at the fractions tau_j = t_j/ntheta
of the scan.  Each ellipsoid has a seeded centre uniform in the inner 60% of
the volume, semi-axes U(0.05, 0.3) times the volume size along each axis
(x, y use n, z uses nz), a density U(0.1, 1), a random in-plane orientation and
a linear displacement of at most 0.1*n over the whole scan.
"""

import numpy as np


def phantom4d(n, nz, m, ntheta, n_ellipsoids=10, seed=0, dtype=np.float32):
    """Return u [nz, m, n, n] (float32 by default)."""
    rng = np.random.default_rng(seed)
    x = np.arange(n, dtype=np.float64) - n / 2 + 0.5
    z = np.arange(nz, dtype=np.float64) - nz / 2 + 0.5
    Z, Y, X = np.meshgrid(z, x, x, indexing="ij")
    u = np.zeros((nz, m, n, n), dtype=np.float64)
    tj = (np.arange(m) * ntheta) // m
    for _ in range(n_ellipsoids):
        c0 = np.array([rng.uniform(-0.3, 0.3) * nz, rng.uniform(-0.3, 0.3) * n,
                       rng.uniform(-0.3, 0.3) * n])
        ax = np.array([rng.uniform(0.05, 0.3) * nz, rng.uniform(0.05, 0.3) * n,
                       rng.uniform(0.05, 0.3) * n])
        ax = np.maximum(ax, 0.75)
        dens = rng.uniform(0.1, 1.0)
        ang = rng.uniform(0, np.pi)
        direc = rng.normal(size=2)
        direc /= np.linalg.norm(direc) + 1e-12
        disp = direc * rng.uniform(0, 0.1 * n)
        ca, sa = np.cos(ang), np.sin(ang)
        for j in range(m):
            tau = tj[j] / ntheta
            cz = c0[0]
            cy = c0[1] + tau * disp[0]
            cx = c0[2] + tau * disp[1]
            dy, dx = Y - cy, X - cx
            ry = ca * dy - sa * dx
            rx = sa * dy + ca * dx
            inside = ((Z - cz) / ax[0]) ** 2 + (ry / ax[1]) ** 2 + (rx / ax[2]) ** 2 <= 1.0
            u[:, j][inside] += dens
    return u.astype(dtype)


def scan_angles(ntheta, nrot):
    """Equally spaced angles over nrot half-turns, float32 [ntheta]."""
    return np.linspace(0, nrot * np.pi, ntheta, endpoint=False).astype("float32")


def add_noise(g, rel_sigma=0.01, seed=0):
    """Gaussian noise with sigma = rel_sigma * max|g|."""
    rng = np.random.default_rng(seed + 12345)
    sigma = rel_sigma * float(np.max(np.abs(g)))
    return (g + rng.normal(0.0, sigma, size=g.shape)).astype(np.float32)
