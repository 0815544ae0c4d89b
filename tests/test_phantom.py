"""CPU tests of the synthetic phantom and the basis helper."""

import numpy as np

from oracle import rectv_oracle as orc
from rectv_gpu_gb300 import takephi
from rectv_gpu_gb300.phantom import add_noise, phantom4d, scan_angles


def test_phantom_shape_determinism_and_motion():
    a = phantom4d(32, 4, 8, 256, seed=3)
    b = phantom4d(32, 4, 8, 256, seed=3)
    assert a.shape == (4, 8, 32, 32) and a.dtype == np.float32
    assert np.array_equal(a, b)
    assert a.max() > 0.1
    assert not np.array_equal(a[:, 0], a[:, -1])  # objects move over the scan
    assert not np.array_equal(a, phantom4d(32, 4, 8, 256, seed=4))


def test_angles_and_noise():
    th = scan_angles(2880, 8)
    assert th.dtype == np.float32 and th.shape == (2880,)
    assert abs(float(th[360]) - np.pi) < 1e-6
    g = np.ones((2, 3, 4), np.float32)
    gn = add_noise(g, 0.01, 0)
    assert gn.dtype == np.float32 and 0 < np.std(gn - g) < 0.05


def test_takephi_matches_reference_helper():
    assert np.array_equal(takephi(64, 8), orc.takephi(64, 8))
