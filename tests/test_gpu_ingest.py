"""GPU test of the ingest kernel (flat/dark normalisation, -log, transpose)
against the oracle's restatement of the reference's tao example."""

import numpy as np
import pytest

from oracle import rectv_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float32, np.uint16])
def test_preprocess_matches_oracle(lib_built, torch_cuda, dtype):
    from rectv_gpu_gb300 import ingest
    rng = np.random.default_rng(2)
    ntheta, nz, n = 37, 5, 64
    dark = rng.uniform(90, 110, (7, nz, n)).astype(dtype)
    flat = rng.uniform(3000, 4000, (9, nz, n)).astype(dtype)
    data = rng.uniform(500, 2900, (ntheta, nz, n)).astype(dtype)
    got = ingest.preprocess(data, dark, flat)
    ref = orc.preprocess(data, dark, flat)
    assert got.shape == (nz, ntheta, n) and got.dtype == np.float32
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-6)


def test_preprocess_validation(lib_built, torch_cuda):
    from rectv_gpu_gb300 import ingest
    with pytest.raises(ValueError):
        ingest.preprocess(np.ones((2, 3, 4), np.float32), np.ones((1, 3, 5), np.float32),
                          np.ones((1, 3, 4), np.float32))
