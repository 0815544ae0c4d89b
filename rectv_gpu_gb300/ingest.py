"""Data ingest: detector frames -> sinograms, on the GPU.

Replaces the preprocessing the reference's tao example does with NumPy
(examples/tao/tao.py:34-41):

    data = -log((data - mean(dark, 0)) / (1e-3 + mean(flat, 0) - mean(dark, 0))).swapaxes(0, 1)

turning projections [ntheta, nz, n] into the solver's input [nz, ntheta, n].
"""

import ctypes

import numpy as np

from . import _lib

_DTYPES = {np.dtype(np.float32): 0, np.dtype(np.uint16): 1}


def preprocess(data, dark, flat):
    """Flat/dark normalisation, -log and transpose.

    data [ntheta, nz, n], dark [ndark, nz, n], flat [nflat, nz, n]; float32
    or uint16 (all the same type).  Returns float32 [nz, ntheta, n]."""
    data = np.ascontiguousarray(data)
    dt = data.dtype
    if dt not in _DTYPES:
        data = data.astype(np.float32)
        dt = data.dtype
    dark = np.ascontiguousarray(dark, dtype=dt)
    flat = np.ascontiguousarray(flat, dtype=dt)
    if data.ndim != 3 or dark.ndim != 3 or flat.ndim != 3:
        raise ValueError("data, dark and flat must be 3-D [frames, nz, n]")
    ntheta, nz, n = data.shape
    if dark.shape[1:] != (nz, n) or flat.shape[1:] != (nz, n):
        raise ValueError("dark and flat frames must be [frames, %d, %d]" % (nz, n))
    out = np.empty((nz, ntheta, n), dtype=np.float32)
    lib = _lib.load()
    _lib.check(lib.rectv_preprocess(out.ctypes.data, data.ctypes.data, dark.ctypes.data, flat.ctypes.data,
                                    _DTYPES[dt], ntheta, nz, n, dark.shape[0], flat.shape[0]))
    return out
