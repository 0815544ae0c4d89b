"""CPU tests of the I/O rows around the path: the TIFF-stack writer and the
oracle's restatement of the reference's ingest formula."""

import numpy as np

from oracle import rectv_oracle as orc
from rectv_gpu_gb300 import tiff


def test_tiff_stack_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    vol = rng.standard_normal((3, 17, 23)).astype(np.float32)
    names = tiff.write_tiff_stack(vol, str(tmp_path / "rec_tv" / "rec_0"))
    assert [n.rsplit("/", 1)[1] for n in names] == ["rec_0_00000.tiff", "rec_0_00001.tiff", "rec_0_00002.tiff"]
    back = np.stack([tiff.read_tiff(n) for n in names])
    assert np.array_equal(back, vol)
    try:
        tiff.write_tiff_stack(vol, str(tmp_path / "rec_tv" / "rec_0"))
        raise AssertionError("overwrite must be refused by default")
    except FileExistsError:
        pass
    tiff.write_tiff_stack(vol, str(tmp_path / "rec_tv" / "rec_0"), overwrite=True)


def test_tiff_header_is_float32_baseline(tmp_path):
    p = str(tmp_path / "a.tiff")
    tiff.write_tiff(p, np.ones((4, 5), np.float32))
    buf = open(p, "rb").read()
    assert buf[:4] == b"II*\x00"
    assert len(buf) == 8 + 4 * 5 * 4 + 2 + 11 * 12 + 4


def test_oracle_ingest_matches_reference_formula():
    rng = np.random.default_rng(1)
    ntheta, nz, n = 6, 3, 8
    dark = rng.uniform(90, 110, (4, nz, n))
    flat = rng.uniform(900, 1100, (5, nz, n))
    data = rng.uniform(200, 800, (ntheta, nz, n))
    # examples/tao/tao.py:41, written out literally
    ref = -np.log((data - np.mean(dark, axis=0)) / (1e-3 + np.mean(flat, axis=0) - np.mean(dark, axis=0))).swapaxes(0, 1)
    got = orc.preprocess(data, dark, flat)
    assert got.shape == (nz, ntheta, n)
    assert np.allclose(got, ref, rtol=1e-14, atol=0)
