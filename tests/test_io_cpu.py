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


def test_tiff_ifd_follows_the_baseline_spec(tmp_path):
    """Checks the file against the TIFF 6.0 baseline rules, independently of
    read_tiff: IFD entries sorted by tag, the required tags of a grayscale
    image present, one strip covering the whole image, IEEE float samples."""
    import struct
    p = str(tmp_path / "b.tiff")
    img = np.arange(35, dtype=np.float32).reshape(5, 7)
    tiff.write_tiff(p, img)
    buf = open(p, "rb").read()
    (ifd,) = struct.unpack_from("<I", buf, 4)
    (n,) = struct.unpack_from("<H", buf, ifd)
    tags = {}
    order = []
    for i in range(n):
        tag, typ, cnt = struct.unpack_from("<HHI", buf, ifd + 2 + 12 * i)
        val = struct.unpack_from("<H" if typ == 3 else "<I", buf, ifd + 10 + 12 * i)[0]
        tags[tag] = val
        order.append(tag)
    assert order == sorted(order)
    for required in (256, 257, 258, 259, 262, 273, 277, 278, 279):
        assert required in tags
    assert (tags[256], tags[257], tags[258], tags[259], tags[277], tags[339]) == (7, 5, 32, 1, 1, 3)
    assert tags[278] == 5 and tags[279] == 35 * 4
    assert np.array_equal(np.frombuffer(buf, "<f4", 35, tags[273]).reshape(5, 7), img)
    assert struct.unpack_from("<I", buf, ifd + 2 + 12 * n)[0] == 0  # single image


def test_standard_readers_read_the_stack(tmp_path):
    """tifffile or PIL, where installed, read the files back (neither is on
    the build image)."""
    vol = np.random.default_rng(2).standard_normal((2, 9, 11)).astype(np.float32)
    names = tiff.write_tiff_stack(vol, str(tmp_path / "rec_t"))
    readers = []
    try:
        import tifffile
        readers.append(lambda f: tifffile.imread(f))
    except ImportError:
        pass
    try:
        from PIL import Image
        readers.append(lambda f: np.asarray(Image.open(f), dtype=np.float32))
    except ImportError:
        pass
    if not readers:
        import pytest
        pytest.skip("no standard TIFF reader installed (tifffile, PIL)")
    for rd in readers:
        assert np.array_equal(np.stack([rd(n) for n in names]), vol)
