"""Output writer: TIFF stacks of reconstructed slices.

The reference's examples save each time sample of the reconstruction as a
stack of 32-bit float TIFF images, one file per slice
(examples/foam/foam_example.py:103-104, dxchange.write_tiff_stack(rtv[k],
'rec_tv/rec_'+str(k))).  This module writes the same: baseline TIFF,
uncompressed, one float32 image per file, files named prefix_00000.tiff, ...
"""

import os
import struct

import numpy as np


def write_tiff(fname, img):
    """Write one 2-D array as an uncompressed float32 TIFF."""
    img = np.ascontiguousarray(img, dtype="<f4")
    if img.ndim != 2:
        raise ValueError("write_tiff expects a 2-D array")
    h, w = img.shape
    data = img.tobytes()
    entries = [  # tag, type, count, value (types: 3 SHORT, 4 LONG)
        (256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, 32), (259, 3, 1, 1), (262, 3, 1, 1),
        (273, 4, 1, 8), (277, 3, 1, 1), (278, 4, 1, h), (279, 4, 1, len(data)), (284, 3, 1, 1),
        (339, 3, 1, 3),  # SampleFormat = IEEE float
    ]
    ifd_off = 8 + len(data)
    with open(fname, "wb") as f:
        f.write(b"II" + struct.pack("<HI", 42, ifd_off))
        f.write(data)
        f.write(struct.pack("<H", len(entries)))
        for tag, typ, cnt, val in entries:
            if typ == 3:
                f.write(struct.pack("<HHIHH", tag, typ, cnt, val, 0))
            else:
                f.write(struct.pack("<HHII", tag, typ, cnt, val))
        f.write(struct.pack("<I", 0))


def read_tiff(fname):
    """Read a TIFF written by write_tiff (float32, one strip)."""
    with open(fname, "rb") as f:
        buf = f.read()
    if buf[:2] != b"II":
        raise ValueError("not a little-endian TIFF")
    (ifd_off,) = struct.unpack_from("<I", buf, 4)
    (n,) = struct.unpack_from("<H", buf, ifd_off)
    tags = {}
    for i in range(n):
        tag, typ, cnt = struct.unpack_from("<HHI", buf, ifd_off + 2 + 12 * i)
        val = struct.unpack_from("<H" if typ == 3 else "<I", buf, ifd_off + 2 + 12 * i + 8)[0]
        tags[tag] = val
    w, h, off, nbytes = tags[256], tags[257], tags[273], tags[279]
    return np.frombuffer(buf, dtype="<f4", count=w * h, offset=off).reshape(h, w).copy()


def write_tiff_stack(data, fname, digit=5, start=0, overwrite=False):
    """Write data[k] for k along axis 0 to fname_<k>.tiff (dxchange naming)."""
    data = np.asarray(data)
    d = os.path.dirname(fname)
    if d:
        os.makedirs(d, exist_ok=True)
    names = []
    for k in range(data.shape[0]):
        name = "%s_%0*d.tiff" % (fname, digit, start + k)
        if os.path.exists(name) and not overwrite:
            raise FileExistsError(name)
        write_tiff(name, data[k])
        names.append(name)
    return names
