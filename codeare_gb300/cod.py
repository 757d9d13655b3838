"""codeare's .cod raw matrix files (src/matrix/io/CODFile.hpp:45-210).

One matrix per file, little-endian on the machines this runs on:
    int32   data type (IOFile.hpp dtype: 0 float, 1 double, 2 complex float,
            3 complex double, 4 long, 5 short)
    uint64  number of dimensions n
    uint64  dims[n]           codeare order, first index fastest
    float32 resolutions[n]
    uint64  name length, then the name bytes
    data    prod(dims) elements
    the 32-character delimiter written after the data (the reader stops
    before it).
Arrays here are the C-order views of codeare's column-major matrices: a
codeare (d0, d1, ..., dk) matrix is the numpy array of shape (dk, ..., d1, d0).
"""
from __future__ import annotations

import struct

import numpy as np

DELIMITER = b"543f562189f1e82beb9c177f89f67822"
_TYPES = {0: np.float32, 1: np.float64, 2: np.complex64, 3: np.complex128, 4: np.int64, 5: np.int16}
_CODES = {np.dtype(v): k for k, v in _TYPES.items()}


def read(path: str):
    """(array, name, resolutions) of the matrix in a .cod file"""
    with open(path, "rb") as f:
        (dt,) = struct.unpack("<i", f.read(4))
        if dt not in _TYPES:
            raise ValueError("unknown COD data type %d" % dt)
        (n,) = struct.unpack("<Q", f.read(8))
        dims = list(struct.unpack("<%dQ" % n, f.read(8 * n)))
        res = list(struct.unpack("<%df" % n, f.read(4 * n)))
        (ln,) = struct.unpack("<Q", f.read(8))
        name = f.read(ln).decode()
        dtype = np.dtype(_TYPES[dt])
        count = int(np.prod(dims)) if dims else 0
        a = np.frombuffer(f.read(count * dtype.itemsize), dtype=dtype).copy()
        if a.size != count:
            raise ValueError("truncated COD file %s" % path)
    return a.reshape(tuple(reversed(dims))), name, res


def write(path: str, a: np.ndarray, name: str = "", res=None):
    a = np.ascontiguousarray(a)
    if a.dtype not in _CODES:
        raise ValueError("COD has no code for %s" % a.dtype)
    dims = list(reversed(a.shape)) if a.ndim > 1 else [a.shape[0], 1]
    res = list(res) if res is not None else [1.0] * len(dims)
    nb = name.encode()
    with open(path, "wb") as f:
        f.write(struct.pack("<i", _CODES[a.dtype]))
        f.write(struct.pack("<Q", len(dims)))
        f.write(struct.pack("<%dQ" % len(dims), *dims))
        f.write(struct.pack("<%df" % len(dims), *res))
        f.write(struct.pack("<Q", len(nb)))
        f.write(nb)
        f.write(a.tobytes())
        f.write(DELIMITER)
