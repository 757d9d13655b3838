"""Read / write the named-matrix container used by the cgsense_run plugin host.

Layout: b"CGSM", u32 count, then per matrix: u32 name length, name, u32 type
(0 float32, 1 complex64), u32 ndims, u64 dims (codeare order, first index
fastest), raw data.  A C-order numpy array of shape (a, b, c) is codeare's
(c, b, a) matrix with the same memory.
"""
from __future__ import annotations

import struct

import numpy as np


def write(path, mats: dict):
    with open(path, "wb") as f:
        f.write(b"CGSM")
        f.write(struct.pack("<I", len(mats)))
        for name, a in mats.items():
            a = np.ascontiguousarray(a)
            if np.iscomplexobj(a):
                a = a.astype(np.complex64)
                t = 1
            else:
                a = a.astype(np.float32)
                t = 0
            dims = list(reversed(a.shape)) if a.ndim > 1 else [a.shape[0], 1]
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)))
            f.write(nb)
            f.write(struct.pack("<II", t, len(dims)))
            for d in dims:
                f.write(struct.pack("<Q", d))
            f.write(a.tobytes())


def read(path) -> dict:
    out = {}
    with open(path, "rb") as f:
        assert f.read(4) == b"CGSM"
        (n,) = struct.unpack("<I", f.read(4))
        for _ in range(n):
            (ln,) = struct.unpack("<I", f.read(4))
            name = f.read(ln).decode()
            t, nd = struct.unpack("<II", f.read(8))
            dims = [struct.unpack("<Q", f.read(8))[0] for _ in range(nd)]
            dt = np.complex64 if t == 1 else np.float32
            cnt = int(np.prod(dims))
            a = np.frombuffer(f.read(cnt * np.dtype(dt).itemsize), dtype=dt).copy()
            out[name] = a.reshape(list(reversed(dims)))
    return out
