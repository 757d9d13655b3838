"""FP64 CPU oracle for the non-Cartesian CG-SENSE path (ctypes front end).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, never by the product package.

PARITY UNPINNED: the reference ships no golden vectors for this path and its
NFFT arithmetic lives in the absent third-party NFFT3 library; see the header
of cgs_oracle.c for what is restated from where.  The NFFT restatement is
pinned to the mathematics by the direct NDFT below.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "cgs_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "libcgs_oracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile cgs_oracle.c with gcc (OpenMP) into oracle/_build/."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + ".tmp%d" % os.getpid()
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", _SRC, "-o", tmp, "-lm"]
        subprocess.check_call(cmd)
        os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.orc_nfft_create.restype = C.c_void_p
        L.orc_nfft_create.argtypes = [C.c_int, _ip, _ip, C.c_int, C.c_long]
        L.orc_nfft_destroy.argtypes = [C.c_void_p]
        L.orc_nfft_set_x.argtypes = [C.c_void_p, _dp]
        L.orc_nfft_trafo.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_nfft_adjoint.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_ndft_trafo.argtypes = [C.c_int, _ip, C.c_long, _dp, _dp, _dp, C.c_int]
        L.orc_ndft_adjoint.argtypes = [C.c_int, _ip, C.c_long, _dp, _dp, _dp, C.c_int]
        L.orc_damp_mask.argtypes = [C.c_int, _ip, _dp]
        L.orc_itrafo.restype = C.c_int
        L.orc_itrafo.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_double, _dp, _dp]
        L.orc_intensity_map.argtypes = [C.c_long, C.c_int, _dp, _dp]
        L.orc_sense_trafo.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int]
        L.orc_sense_adjoint_codeare.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp,
                                                C.c_int, C.c_double, _dp, _dp, C.c_int]
        L.orc_sense_adjoint.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, C.c_int]
        L.orc_cgls_codeare.restype = C.c_int
        L.orc_cgls_codeare.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_double,
                                       C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_int, C.c_int]
        L.orc_cg_sense.restype = C.c_int
        L.orc_cg_sense.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_double, C.c_int, C.c_double,
                                   _dp, _dp, _dp, C.c_int]
        L.orc_kb_phi.restype = C.c_double
        L.orc_kb_phi.argtypes = [C.c_double, C.c_int, C.c_double]
        L.orc_kb_phihut.restype = C.c_double
        L.orc_kb_phihut.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
        L.orc_fft_nd.argtypes = [_dp, C.c_int, _ip, C.c_int]
        L.orc_nfft_trafo_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
        L.orc_nfft_adjoint_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _threads(n):
    return int(n) if n else (os.cpu_count() or 1)


def fft_nd(a, sign):
    a = _c128(a).copy()
    dims = (C.c_int * a.ndim)(*a.shape)
    lib().orc_fft_nd(a.view(np.float64).ctypes.data_as(_dp), a.ndim, dims, int(sign))
    return a


def damp_mask(shape):
    d = len(shape)
    out = np.zeros(shape, dtype=np.float64)
    lib().orc_damp_mask(d, (C.c_int * 3)(*shape, *([0] * (3 - d))), _d(out))
    return out


def intensity_map(S):
    S = _c128(S)
    nc = S.shape[0]
    out = np.zeros(S.shape[1:], dtype=np.float64)
    lib().orc_intensity_map(int(np.prod(S.shape[1:])), nc, _d(S.view(np.float64)), _d(out))
    return out


def ndft_trafo(x, fhat, threads=0):
    """f_j = sum_k fhat_k exp(-2 pi i k.x_j); x: (M, d), fhat: N^d."""
    x = _f64(x); fhat = _c128(fhat)
    d = fhat.ndim
    M = x.shape[0]
    f = np.zeros(M, dtype=np.complex128)
    lib().orc_ndft_trafo(d, (C.c_int * 3)(*fhat.shape, *([0] * (3 - d))), M, _d(x),
                         _d(fhat.view(np.float64)), _d(f.view(np.float64)), _threads(threads))
    return f


def ndft_adjoint(x, f, shape, threads=0):
    x = _f64(x); f = _c128(f)
    d = len(shape)
    out = np.zeros(shape, dtype=np.complex128)
    lib().orc_ndft_adjoint(d, (C.c_int * 3)(*shape, *([0] * (3 - d))), x.shape[0], _d(x),
                           _d(f.view(np.float64)), _d(out.view(np.float64)), _threads(threads))
    return out


class NFFT:
    """FP64 restatement of one NFFT3-style plan (KB window, 2m+2 taps)."""

    def __init__(self, shape, M, m=1, alpha=1.0, n=None):
        self.shape = tuple(int(s) for s in shape)
        self.d = len(self.shape)
        if n is None:
            n = tuple(int(np.ceil(alpha * s)) for s in self.shape)
        self.n = tuple(int(v) for v in n)
        self.m = int(m)
        self.M = int(M)
        pad = [0] * (3 - self.d)
        self._p = lib().orc_nfft_create(self.d, (C.c_int * 3)(*self.shape, *pad),
                                        (C.c_int * 3)(*self.n, *pad), self.m, self.M)
        if not self._p:
            raise ValueError("bad NFFT parameters")
        self.Nt = int(np.prod(self.shape))

    def __del__(self):
        p = getattr(self, "_p", None)
        if p and _lib is not None:
            _lib.orc_nfft_destroy(p)
            self._p = None

    def set_x(self, x):
        x = _f64(x).reshape(self.M, self.d)
        self._x = x
        lib().orc_nfft_set_x(self._p, _d(x))

    def trafo(self, fhat):
        fhat = _c128(fhat).reshape(self.shape)
        f = np.zeros(self.M, dtype=np.complex128)
        lib().orc_nfft_trafo(self._p, _d(fhat.view(np.float64)), _d(f.view(np.float64)))
        return f

    def adjoint(self, f):
        f = _c128(f).reshape(self.M)
        out = np.zeros(self.shape, dtype=np.complex128)
        lib().orc_nfft_adjoint(self._p, _d(f.view(np.float64)), _d(out.view(np.float64)))
        return out

    def trafo_batch(self, fhat, threads=0):
        """NC independent trafos (one thread per coil); fhat: (NC,) + shape"""
        fhat = _c128(fhat)
        nc = fhat.shape[0]
        f = np.zeros((nc, self.M), dtype=np.complex128)
        lib().orc_nfft_trafo_batch(self._p, nc, _d(fhat.view(np.float64)), _d(f.view(np.float64)),
                                   _threads(threads))
        return f

    def adjoint_batch(self, f, threads=0):
        f = _c128(f)
        nc = f.shape[0]
        out = np.zeros((nc,) + self.shape, dtype=np.complex128)
        lib().orc_nfft_adjoint_batch(self._p, nc, _d(f.view(np.float64)), _d(out.view(np.float64)),
                                     _threads(threads))
        return out

    def itrafo(self, y, w, what, maxit=3, eps=1e-3):
        """CGNR inverse NFFT as codeare's NFFT::Adjoint; returns (fhat, dot_r, steps)."""
        y = _c128(y).reshape(self.M)
        w = None if w is None else _f64(w).reshape(self.M)
        what = None if what is None else _f64(what).reshape(self.shape)
        out = np.zeros(self.shape, dtype=np.complex128)
        dr = np.zeros(1)
        steps = lib().orc_itrafo(self._p, _d(y.view(np.float64)), None if w is None else _d(w),
                                 None if what is None else _d(what), int(maxit), float(eps),
                                 _d(out.view(np.float64)), _d(dr))
        return out, float(dr[0]), int(steps)


class Sense:
    """FP64 NCSENSE restatement: NC coils sharing one NFFT plan."""

    def __init__(self, S, kx, w=None, m=1, alpha=1.0, threads=0):
        self.S = _c128(S)
        self.nc = self.S.shape[0]
        self.shape = self.S.shape[1:]
        kx = _f64(kx)
        self.M = kx.size // len(self.shape)
        self.nfft = NFFT(self.shape, self.M, m=m, alpha=alpha)
        self.nfft.set_x(kx)
        self.w = None if w is None else _f64(w).reshape(self.M)
        self.what = damp_mask(self.shape)
        self.I = intensity_map(self.S)
        self.data_shape = (self.nc, self.M)
        self.threads = _threads(threads)

    def _S(self):
        return _d(self.S.view(np.float64))

    def trafo(self, x):
        x = _c128(x).reshape(self.shape)
        y = np.zeros((self.nc, self.M), dtype=np.complex128)
        lib().orc_sense_trafo(self.nfft._p, self.nc, self._S(), _d(x.view(np.float64)),
                              _d(y.view(np.float64)), self.threads)
        return y

    def adjoint_codeare(self, y, ftiter=3, fteps=1e-3):
        y = _c128(y).reshape(self.nc, self.M)
        x = np.zeros(self.shape, dtype=np.complex128)
        lib().orc_sense_adjoint_codeare(self.nfft._p, self.nc, self._S(), _d(self.I),
                                        None if self.w is None else _d(self.w), _d(self.what),
                                        int(ftiter), float(fteps), _d(y.view(np.float64)),
                                        _d(x.view(np.float64)), self.threads)
        return x

    def adjoint(self, y, weighted=True):
        y = _c128(y).reshape(self.nc, self.M)
        x = np.zeros(self.shape, dtype=np.complex128)
        w = self.w if weighted else None
        lib().orc_sense_adjoint(self.nfft._p, self.nc, self._S(), None if w is None else _d(w),
                                _d(y.view(np.float64)), _d(x.view(np.float64)), self.threads)
        return x

    def cgls_codeare(self, y, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3, refprec=False):
        y = _c128(y).reshape(self.nc, self.M)
        x = np.zeros(self.shape, dtype=np.complex128)
        res = np.zeros(max(cgiter, 1), dtype=np.float64)
        n = lib().orc_cgls_codeare(self.nfft._p, self.nc, self._S(), _d(self.I),
                                   None if self.w is None else _d(self.w), _d(self.what),
                                   int(ftiter), float(fteps), int(cgiter), float(cgeps), float(lam),
                                   _d(y.view(np.float64)), _d(x.view(np.float64)), _d(res),
                                   int(bool(refprec)), self.threads)
        return x, res[:n]

    def cg(self, y, maxit=10, tol=1e-6, lam=0.0, weighted=True):
        y = _c128(y).reshape(self.nc, self.M)
        x = np.zeros(self.shape, dtype=np.complex128)
        res = np.zeros(maxit + 1, dtype=np.float64)
        w = self.w if weighted else None
        n = lib().orc_cg_sense(self.nfft._p, self.nc, self._S(), None if w is None else _d(w),
                               float(lam), int(maxit), float(tol), _d(y.view(np.float64)),
                               _d(x.view(np.float64)), _d(res), self.threads)
        return x, res[:n + 1]


class FramesSense:
    """NCSENSE with dim4 (x dim5) frames (NCSENSE.hpp:141-166, 204-348): frame
    f has its own trajectory ks[f]; every frame shares the sensitivities and
    the weights.  Images (F, *shape), data (F, NC, M); CGLS (CGLS.hpp:30-59)
    runs over the stacked frames.  With S a list of per-frame maps it is the
    3rd_dim_cart stack instead (NCSENSE.hpp:81-97, 105; NFFT.hpp:100-103,
    335-358, 382-410): every slice a 2-D problem with its own slice of the
    maps, the CG over the whole stack."""

    def __init__(self, S, ks, w=None, m=1, alpha=1.0, threads=0):
        Ss = list(S) if isinstance(S, (list, tuple)) else [S] * len(ks)
        self.frames = [Sense(Sf, k, w=w, m=m, alpha=alpha, threads=threads) for Sf, k in zip(Ss, ks)]
        s0 = self.frames[0]
        self.F, self.nc, self.M = len(self.frames), s0.nc, s0.M
        self.shape = (self.F,) + tuple(s0.shape)
        self.data_shape = (self.F, self.nc, self.M)

    def trafo(self, x):
        x = np.asarray(x).reshape(self.shape)
        return np.stack([s.trafo(x[f]) for f, s in enumerate(self.frames)])

    def adjoint_codeare(self, y, ftiter=3, fteps=1e-3):
        y = np.asarray(y).reshape(self.data_shape)
        return np.stack([s.adjoint_codeare(y[f], ftiter, fteps) for f, s in enumerate(self.frames)])

    def cgls_codeare(self, y, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3):
        """CGLS.hpp:30-59 in FP64 over the stacked frames"""
        A = lambda v: self.adjoint_codeare(v, ftiter, fteps)
        p = A(y)
        if cgiter == 0:
            return p, np.zeros(0)
        r = p.copy()
        rn = xn = float(np.vdot(r, p).real)
        x = np.zeros_like(p)
        res = []
        for _ in range(cgiter):
            q = rn / xn
            res.append(q)
            if np.isnan(q) or q <= cgeps:
                break
            q = A(self.trafo(p)) + lam * p
            ts = rn / float(np.vdot(p, q).real)
            x += ts * p
            r -= ts * q
            rno, rn = rn, float(np.vdot(r, r).real)
            p = r + (rn / rno) * p
        return x, np.array(res)


# ---------------------------------------------------------------------------
# pure-numpy cross-checks for tiny cases (independent of the C code)
# ---------------------------------------------------------------------------
def ndft_matrix(x, shape):
    """Dense NDFT matrix A[j, k] = exp(-2 pi i k.x_j), k over the centred grid."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, len(shape))
    grids = np.meshgrid(*[np.arange(s) - s // 2 for s in shape], indexing="ij")
    kk = np.stack([g.reshape(-1) for g in grids], axis=1).astype(np.float64)
    return np.exp(-2j * np.pi * (x @ kk.T))
