"""FP64 restatement of codeare's compressed sensing over the NCSENSE operator.

TEST INFRASTRUCTURE ONLY: imported by tests/, which compare the CUDA path
against it; never by the product package.

PARITY UNPINNED: the reference ships no test or golden vector for its CS
code; this restates the reference's source line by line, in FP64, on top of
the NCSENSE restatement in oracle.py.

  TV operators        src/matrix/TVOP.hpp:37-64 (TV2D), 81-131 (TV3D, all
                      axes), 134-166 (TV3D, third axis), 277-318 (dispatch)
  CS objective        src/matrix/ft/CS_XSENSE.hpp:197-255 (obj, df, Update),
                      279-322 (Adjoint), 329-414 (Obj, TV, XFM, dObj, dXFM, dTV)
  NLCG                src/optimisation/NLCG.hpp:42-125
  wavelets            src/matrix/dwt/DWT.hpp:354-418 (forward), 756-823
                      (inverse), 644-740 and 1046-1180 (filters along a line),
                      Wavelet.hpp:12-19, 75-190 (filter sets)
  module keys         src/modules/CompressedSensing.cpp:86-136

Images are numpy arrays in C order, so the codeare (D0, D1[, D2]) image is
the array of shape ([D2,] D1, D0); the TV code works on its transpose, which
indexes like codeare's Matrix.
"""
from __future__ import annotations

import numpy as np


def tv_mode(ndim: int, dims) -> str:
    """TVOP::Trafo's choice of operator (TVOP.hpp:277-295)."""
    dims = list(dims or [])
    if ndim == 2 and (not dims or (len(dims) >= 2 and dims[0] == 1 and dims[1] == 1)):
        return "2d"
    if ndim == 3 and (not dims or (len(dims) >= 3 and dims[:3] == [1, 1, 1])):
        return "3d"
    if ndim == 3 and len(dims) >= 3 and dims[:3] == [0, 0, 1]:
        return "z"
    raise ValueError("no TV operator for %d-D images over axes %s" % (ndim, dims))


def tv_fwd(c, mode):
    """Forward differences of the codeare-ordered image c."""
    if mode == "2d":  # TVOP.hpp:39-50
        r = np.zeros(c.shape + (2,), c.dtype)
        r[:-1, :, 0] = c[1:, :] - c[:-1, :]
        r[:, :-1, 1] = c[:, 1:] - c[:, :-1]
        return r
    if mode == "3d":  # TVOP.hpp:83-99: the third loop writes component 1 again
        r = np.zeros(c.shape + (3,), c.dtype)
        r[:-1, :, :, 0] = c[1:] - c[:-1]
        r[:, :-1, :, 1] = c[:, 1:, :] - c[:, :-1, :]
        r[:, :, :-1, 1] = c[:, :, 1:] - c[:, :, :-1]
        return r
    if mode == "z":  # TVOP.hpp:135-144
        r = np.zeros_like(c)
        r[:, :, :-1] = c[:, :, 1:] - c[:, :, :-1]
        return r
    raise ValueError(mode)


def tv_adj(A, mode):
    """The reference's adjoints: interior ranges only for 2d/3d (their border
    rows stay zero), a complete adjoint for z."""
    if mode == "2d":  # TVOP.hpp:52-63 (square images)
        M, N = A.shape[0], A.shape[1]
        r = np.zeros((M, N), A.dtype)
        r[1:N - 1, :] = A[0:N - 2, :, 0] - A[1:N - 1, :, 0]
        r[:, 1:M - 1] += A[:, 0:M - 2, 1] - A[:, 1:M - 1, 1]
        return r
    if mode == "3d":  # TVOP.hpp:101-118
        M, N, L = A.shape[0], A.shape[1], A.shape[2]
        r = np.zeros((M, N, L), A.dtype)
        r[1:N - 1, :, :] = A[0:N - 2, :, :, 0] - A[1:N - 1, :, :, 0]
        r[:, 1:M - 1, :] += A[:, 0:M - 2, :, 1] - A[:, 1:M - 1, :, 1]
        r[:, :, 1:L - 1] += A[:, :, 0:L - 2, 2] - A[:, :, 1:L - 1, 2]
        return r
    if mode == "z":  # TVOP.hpp:146-165
        L = A.shape[2]
        r = np.zeros_like(A)
        r[:, :, 1:L - 1] = A[:, :, 0:L - 2] - A[:, :, 1:L - 1]
        r[:, :, 0] = -A[:, :, 0]
        r[:, :, L - 1] = A[:, :, L - 2]
        return r
    raise ValueError(mode)


# ---------------------------------------------------------------------------
# periodic orthonormal wavelet transform (src/matrix/dwt/DWT.hpp,
# Wavelet.hpp): the reference initialises filters for Daubechies 4 and 8
# taps (family 0) and Haar (family 2, 2 taps) only
# ---------------------------------------------------------------------------
def daubechies(taps: int):
    """Minimum-phase Daubechies low-pass filter with taps/2 vanishing moments,
    by spectral factorisation of P(y) = sum_k C(p-1+k, k) y^k (Daubechies
    1988), ordered with the large coefficients first and sum sqrt(2)."""
    from math import comb
    p = taps // 2
    poly = np.array([1.0 + 0j])
    for _ in range(p):
        poly = np.convolve(poly, [1.0, 1.0])          # (1 + w)^p, ascending powers
    if p > 1:
        for y in np.roots([comb(p - 1 + k, k) for k in range(p)][::-1]):
            r = np.roots([1.0, -(2.0 - 4.0 * y), 1.0])  # w + 1/w = 2 - 4y
            poly = np.convolve(poly, [-r[np.argmax(np.abs(r))], 1.0])
    h = poly.real
    return h * (np.sqrt(2.0) / h.sum())


def wavelet_filters(family: int, member: int):
    """(low, high) decomposition filters; high[i] = (-1)^i low[i] (Wavelet.hpp:12-19)."""
    if (family, member) not in ((0, 4), (0, 8), (2, 2)):
        raise ValueError("no wavelet filters for family %d member %d" % (family, member))
    lo = daubechies(member)
    return lo, lo * (-1.0) ** np.arange(lo.size)


def _down(b, lo, hi, axis):
    """DWT::downlo / downhi along one axis of the block (DWT.hpp:644-740)."""
    b = np.moveaxis(b, axis, 0)
    n = b.shape[0]
    i = np.arange(n // 2)
    low = sum(lo[h] * b[(2 * i + h) % n] for h in range(lo.size))
    high = sum(hi[h] * b[(2 * i + 1 - h) % n] for h in range(hi.size))
    return np.moveaxis(np.concatenate([low, high]), 0, axis)


def _up(b, lo, hi, axis):
    """DWT::uplo + uphi along one axis (DWT.hpp:1046-1180), even filter lengths."""
    b = np.moveaxis(b, axis, 0)
    n = b.shape[0] // 2
    low, high = b[:n], b[n:]
    i = np.arange(n)
    out = np.zeros_like(b)
    for e in (0, 1):
        s = sum(lo[2 * h + e] * low[(i - h) % n] for h in range(lo.size // 2))
        s = s + sum(hi[2 * h + (1 - e)] * high[(i + h) % n] for h in range(hi.size // 2))
        out[e::2] = s
    return np.moveaxis(out, 0, axis)


def dwt_levels(side: int, min_level: int = 4):
    L = int(round(np.log2(side)))
    if 2 ** L != side:
        raise ValueError("the wavelet transform needs dyadic sides")
    return L, min_level


def dwt_fwd(c, lo, hi, min_level=4):
    """DWT::dpwt2 on the codeare-ordered square image c (DWT.hpp:354-418)."""
    L, _ = dwt_levels(c.shape[0], min_level)
    r = np.array(c, dtype=np.complex128)
    n = c.shape[0]
    for _ in range(L - 1, min_level - 1, -1):
        r[:n, :n] = _down(r[:n, :n], lo, hi, 0)
        r[:n, :n] = _down(r[:n, :n], lo, hi, 1)
        n //= 2
    return r


def dwt_inv(c, lo, hi, min_level=4):
    """DWT::idpwt2 (DWT.hpp:756-823): coarse to fine, axis 1 then axis 0."""
    L, _ = dwt_levels(c.shape[0], min_level)
    r = np.array(c, dtype=np.complex128)
    n = 2 ** min_level
    for _ in range(min_level, L):
        r[:2 * n, :2 * n] = _up(r[:2 * n, :2 * n], lo, hi, 1)
        r[:2 * n, :2 * n] = _up(r[:2 * n, :2 * n], lo, hi, 0)
        n *= 2
    return r


class NFFTOp:
    """codeare's NFFT operator as CS_XSENSE uses it with ft = 2: * is the NFFT,
    ->* its CGNR inverse with the density weights and the damping mask
    (NFFT.hpp:305-436), one coil."""

    def __init__(self, shape, k, w=None, m=1, alpha=1.0):
        from . import oracle as O
        self.shape = tuple(shape)
        self.M = int(np.asarray(k).size // len(self.shape))
        self.nfft = O.NFFT(self.shape, self.M, m=m, alpha=alpha)
        self.nfft.set_x(np.asarray(k, np.float64))
        self.w = None if w is None else np.asarray(w, np.float64)
        self.what = O.damp_mask(self.shape)
        self.nc, self.data_shape = 1, (self.M,)

    def trafo(self, x):
        return self.nfft.trafo(np.asarray(x, np.complex128).reshape(self.shape))

    def inverse(self, y, maxit, eps):
        return self.nfft.itrafo(y, self.w, self.what, maxit, eps)[0]


def _pw(v, l1, e):
    """(|v|^2 + l1)^e, the reference's om *= conj(om); om += l1; om ^= e."""
    return (np.abs(v) ** 2 + l1) ** e


class CSXSense:
    """CS_XSENSE<cxfl> with ft = 3 (NCSENSE, `sense` an oracle.Sense or
    FramesSense) or ft = 2 (plain NFFT, `sense` an NFFTOp); with wl_family >= 0 the NLCG
    variable is the image's wavelet coefficients (CS_XSENSE.hpp:131-134)."""

    def __init__(self, sense, tvw=(0.0, 0.0), tvdims=(None, None), xfmw=0.0, l1=0.0, pnorm=0.0,
                 nlopt=0, csiter=1, nliter=4, lsiter=8, lsa=0.01, lsb=0.6, cgconv=1e-4,
                 parallel_linesearch=False, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3,
                 wl_family=-1, wl_member=0, ft=3):
        self.s = sense
        self.ft = ft
        self.filt = wavelet_filters(wl_family, wl_member) if wl_family > -1 else None
        self.nd = len(sense.shape)
        self.tvw = [float(tvw[0]), float(tvw[1])]
        self.modes = [tv_mode(self.nd, tvdims[0]) if tvw[0] else None,
                      tv_mode(self.nd, tvdims[1]) if tvw[1] else None]
        self.xfmw, self.l1, self.p = float(xfmw), float(l1), float(pnorm)
        self.nlopt, self.csiter, self.nliter, self.lsiter = nlopt, csiter, nliter, lsiter
        self.lsa, self.lsb, self.cgconv, self.pls = float(lsa), float(lsb), float(cgconv), parallel_linesearch
        self.solve = dict(cgiter=cgiter, cgeps=cgeps, lam=lam, ftiter=ftiter, fteps=fteps)
        self.log = []

    # the NCSENSE operator: * and ->*
    def E(self, x):
        return self.s.trafo(x)

    def Einv(self, y):
        if self.ft == 2:
            return self.s.inverse(y, self.solve["ftiter"], self.solve["fteps"])
        return self.s.cgls_codeare(y, **self.solve)[0]

    def _c(self, x):  # codeare-ordered view
        return np.asarray(x).T

    # the wavelet operator: * (forward) and ->* (inverse); identity without one
    def W(self, x):
        return x if self.filt is None else dwt_fwd(self._c(x), *self.filt).T

    def Winv(self, x):
        return x if self.filt is None else dwt_inv(self._c(x), *self.filt).T

    def set_data(self, y):
        self.data = np.asarray(y, np.complex128).reshape(self.s.data_shape)
        self.ndnz = float(np.count_nonzero(self.data))

    # CS_XSENSE.hpp:223-232
    def df(self, x):
        self.wx = self.Winv(x)
        g = 2.0 * self.W(self.Einv(self.E(self.wx) - self.data))  # dObj, :367-372
        if self.xfmw:  # dXFM, :383-385
            g = g + self.xfmw * (x * _pw(x, self.l1, 0.5 * self.p - 1.0))
        for i in range(2):
            if self.tvw[i]:  # dTV, :395-405
                d = tv_fwd(self._c(self.wx), self.modes[i])
                G = self.p * (d * _pw(d, self.l1, 0.5 * self.p - 1.0))
                g = g + self.tvw[i] * self.W(tv_adj(G, self.modes[i]).T)
        return g

    # CS_XSENSE.hpp:234-255
    def update(self, dx):
        wdx = self.Winv(dx)
        self.ffdbx = self.E(self.wx)
        self.ffdbg = self.E(wdx)
        self.ttdbx = [tv_fwd(self._c(self.wx), m) if m else None for m in self.modes]
        self.ttdbg = [tv_fwd(self._c(wdx), m) if m else None for m in self.modes]

    # CS_XSENSE.hpp:197-221, 329-365
    def obj(self, x, dx, t):
        om = self.ffdbx + t * self.ffdbg if t > 0 else self.ffdbx
        o = float(np.sum(np.abs(om - self.data) ** 2))
        rmse = np.sqrt(o / self.ndnz)
        for i in range(2):
            if self.tvw[i]:
                u = self.ttdbx[i] + t * self.ttdbg[i] if t > 0 else self.ttdbx[i]
                o += self.tvw[i] * float(np.sum(_pw(u, self.l1, 0.5 * self.p)))
        if self.xfmw:
            u = x + t * dx if t > 0 else x
            o += self.xfmw * float(np.sum(_pw(u, self.l1, 0.5 * self.p)))
        return o, rmse

    # NLCG.hpp:84-125 (the sequential line search, :42-54; with
    # parallel_linesearch the test uses the previous step t, :56-80, and a
    # search that accepts nothing reports the last trial's rmse here, where
    # the reference reads rmses[-1])
    def minimise(self, x):
        t0, t = 1.0, 1.0
        xn = np.linalg.norm(x)
        g0 = self.df(x)
        dx = -g0
        for k in range(self.nliter):
            self.update(dx)
            f0, rmse = self.obj(x, dx, 0.0)
            g0dx = abs(np.vdot(g0, dx))
            li, tprev = self.lsiter, t
            for i in range(self.lsiter):
                ti = t0 * self.lsb ** (i + 1)
                f1, rmse = self.obj(x, dx, ti)  # rmse is an output of every obj call
                if f1 <= f0 - self.lsa * (tprev if self.pls else ti) * g0dx:
                    li, t = i, ti
                    break
            self.log.append((li, rmse))
            if li == self.lsiter:
                return x
            if li > 2:
                t0 *= self.lsb
            elif li < 1:
                t0 /= self.lsb
            x = x + dx * t
            g1 = self.df(x)
            bk = np.vdot(g1, g1).real / np.vdot(g0, g0).real
            g0 = g1
            dx = -g1 + dx * bk
            if np.linalg.norm(dx) / xn < self.cgconv:
                break
        return x

    # CS_XSENSE.hpp:283-322
    def adjoint(self, y):
        self.set_data(y)
        x = self.W(self.Einv(self.data))
        ma = float(np.abs(x).max())
        self.tvw = [w * ma for w in self.tvw]
        for _ in range(self.csiter):
            if self.nlopt == 0:
                x = self.minimise(x)
        return self.Winv(x)
