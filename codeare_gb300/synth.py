"""Seeded synthetic inputs for the CG-SENSE workloads (no public dataset is involved).

Shapes, orders and value ranges follow the reference's data exchange
(src/modules/CGSENSE.cpp:132-179): `kspace` is (d, M) float with row 0 the
slowest image axis, `weights` is (M,), `sensitivities` is (N.., NC) and
`signals` is (M, NC), all column-major in codeare.  Here every array is
returned in the C order that has the same memory image:
    image  (N0, N1[, N2])   complex64, last axis fastest (codeare's first index)
    sens   (NC, N0, N1[, N2]) complex64
    k      (M, d) float32   k[j, t] in [-0.5, 0.5), t = 0 slowest image axis
    w      (M,) float32
"""
from __future__ import annotations

import math

import numpy as np

SEED_BASE = 20261203

# Shepp-Logan ellipses as tabulated by the reference (src/matrix/Creators.hpp:459-475):
# (semi-axis a0, semi-axis a1, centre offset 0, centre offset 1, angle), intensity.
_SL_GEOM = [
    (.69, .92, .0, .0, .0), (.6624, .874, .0, -.0184, .0), (.11, .31, -.22, .0, -.3),
    (.16, .41, .22, .0, .3), (.21, .25, .0, .35, .0), (.046, .046, .00, .1, .0),
    (.046, .046, .0, -.1, .0), (.046, .023, .08, -.605, .0), (.023, .023, .0, -.606, .0),
    (.023, .046, -.06, -.605, .0),
]
_SL_VAL = [1., -.8, -.2, -.2, .1, .1, .1, .1, .1, .1]


def phantom(n: int) -> np.ndarray:
    """2-D Shepp-Logan phantom with the reference's float arithmetic
    (src/matrix/Creators.hpp:369-395, 453-490).  Returns P[r, c] (c fastest)."""
    res = np.zeros((n, n), dtype=np.complex64)
    r = np.arange(n, dtype=np.float32)[:, None]
    c = np.arange(n, dtype=np.float32)[None, :]
    fn = np.float32(n)
    for p, v in zip(_SL_GEOM, _SL_VAL):
        p = [np.float32(q) for q in p]
        a0 = p[0] * fn / np.float32(2.0)
        a1 = p[1] * fn / np.float32(2.0)
        m0 = (np.float32(1.0) - p[2]) * fn / np.float32(2.0)
        m1 = (np.float32(1.0) - p[3]) * fn / np.float32(2.0)
        cosp = np.float32(math.cos(p[4]))
        sinp = np.float32(math.sin(p[4]))
        x = ((c - m1) * cosp + (r - m0) * sinp) / a1
        y = ((r - m0) * cosp - (c - m1) * sinp) / a0
        res += np.where(x * x + y * y <= np.float32(1.0), np.complex64(v), np.complex64(0))
    return res


_SL3_GEOM = [
    (.69, .92, .9, .0, .0, .0, .0), (.662, .874, .88, .0, .0, .0, .0),
    (.11, .31, .22, -.22, .0, -.25, -.3), (.16, .41, .21, .22, .0, -.25, .3),
    (.21, .25, .5, .0, .35, -.25, .0), (.046, .046, .046, .0, .1, -.25, .0),
    (.046, .023, .02, .08, -.65, -.25, .0), (.046, .023, .02, .06, -.65, -.25, .0),
    (.056, .04, .1, -.06, -.105, .625, .0), (.056, .056, .1, .0, .1, .625, .0),
]
_SL3_VAL = [2., -.8, -.2, -.2, .2, .2, .1, .1, .2, -.2]


def phantom3d(n: int) -> np.ndarray:
    """3-D Shepp-Logan (Koay et al. 2007 table as in src/matrix/Creators.hpp:511-537).

    The reference's `ellipsoid` (Creators.hpp:408-437) shadows its intensity
    argument with the slice index, so its voxels carry the slice number; this
    restatement uses the tabulated intensities instead.  Returns P[s, r, c].
    """
    res = np.zeros((n, n, n), dtype=np.complex64)
    s = np.arange(n, dtype=np.float32)[:, None, None]
    r = np.arange(n, dtype=np.float32)[None, :, None]
    c = np.arange(n, dtype=np.float32)[None, None, :]
    fn = np.float32(n)
    for p, v in zip(_SL3_GEOM, _SL3_VAL):
        p = [np.float32(q) for q in p]
        a = [p[i] * fn / np.float32(2.0) for i in range(3)]
        m = [(np.float32(1.0) - p[3 + i]) * fn / np.float32(2.0) for i in range(3)]
        cosp = np.float32(math.cos(p[6]))
        sinp = np.float32(math.sin(p[6]))
        x = ((c - m[1]) * cosp + (r - m[0]) * sinp) / a[1]
        y = ((r - m[0]) * cosp - (c - m[1]) * sinp) / a[0]
        z = (s - m[2]) / a[2]
        res += np.where(x * x + y * y + z * z <= np.float32(1.0), np.complex64(v), np.complex64(0))
    return res


def _positions(shape):
    """pixel centres in FOV units, each axis in [-0.5, 0.5)"""
    axes = [(np.arange(s, dtype=np.float64) - s // 2) / s for s in shape]
    return np.meshgrid(*axes, indexing="ij")


def coils2d(n: int, nc: int, sigma: float = 0.4, radius: float = 0.6) -> np.ndarray:
    """Smooth complex Gaussian sensitivities, centre c at angle 2 pi c / nc on a
    circle of `radius` FOV, with a phase linear in that angle plus a gentle
    linear ramp along the coil direction."""
    Y, X = _positions((n, n))
    out = np.empty((nc, n, n), dtype=np.complex64)
    for c in range(nc):
        th = 2.0 * np.pi * c / nc
        cy, cx = radius * np.sin(th), radius * np.cos(th)
        mag = np.exp(-((Y - cy) ** 2 + (X - cx) ** 2) / (2.0 * sigma ** 2))
        ph = th + 0.5 * np.pi * (Y * np.sin(th) + X * np.cos(th))
        out[c] = (mag * np.exp(1j * ph)).astype(np.complex64)
    return out


def coils3d(n: int, nc: int, sigma: float = 0.45, radius: float = 0.6) -> np.ndarray:
    """Gaussian sensitivities centred on a Fibonacci sphere of `radius` FOV."""
    Z, Y, X = _positions((n, n, n))
    out = np.empty((nc, n, n, n), dtype=np.complex64)
    ga = np.pi * (3.0 - np.sqrt(5.0))
    for c in range(nc):
        zc = 1.0 - 2.0 * (c + 0.5) / nc
        rc = np.sqrt(max(0.0, 1.0 - zc * zc))
        ph0 = ga * c
        cz, cy, cx = radius * zc, radius * rc * np.sin(ph0), radius * rc * np.cos(ph0)
        mag = np.exp(-((Z - cz) ** 2 + (Y - cy) ** 2 + (X - cx) ** 2) / (2.0 * sigma ** 2))
        out[c] = (mag * np.exp(1j * (ph0 + 0.5 * np.pi * (Z * zc + Y * np.sin(ph0) + X * np.cos(ph0))))).astype(np.complex64)
    return out


def _clip_k(k):
    return np.clip(k, -0.5, np.nextafter(np.float32(0.5), np.float32(0))).astype(np.float32)


def radial2d(nspokes: int, nsamp: int, golden: bool = False) -> np.ndarray:
    """Radial spokes through the centre; k = (i - nsamp/2)/nsamp along each spoke.
    Uniform angles pi*s/nspokes, or golden-angle increments of pi*(sqrt5-1)/2."""
    if golden:
        ang = np.mod(np.arange(nspokes) * np.pi * (np.sqrt(5.0) - 1.0) / 2.0, np.pi)
    else:
        ang = np.pi * np.arange(nspokes) / nspokes
    kr = (np.arange(nsamp, dtype=np.float64) - nsamp // 2) / nsamp
    ky = np.sin(ang)[:, None] * kr[None, :]
    kx = np.cos(ang)[:, None] * kr[None, :]
    return _clip_k(np.stack([ky.ravel(), kx.ravel()], axis=1))


def spiral2d(ninter: int, nsamp: int, density_exp: float = 1.5, turns: float = 16.0) -> np.ndarray:
    """Variable-density Archimedean-type spiral: |k| = 0.5 (t)^alpha, t in [0,1)."""
    t = np.arange(nsamp, dtype=np.float64) / nsamp
    r = 0.5 * t ** density_exp
    out = []
    for i in range(ninter):
        th = 2.0 * np.pi * turns * t + 2.0 * np.pi * i / ninter
        out.append(np.stack([r * np.sin(th), r * np.cos(th)], axis=1))
    return _clip_k(np.concatenate(out, axis=0))


def spiral_weights(k: np.ndarray, ninter: int) -> np.ndarray:
    """density compensation for interleaved spirals: the area |k x dk/dt| swept
    per sample, scaled to a maximum of 0.5 (the ramp's maximum)"""
    kk = k.astype(np.float64).reshape(ninter, -1, 2)
    g = np.gradient(kk, axis=1)
    w = np.abs(kk[..., 0] * g[..., 1] - kk[..., 1] * g[..., 0]).ravel()
    return (0.5 * w / max(float(w.max()), 1e-30)).astype(np.float32)


def kooshball3d(nspokes: int, nsamp: int) -> np.ndarray:
    """3-D radial spokes with directions on a Fibonacci hemisphere."""
    i = np.arange(nspokes, dtype=np.float64)
    z = 1.0 - (i + 0.5) / nspokes
    rr = np.sqrt(1.0 - z * z)
    ph = i * np.pi * (3.0 - np.sqrt(5.0))
    d = np.stack([z, rr * np.sin(ph), rr * np.cos(ph)], axis=1)
    kr = (np.arange(nsamp, dtype=np.float64) - nsamp // 2) / nsamp
    k = d[:, None, :] * kr[None, :, None]
    return _clip_k(k.reshape(-1, 3))


def ramp_weights(k: np.ndarray) -> np.ndarray:
    """density compensation |k| (ramp)"""
    return np.sqrt(np.sum(k.astype(np.float64) ** 2, axis=1)).astype(np.float32)


def add_noise(y: np.ndarray, rel: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    s = rel * float(np.abs(y).max())
    n = rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)
    return (y + s * n).astype(np.complex64)


def radial2d_128_8coils():
    """128^2 Shepp-Logan, 8 coils, 96 uniform spokes x 256, sigma=2, m=4, 10 CG iterations."""
    N, nc = 128, 8
    k = radial2d(96, 256)
    return dict(name="radial2d_128_8c", shape=(N, N), image=phantom(N), sens=coils2d(N, nc),
                k=k, w=ramp_weights(k), alpha=2.0, m=4, cgiter=10, cgeps=1e-6,
                noise=1e-3, seed=SEED_BASE + 0)


def radial2d_256_32coils():
    """NuFFT operator alone: 256^2, 32 coils, golden-angle 403 x 512, sigma=2, m=4."""
    N, nc = 256, 32
    k = radial2d(403, 512, golden=True)
    return dict(name="nufft_256_32c_ga403x512", shape=(N, N), image=phantom(N),
                sens=coils2d(N, nc), k=k, w=ramp_weights(k), alpha=2.0, m=4,
                seed=SEED_BASE + 1)


def kooshball3d_128_16coils(N: int = 128, nc: int = 16, nspokes: int = 20000, nsamp: int = 256):
    """3-D kooshball CG-SENSE: 128^3 3-D Shepp-Logan (tabulated intensities),
    16 Gaussian coils (sigma 0.45 FOV) on a Fibonacci sphere, 20000 spokes x 256
    samples, density compensation |k|^2 (3-D radial), noise-free data, sigma=2,
    m=4, standard CG to ||r||/||r0|| = 1e-4 with the Toeplitz-embedded E^H W E.  Smaller
    arguments give the reduced cases the FP64 oracle can finish."""
    k = kooshball3d(nspokes, nsamp)
    w = (ramp_weights(k).astype(np.float64) ** 2).astype(np.float32)
    return dict(name="kooshball_%d_%dc_%dx%d" % (N, nc, nspokes, nsamp), shape=(N, N, N), image=phantom3d(N),
                sens=coils3d(N, nc), k=k, w=w, alpha=2.0, m=4, cgeps=1e-4, noise=0.0, seed=SEED_BASE + 3)


def kooshball3d_64_downsample():
    """The 64^3 downsample of the 128^3 kooshball workload: every length halved
    (64^3 phantom, 5000 spokes x 128 samples, the same spokes per N^2 and the
    same 2x readout oversampling), 16 coils, |k|^2 weights, sigma=2, m=4."""
    return kooshball3d_128_16coils(N=64, nc=16, nspokes=5000, nsamp=128)


def uneven_batch(count: int = 64, seed: int = SEED_BASE + 2):
    """Batched uneven CG-SENSE: per problem N in 96..320 (step 32), NC in
    {4, 8, 16, 32}, golden-angle radial 32..400 spokes x 512; every fourth
    problem a variable-density spiral (16 interleaves x 4096, exponent 1.5).
    Shepp-Logan images, sigma=2, m=4, 15 CG iterations, 1e-3 noise."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        N = int(rng.choice(np.arange(96, 321, 32)))
        nc = int(rng.choice([4, 8, 16, 32]))
        if i % 4 == 3:
            k = spiral2d(16, 4096, density_exp=1.5)
            w, kind = spiral_weights(k, 16), "spiral16x4096"
        else:
            spokes = int(rng.integers(32, 401))
            k = radial2d(spokes, 512, golden=True)
            w, kind = ramp_weights(k), "radial%dx512" % spokes
        out.append(dict(name="uneven_%02d_%d_%dc_%s" % (i, N, nc, kind), shape=(N, N), N=N, nc=nc, kind=kind,
                        k=k, w=w, alpha=2.0, m=4, cgiter=15, noise=1e-3, seed=seed + 1000 * i))
    return out


def small_config(N=32, nc=4, nspokes=24, nsamp=64, alpha=2.0, m=4, golden=True, seed=7):
    """A size the FP64 oracle finishes in well under a second."""
    k = radial2d(nspokes, nsamp, golden=golden)
    return dict(name="small", shape=(N, N), image=phantom(N), sens=coils2d(N, nc), k=k,
                w=ramp_weights(k), alpha=alpha, m=m, seed=seed)
