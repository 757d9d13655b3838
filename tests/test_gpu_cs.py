"""Compressed sensing over the NCSENSE operator (codeare's CS_XSENSE with
ft = 3 and NLCG) on the GPU, against the FP64 restatement in oracle/cs.py.

The objective and gradient are compared term by term at fixed inputs; the
whole reconstruction is compared through the NLCG path it takes (the
accepted line-search index of every iteration must agree) and its image.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_OBJ = 2e-5    # objective: FP32 terms, FP64 sums
TOL_GRAD = 2e-4   # gradient: one codeare CGLS solve inside (its parity bar is 1e-4)
TOL_IMG = 2e-3    # reconstruction after several NLCG steps, each with a solve


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def setup_2d(cg, N=32, nc=4):
    from codeare_gb300 import synth
    from oracle import oracle as O
    cfg = synth.small_config(N=N, nc=nc, nspokes=32, nsamp=64, alpha=1.0, m=1)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = O.Sense(S, k, w=w, m=1, alpha=1.0)
    y = synth.add_noise(s.trafo(cfg["image"]), 1e-3, seed=4)
    p = cg.Plan((N, N), k.shape[0], ncoils=nc, m=1, alpha=1.0)
    p.set_kspace(np.ascontiguousarray(k, np.float32))
    p.set_weights(np.ascontiguousarray(w, np.float32))
    p.set_sensitivities(c64(S))
    return s, p, c64(y), cfg["image"]


def setup_3d(cg, N=16, nc=2):
    from codeare_gb300 import synth
    from oracle import oracle as O
    k = synth.kooshball3d(300, 32)
    w = synth.ramp_weights(k) ** 2 + 1e-3
    S = synth.coils3d(N, nc)
    s = O.Sense(S, k, w=w, m=1, alpha=1.0)
    y = synth.add_noise(s.trafo(synth.phantom3d(N)), 1e-3, seed=5)
    p = cg.Plan((N, N, N), k.shape[0], ncoils=nc, m=1, alpha=1.0)
    p.set_kspace(np.ascontiguousarray(k, np.float32))
    p.set_weights(np.ascontiguousarray(w, np.float32))
    p.set_sensitivities(c64(S))
    return s, p, c64(y)


SOLVE = dict(cgiter=6, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
TERMS_2D = [
    dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-15, pnorm=1.0),
    dict(tvw=(1e-2, 5e-3), tvdims=([1, 1], None), xfmw=0.0, l1=1e-6, pnorm=1.5),
    dict(tvw=(0.0, 0.0), xfmw=1e-2, l1=1e-4, pnorm=2.0),
]
TERMS_3D = [
    dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-15, pnorm=1.0),                 # TV3D, every axis
    dict(tvw=(3e-3, 1e-3), tvdims=([0, 0, 1], None), l1=1e-8, pnorm=1.0),  # third axis + every axis
]


def rand_img(shape, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    return c64(scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))


def check_obj_and_df(cg, s, p, y, terms, shape):
    from oracle import cs
    o = cs.CSXSense(s, **terms, **SOLVE)
    g = cg.CS(p, **terms, **SOLVE)
    x0 = np.zeros(shape, np.complex64)
    p.solve(y, x0, cgiter=SOLVE["cgiter"], cgeps=SOLVE["cgeps"], lam=SOLVE["lam"])
    dx = rand_img(shape, 3, scale=0.1 * float(np.abs(x0).max()))
    o.set_data(y)
    go = o.df(x0)
    gg = np.zeros(shape, np.complex64)
    g.df(y, x0, gg)
    assert rel(gg, go) < TOL_GRAD
    o.update(dx)
    for t in (0.0, 0.36, 1.0):
        fo, ro = o.obj(x0, dx, t)
        fg, rg = g.obj(y, x0, dx, t)
        assert abs(fg - fo) <= TOL_OBJ * abs(fo), (t, fg, fo)
        assert abs(rg - ro) <= TOL_OBJ * ro


@pytest.mark.parametrize("case", range(len(TERMS_2D)))
def test_cs_obj_and_df_2d(gpu, case):
    s, p, y, _ = setup_2d(gpu)
    check_obj_and_df(gpu, s, p, y, TERMS_2D[case], (32, 32))


@pytest.mark.parametrize("case", range(len(TERMS_3D)))
def test_cs_obj_and_df_3d(gpu, case):
    s, p, y = setup_3d(gpu)
    check_obj_and_df(gpu, s, p, y, TERMS_3D[case], (16, 16, 16))


@pytest.mark.parametrize("pls", [False, True])
def test_cs_reconstruction_matches_oracle(gpu, pls):
    """CS_XSENSE::Adjoint with NLCG: same line-search path, same image."""
    from oracle import cs
    s, p, y, _ = setup_2d(gpu)
    kw = dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-15, pnorm=1.0, csiter=2, nliter=4, lsiter=10, lsa=1e-3,
              lsb=0.6, cgconv=1e-5, parallel_linesearch=pls, **SOLVE)
    o = cs.CSXSense(s, **kw)
    xo = o.adjoint(y)
    g = gpu.CS(p, **kw)
    x = np.zeros((32, 32), np.complex64)
    rep = g.adjoint(y, x)
    assert rep["ls_index"] == [li for li, _ in o.log]
    assert np.allclose(rep["rmse"], [r for _, r in o.log], rtol=1e-3)
    assert abs(rep["tvw_used"][0] - o.tvw[0]) <= 1e-5 * o.tvw[0]
    assert rel(x, xo) < TOL_IMG
    assert rep["solves"] >= 1 + rep["iterations"]


def test_split_bregman_is_the_cgls_image(gpu):
    """nlopt = 2: the reference's Split Bregman minimiser is empty, so the
    result is the CG-SENSE solve of the data."""
    s, p, y, _ = setup_2d(gpu)
    x = np.zeros((32, 32), np.complex64)
    rep = gpu.CS(p, tvw=(2e-3, 0.0), nlopt=2, csiter=3, **SOLVE).adjoint(y, x)
    ref = np.zeros_like(x)
    p.solve(y, ref, cgiter=SOLVE["cgiter"], cgeps=SOLVE["cgeps"], lam=SOLVE["lam"])
    assert np.array_equal(x, ref)
    assert rep["iterations"] == 0 and rep["solves"] == 1


def test_cs_rejects_unsupported_settings(gpu):
    s, p, y, _ = setup_2d(gpu)
    with pytest.raises(gpu.capi.CgsError):
        gpu.CS(p, nlopt=1)                        # L-BFGS
    for fam, mem in ((0, 6), (1, 4), (2, 4), (4, 2)):
        with pytest.raises(gpu.capi.CgsError):    # wavelets without filters in the reference
            gpu.CS(p, wl_family=fam, wl_member=mem)
    with pytest.raises(gpu.capi.CgsError):
        gpu.CS(p, tvw=(1e-3, 0.0), tvdims=([0, 0, 1], None))  # third-axis TV on a 2-D image
    s3, p3, y3 = setup_3d(gpu)
    with pytest.raises(gpu.capi.CgsError):
        gpu.CS(p3, wl_family=0, wl_member=4)      # the reference's DWT is 2-D


WAVELETS = [(0, 4), (0, 8), (2, 2)]


@pytest.mark.parametrize("fam,mem", WAVELETS)
@pytest.mark.parametrize("N", [32, 64])
def test_wavelet_transform_matches_oracle(gpu, fam, mem, N):
    """DWT::operator* and ->* (DWT.hpp:354-418, 756-823): forward and inverse
    against the FP64 restatement; the inverse undoes the forward."""
    from oracle import cs
    s, p, y, _ = setup_2d(gpu, N=N, nc=2)
    g = gpu.CS(p, wl_family=fam, wl_member=mem, **SOLVE)
    x = rand_img((N, N), 11)
    w = np.zeros_like(x)
    g.wavelet(x, w)
    lo, hi = cs.wavelet_filters(fam, mem)
    wo = cs.dwt_fwd(x.T, lo, hi).T
    assert rel(w, wo) < 2e-6
    xi = np.zeros_like(x)
    g.wavelet(w, xi, inverse=True)
    assert rel(xi, cs.dwt_inv(w.T, lo, hi).T) < 2e-6
    assert rel(xi, x) < 4e-6


# With a wavelet each side forms the image W^-1 x itself, the GPU in FP32.
# For p = 1 the TV factor d / sqrt(|d|^2 + l1) has slope 1/sqrt(l1) at d = 0,
# so at l1 = 1e-15 the FP32 rounding noise of the image (~1e-8 in flat
# regions) alone moves the FP64 gradient by several percent -- the
# reference's FP32 code is as sensitive.  These cases use l1 = 1e-6, where
# the same noise moves it by ~4e-6.
L1_WAVELET = 1e-6


@pytest.mark.parametrize("fam,mem", WAVELETS)
def test_cs_obj_and_df_wavelet(gpu, fam, mem):
    """With a wavelet the NLCG variable is the coefficient array: the data and
    TV terms act on its inverse transform, the L1 term on the coefficients."""
    from oracle import cs
    s, p, y, _ = setup_2d(gpu, N=64, nc=2)
    terms = dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=L1_WAVELET, pnorm=1.0, wl_family=fam, wl_member=mem)
    o = cs.CSXSense(s, **terms, **SOLVE)
    g = gpu.CS(p, **terms, **SOLVE)
    x0 = np.zeros((64, 64), np.complex64)
    p.solve(y, x0, cgiter=SOLVE["cgiter"], cgeps=SOLVE["cgeps"], lam=SOLVE["lam"])
    w0 = c64(o.W(x0))
    dx = rand_img((64, 64), 3, scale=0.1 * float(np.abs(w0).max()))
    o.set_data(y)
    go = o.df(w0)
    gg = np.zeros_like(w0)
    g.df(y, w0, gg)
    assert rel(gg, go) < TOL_GRAD
    o.update(dx)
    for t in (0.0, 0.36):
        fo, ro = o.obj(w0, dx, t)
        fg, rg = g.obj(y, w0, dx, t)
        assert abs(fg - fo) <= TOL_OBJ * abs(fo), (t, fg, fo)


def test_cs_reconstruction_wavelet_matches_oracle(gpu):
    """The reference's example settings (Daubechies 4, TV and L1 weights,
    p = 1; l1 as above): same line-search path and image as the FP64
    restatement."""
    from oracle import cs
    s, p, y, _ = setup_2d(gpu, N=64, nc=4)
    kw = dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=L1_WAVELET, pnorm=1.0, csiter=2, nliter=4, lsiter=10, lsa=1e-3,
              lsb=0.6, cgconv=1e-5, wl_family=0, wl_member=4, **SOLVE)
    o = cs.CSXSense(s, **kw)
    xo = o.adjoint(y)
    x = np.zeros((64, 64), np.complex64)
    rep = gpu.CS(p, **kw).adjoint(y, x)
    assert rep["ls_index"] == [li for li, _ in o.log]
    assert rel(x, xo) < TOL_IMG


def setup_nfft(cg, N=32, m=1, alpha=1.0):
    """single-coil NFFT data for CS with ft = 2"""
    from codeare_gb300 import synth
    from oracle import cs
    k = synth.radial2d(24, 64, golden=True)
    w = synth.ramp_weights(k)
    op = cs.NFFTOp((N, N), k, w=w, m=m, alpha=alpha)
    y = c64(synth.add_noise(op.trafo(synth.phantom(N)), 1e-3, seed=6))
    p = cg.Plan((N, N), k.shape[0], ncoils=1, m=m, alpha=alpha)
    p.set_kspace(np.ascontiguousarray(k, np.float32))
    p.set_weights(np.ascontiguousarray(w, np.float32))
    return op, p, y


@pytest.mark.parametrize("m,alpha", [(1, 1.0), (4, 2.0)])
def test_cs_over_nfft_matches_oracle(gpu, m, alpha):
    """ft = 2 (CompressedSensing.cpp:73-85): E is the single-coil NFFT and its
    ->* the CGNR inverse NFFT (ftiter steps, threshold fteps)."""
    from oracle import cs
    op, p, y = setup_nfft(gpu, m=m, alpha=alpha)
    kw = dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-6, pnorm=1.0, csiter=2, nliter=5, lsiter=8, lsa=1e-3, lsb=0.6,
              cgconv=1e-5, ftiter=3, fteps=7e-4, ft=2)
    o = cs.CSXSense(op, **kw)
    g = gpu.CS(p, **kw)
    x0 = np.zeros((1, 32, 32), np.complex64)
    p.nfft_itrafo(y, x0, maxit=3, eps=7e-4)
    x0 = x0[0]
    o.set_data(y)
    go = o.df(x0)
    gg = np.zeros_like(x0)
    g.df(y, x0, gg)
    assert rel(gg, go) < TOL_GRAD
    dx = rand_img((32, 32), 5, scale=0.1 * float(np.abs(x0).max()))
    o.update(dx)
    fo, _ = o.obj(x0, dx, 0.36)
    fg, _ = g.obj(y, x0, dx, 0.36)
    assert abs(fg - fo) <= TOL_OBJ * abs(fo)
    o2 = cs.CSXSense(op, **kw)
    xo = o2.adjoint(y)
    x = np.zeros_like(x0)
    rep = gpu.CS(p, **kw).adjoint(y, x)
    assert rep["ls_index"] == [li for li, _ in o2.log]
    assert rel(x, xo) < TOL_IMG
