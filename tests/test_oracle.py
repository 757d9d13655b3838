"""CPU tests of the FP64 oracle (no GPU): pins the restatement to the exact NDFT,
to the Kaiser-Bessel transform pair, and to the committed golden fixtures."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.mark.parametrize("shape", [(448,), (192,), (320,), (640,), (576,), (12, 20), (8, 6, 10)])
def test_fft_matches_numpy(oracle, shape):
    rng = np.random.default_rng(0)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel(oracle.fft_nd(a, -1), np.fft.fftn(a)) < 1e-13
    assert rel(oracle.fft_nd(a, +1), np.fft.ifftn(a) * a.size) < 1e-13


def test_ndft_c_matches_dense_numpy(oracle):
    rng = np.random.default_rng(1)
    N = (8, 10)
    x = rng.uniform(-0.5, 0.5, (50, 2))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    A = oracle.ndft_matrix(x, N)
    assert rel(oracle.ndft_trafo(x, fh), A @ fh.ravel()) < 1e-13
    y = rng.standard_normal(50) + 1j * rng.standard_normal(50)
    assert rel(oracle.ndft_adjoint(x, y, N).ravel(), A.conj().T @ y) < 1e-13


@pytest.mark.parametrize("N,m,alpha,tol", [((16, 16), 4, 2.0, 1e-6), ((32, 32), 4, 2.0, 1e-6),
                                           ((8, 8, 8), 3, 2.0, 1e-4), ((16, 16), 6, 2.0, 1e-9)])
def test_nfft_matches_ndft(oracle, N, m, alpha, tol):
    rng = np.random.default_rng(2)
    M = 300
    x = rng.uniform(-0.5, 0.5, (M, len(N)))
    P = oracle.NFFT(N, M, m=m, alpha=alpha)
    P.set_x(x)
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    assert rel(P.trafo(fh), oracle.ndft_trafo(x, fh)) < tol
    assert rel(P.adjoint(y), oracle.ndft_adjoint(x, y, N)) < tol


@pytest.mark.parametrize("m,alpha", [(1, 1.0), (4, 2.0), (2, 1.25)])
def test_nfft_is_exactly_adjoint(oracle, m, alpha):
    rng = np.random.default_rng(3)
    N, M = (16, 16), 200
    x = rng.uniform(-0.5, 0.5, (M, 2))
    P = oracle.NFFT(N, M, m=m, alpha=alpha)
    P.set_x(x)
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    lhs = np.vdot(y, P.trafo(fh))
    rhs = np.vdot(P.adjoint(y), fh)
    assert abs(lhs - rhs) < 1e-11 * abs(lhs)


def test_kb_transform_pair(oracle):
    """phihut(k) = n * integral phi(x) exp(2 pi i k x) dx over the window support
    (the deapodisation normalisation), checked by quadrature."""
    L = oracle.lib()
    n, m = 64, 4
    b = np.pi * (2.0 - 1.0 / 2.0)
    tau = np.linspace(-m, m, 200001)
    phi = np.array([L.orc_kb_phi(float(t), m, b) for t in tau[::50]])
    tt = tau[::50]
    for k in [0, 3, 10, 17]:
        # integral over tau = n x : phihut = integral phi(tau) exp(2 pi i k tau / n) dtau
        integ = np.trapezoid(phi * np.cos(2 * np.pi * k * tt / n), tt)
        assert abs(integ - L.orc_kb_phihut(k, n, m, b)) < 1e-6 * L.orc_kb_phihut(k, n, m, b)
    # continuity of the window at |tau| = m (sinh and sin branches meet at b/pi)
    for t in (m - 1e-7, m, m + 1e-7):
        assert abs(L.orc_kb_phi(t, m, b) - b / np.pi) < 1e-5


def test_damping_mask(oracle):
    what = oracle.damp_mask((16, 16))
    i = np.arange(16) - 8
    ref = (np.sqrt(i[:, None] ** 2 + i[None, :] ** 2) <= 8).astype(float)
    assert np.array_equal(what, ref)
    w3 = oracle.damp_mask((8, 8, 8))
    j = np.arange(8) - 4
    r3 = np.sqrt(j[:, None, None] ** 2 + j[None, :, None] ** 2 + j[None, None, :] ** 2)
    assert np.array_equal(w3, (r3 <= 4).astype(float))


def test_itrafo_semantics(oracle):
    """CGNR inverse NFFT: zero start, early exit on the absolute weighted residual."""
    from codeare_gb300 import synth
    k = synth.radial2d(12, 32, golden=True)
    w = synth.ramp_weights(k)
    P = oracle.NFFT((16, 16), k.shape[0], m=1, alpha=1.0)
    P.set_x(k)
    what = oracle.damp_mask((16, 16))
    rng = np.random.default_rng(4)
    y = rng.standard_normal(k.shape[0]) + 1j * rng.standard_normal(k.shape[0])
    f0, dr0, s0 = P.itrafo(y, w, what, maxit=0, eps=1e-3)
    assert s0 == 0 and np.all(f0 == 0)
    # tiny data: ||y||_W^2 < eps -> returns zeros without a step (data-scale dependence)
    f1, dr1, s1 = P.itrafo(1e-4 * y, w, what, maxit=3, eps=1e-3)
    assert s1 == 0 and np.all(f1 == 0)
    f3, dr3, s3 = P.itrafo(y, w, what, maxit=3, eps=1e-3)
    assert s3 == 3
    f10, dr10, _ = P.itrafo(y, w, what, maxit=10, eps=0.0)
    assert dr10 <= dr3
    # search directions live inside the damping mask
    assert np.all(f10[what == 0] == 0)


def test_cgls_codeare_semantics(oracle):
    from codeare_gb300 import synth
    cfg = synth.small_config(N=16, nc=3, nspokes=16, nsamp=32, alpha=2.0, m=4)
    s = oracle.Sense(cfg["sens"], cfg["k"], w=cfg["w"], m=4, alpha=2.0, threads=1)
    y = s.trafo(cfg["image"])
    x0, r0 = s.cgls_codeare(y, cgiter=0)
    assert rel(x0, s.adjoint_codeare(y)) < 1e-14 and len(r0) == 0
    x, res = s.cgls_codeare(y, cgiter=6, cgeps=0.0, lam=5e-2)
    assert res[0] == 1.0 and len(res) == 6
    assert res[-1] < res[0]
    # FP32 reference precision stays within 1e-4 of FP64 at equal iterations
    xr, _ = s.cgls_codeare(y, cgiter=6, cgeps=0.0, lam=5e-2, refprec=True)
    assert rel(xr, x) < 1e-4


def test_cg_standard_converges_to_ndft_solution(oracle):
    """At sigma=2, m=4 the standard CG-SENSE solution equals the dense NDFT normal
    equations' solution."""
    from codeare_gb300 import synth
    N, nc = 12, 3
    k = synth.radial2d(20, 24, golden=True)
    w = synth.ramp_weights(k) + 0.05
    S = synth.coils2d(N, nc)
    s = oracle.Sense(S, k, w=w, m=4, alpha=2.0, threads=1)
    x_true = synth.phantom(N)
    y = s.trafo(x_true)
    lam = 1e-3
    x, res = s.cg(y, maxit=300, tol=1e-12, lam=lam, weighted=True)
    A = oracle.ndft_matrix(k, (N, N))
    E = np.concatenate([A * S[c].reshape(1, -1) for c in range(nc)], axis=0)
    W = np.tile(w.astype(np.float64), nc)
    H = E.conj().T @ (W[:, None] * E) + lam * np.eye(N * N)
    xd = np.linalg.solve(H, E.conj().T @ (W * y.reshape(-1)))
    assert rel(x.ravel(), xd) < 1e-6


@pytest.mark.parametrize("name", ["small2d_s2m4", "small2d_s1m1"])
def test_golden_2d(oracle, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    m, alpha = int(g["m"]), float(g["alpha"])
    s = oracle.Sense(g["S"], g["k"], w=g["w"], m=m, alpha=alpha, threads=1)
    nc = int(g["nc"])
    assert rel(np.stack([s.nfft.trafo(g["fh"][c]) for c in range(nc)]), g["trafo"]) < 1e-12
    assert rel(np.stack([s.nfft.adjoint(g["ys"][c]) for c in range(nc)]), g["adjoint"]) < 1e-12
    assert rel(s.adjoint_codeare(g["y"]), g["eh_codeare"]) < 1e-10
    x, res = s.cgls_codeare(g["y"], cgiter=5, cgeps=1e-7, lam=5e-2)
    assert rel(x, g["x_cgls"]) < 1e-9
    assert np.array_equal(s.what, g["what"])


def test_golden_3d(oracle):
    g = np.load(os.path.join(GOLD, "small3d_s2m2.npz"))
    N = int(g["N"])
    P = oracle.NFFT((N, N, N), g["k"].shape[0], m=int(g["m"]), alpha=float(g["alpha"]))
    P.set_x(g["k"])
    assert rel(P.trafo(g["fh"][0]), g["trafo"][0]) < 1e-12
    assert rel(P.adjoint(g["ys"][1]), g["adjoint"][1]) < 1e-12


def test_cnn_oracle_gradients_match_finite_differences():
    from oracle import cnn
    rng = np.random.default_rng(0)
    w = rng.standard_normal(28800) * 0.1
    x = rng.standard_normal((1, 6, 7, 2))
    t = rng.standard_normal((1, 6, 7, 2))
    _, g = cnn.gradients(w, x, t)
    eps = 1e-6
    for i in [5, 700, 10000, 20000, 28500]:
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        fd = (cnn.gradients(wp, x, t)[0] - cnn.gradients(wm, x, t)[0]) / (2 * eps)
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(g[i])) + 1e-9


def test_wavelet_filters_and_transform():
    """The oracle's Daubechies filters are orthonormal with taps/2 vanishing
    moments, and its periodic transform is orthogonal (inverse = adjoint)."""
    from oracle import cs
    for taps in (2, 4, 8):
        h = cs.daubechies(taps)
        assert abs(h.sum() - np.sqrt(2.0)) < 1e-12
        for m in range(taps // 2):
            assert abs(np.dot(h[:taps - 2 * m], h[2 * m:]) - (m == 0)) < 1e-12
        g = h * (-1.0) ** np.arange(taps)
        for q in range(taps // 2):
            assert abs(np.dot(g, np.arange(taps, dtype=float) ** q)) < 1e-9
    assert h[0] > h[-1] > -0.02  # large coefficients first (Wavelet.hpp:142-153 ordering)
    lo, hi = cs.wavelet_filters(0, 8)
    rng = np.random.default_rng(0)
    c = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    d = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    assert np.abs(cs.dwt_inv(cs.dwt_fwd(c, lo, hi), lo, hi) - c).max() < 1e-12
    assert abs(np.vdot(d, cs.dwt_fwd(c, lo, hi)) - np.vdot(cs.dwt_inv(d, lo, hi), c)) < 1e-9


def test_tv_operators():
    """The third-axis TV adjoint is exact; the 2-D adjoint leaves the border
    rows of each component out (TVOP.hpp:52-63)."""
    from oracle import cs
    rng = np.random.default_rng(1)
    c = rng.standard_normal((6, 6, 5)) + 1j * rng.standard_normal((6, 6, 5))
    A = rng.standard_normal((6, 6, 5)) + 1j * rng.standard_normal((6, 6, 5))
    assert abs(np.vdot(A, cs.tv_fwd(c, "z")) - np.vdot(cs.tv_adj(A, "z"), c)) < 1e-10
    c2 = c[:, :, 0]
    A2 = np.zeros((6, 6, 2), complex)
    A2[2, 3, 0] = 1.0
    r = cs.tv_adj(A2, "2d")
    assert r[2, 3] == -1.0 and r[3, 3] == 1.0 and np.count_nonzero(r) == 2
    A2[:] = 0
    A2[0, 3, 0] = 1.0  # border row: the reference's adjoint drops the -1 at index 0
    assert np.count_nonzero(cs.tv_adj(A2, "2d")) == 1
    assert cs.tv_fwd(c2, "2d").shape == (6, 6, 2)
