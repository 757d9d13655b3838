"""The circulant preconditioner of the standard-mode normal equations
(cgs_precond_apply) against a numpy restatement built from the FP64 oracle's
point-spread function, and flexible CG with it (alone and as the base the
learned network corrects) against plain CG."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def small_problem(gpu, N=64, nc=8, spokes=24, lam_rel=1e-3):
    from codeare_gb300 import synth
    k = synth.radial2d(spokes, 2 * N, golden=True)
    w = (synth.ramp_weights(k) + 0.5 / (2 * N)).astype(np.float32)
    S = synth.coils2d(N, nc)
    p = gpu.Plan((N, N), k.shape[0], ncoils=nc, m=4, alpha=2.0)
    p.set_kspace(k)
    p.set_weights(w)
    p.set_sensitivities(S)
    lam = lam_rel * float(np.sum(w, dtype=np.float64)) * float(np.mean(np.sum(np.abs(S) ** 2, axis=0)))
    return p, k, w, S, lam


def circulant_reference(oracle, k, w, S, lam, r, floor=0.2):
    """z = Q F^-1 (F Q r / (c + lambda / mean D)) with c the floored T. Chan
    spectrum of the FP64 point-spread function, Q = D^-1/2, D = sum |S|^2."""
    N = S.shape[1]
    P2 = oracle.NFFT((2 * N, 2 * N), k.shape[0], m=4, alpha=2.0)
    P2.set_x(k.astype(np.float64))
    T = P2.adjoint(w.astype(np.complex128))      # T[d], index d + N
    T[0, :] = 0
    T[:, 0] = 0
    d = np.arange(2 * N) - N
    wgt = np.clip(1 - np.abs(d) / N, 0, None)
    cN = np.fft.ifftshift(T * wgt[:, None] * wgt[None, :]).reshape(2, N, 2, N).sum(axis=(0, 2))
    c = np.fft.fft2(cN).real
    c = np.maximum(c, floor * max(c.mean(), 0.0))
    D = np.sum(np.abs(S.astype(np.complex128)) ** 2, axis=0)
    q = 1.0 / np.sqrt(D)
    return q * np.fft.ifft2(np.fft.fft2(q * r) / (c + lam / D.mean()))


def test_circulant_matches_numpy_restatement(gpu, oracle):
    p, k, w, S, lam = small_problem(gpu)
    rng = np.random.default_rng(4)
    r = (rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))).astype(np.complex64)
    z = np.zeros_like(r)
    p.precond_apply(r, z, lam=lam, weighted=True)
    p.close()
    ref = circulant_reference(oracle, k, w, S, lam, r.astype(np.complex128))
    assert rel(z, ref) < 2e-4       # FP32 point-spread function and FFTs against FP64
    # symmetric positive definite: <r, C r> > 0 and <a, C b> = <C a, b>
    assert np.vdot(r, z).real > 0


def test_circulant_fcg_converges_to_plain_solution(gpu):
    import torch
    p, k, w, S, lam = small_problem(gpu)
    N, nc = 64, 8
    from codeare_gb300 import synth
    y = np.zeros((nc, k.shape[0]), np.complex64)
    p.sense_trafo(synth.phantom(N), y)
    y = synth.add_noise(y, 1e-3, seed=3)
    ref = np.zeros((N, N), np.complex64)
    rp = p.solve_fcg(ref, y=y, cgiter=2000, cgeps=1e-6, lam=lam)
    xc = np.zeros_like(ref)
    rc = p.solve_fcg(xc, y=y, cgiter=2000, cgeps=1e-6, lam=lam, circulant=True)
    assert rc["res_last"] <= 1e-6 and rp["res_last"] <= 1e-6
    # two solutions at ||r||/||r0|| = 1e-6 of a system with condition ~1e3
    assert rel(xc, ref) < 1e-3
    assert rc["iterations"] < rp["iterations"]
    # the network mode on the circulant base (freshly initialised weights):
    # the fallback keeps it convergent
    net = gpu.capi.Net(max_batch=1, max_h=N, max_w=N)
    xl = np.zeros_like(ref)
    rl = p.solve_fcg(xl, y=y, net=net, cgiter=2000, cgeps=1e-6, lam=lam, circulant=True)
    net.close()
    p.close()
    assert rl["res_last"] <= 1e-6
    assert rel(xl, ref) < 1e-3
