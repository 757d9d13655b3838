"""Parity with the FP64 oracle at the full sizes of the benchmark workloads.

Each case runs the CUDA path through the C ABI on the workload at its own size
and compares it with the FP64 restatement of the reference path
(oracle/cgs_oracle.c):

  * CG-SENSE 128^2, 8 coils, 96 x 256 uniform radial, sigma 2, m 4: codeare's
    CGLS over its CGNR-based E^H (CGLS.hpp:30-59, NCSENSE.hpp:251-348), 10
    iterations, lambda 5e-2 and 0, and standard CG with the Toeplitz-embedded
    E^H W E to ||r||/||r0|| = 1e-4;
  * the NuFFT operator 256^2, 32 coils, golden-angle 403 x 512: forward and
    adjoint of all 32 coils;
  * the batch of 64 uneven problems: 16 of them, one graph launch, chosen to
    cover every image size (96..320), every coil count (4, 8, 16, 32) and the
    variable-density spirals;
  * the 3-D kooshball on its 64^3 downsample (tests/golden/kooshball64.npz,
    made by tests/golden/make_kooshball64.py).

Tolerances: 2e-5 relative L2 per operator, 1e-4 for images (the bar the
parity target names), equal iteration counts throughout.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_OP = 2e-5
TOL_IMG = 1e-4

# 16 of the 64 uneven problems: N 96..320 each twice, coils 4/8/16/32, five spirals
BATCH_SUBSET = [2, 12, 19, 21, 22, 31, 38, 42, 43, 44, 46, 47, 50, 52, 59, 60]


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def cgsense_case(gpu):
    from codeare_gb300 import synth
    c = synth.radial2d_128_8coils()
    N, nc = c["shape"][0], c["sens"].shape[0]
    p = gpu.Plan((N, N), c["k"].shape[0], ncoils=nc, m=c["m"], alpha=c["alpha"])
    p.set_kspace(c["k"])
    p.set_weights(c["w"])
    p.set_sensitivities(c64(c["sens"]))
    y = np.zeros((nc, c["k"].shape[0]), np.complex64)
    p.sense_trafo(c64(c["image"]), y)
    y = synth.add_noise(y, c["noise"], seed=c["seed"])
    return c, p, y


@pytest.mark.parametrize("toeplitz", [False, True])
@pytest.mark.parametrize("lam", [5e-2, 0.0])
def test_cgsense_128_8coils_codeare_cgls_full_size(gpu, oracle, lam, toeplitz):
    """codeare CGLS: each CG step's E^H(E p) through the NFFT pair, or (toeplitz)
    with the inner CGNR run in image space on the Toeplitz kernel."""
    c, p, y = cgsense_case(gpu)
    N = c["shape"][0]
    x = np.zeros((N, N), np.complex64)
    rep = p.solve(y, x, mode=gpu.MODE_CODEARE, cgiter=10, cgeps=1e-7, lam=lam, ftiter=3, fteps=1e-3,
                  toeplitz=toeplitz)
    p.close()
    s = oracle.Sense(c["sens"], c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
    xo, res = s.cgls_codeare(y, cgiter=10, cgeps=1e-7, lam=lam, ftiter=3, fteps=1e-3)
    # res holds every check of the loop, including the one that ends it early
    updates = len(res) - (1 if res[-1] <= 1e-7 else 0)
    assert rep["iterations"] == updates
    np.testing.assert_allclose(rep["res_hist"][:len(res)], res, rtol=1e-3)
    assert rel(x, xo) < TOL_IMG


@pytest.mark.parametrize("toeplitz", [True, False])
def test_cgsense_128_8coils_standard_cg_full_size(gpu, oracle, toeplitz):
    """Standard CG (true adjoint, E^H W E by Toeplitz embedding or by the NFFT
    pair, lambda 0) against the oracle's FP64 NFFT-pair CG at 10 and 20
    iterations.  The unregularised problem is ill-conditioned (the ramp weight
    is zero at the k-space centre): FP32 and FP64 CG drift apart by ~1e-3 after
    40 iterations and reach ||r||/||r0|| = 1e-4 (about 250 iterations) along
    different paths, so beyond 20 iterations the test compares residual
    histories and the two FP32 operators with each other."""
    c, p, y = cgsense_case(gpu)
    N = c["shape"][0]
    s = oracle.Sense(c["sens"], c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
    x = np.zeros((N, N), np.complex64)
    for it in (10, 20):
        rep = p.solve(y, x, mode=gpu.MODE_STANDARD, cgiter=it, cgeps=0.0, lam=0.0, weighted=True, toeplitz=toeplitz)
        assert rep["iterations"] == it
        xo, res = s.cg(y, maxit=it, tol=0.0, lam=0.0, weighted=True)
        assert rel(x, xo) < TOL_IMG, it
        np.testing.assert_allclose(rep["res_hist"][:it + 1], res, rtol=1e-3)
    rep = p.solve(y, x, mode=gpu.MODE_STANDARD, cgiter=1000, cgeps=1e-4, lam=0.0, weighted=True, toeplitz=toeplitz)
    it = rep["iterations"]
    assert rep["res_last"] <= 1e-4 and it < 1000
    _, res = s.cg(y, maxit=it, tol=0.0, lam=0.0, weighted=True)
    assert res[-1] < 1.5e-4
    np.testing.assert_allclose(rep["res_hist"][:26], res[:26], rtol=1e-2)   # drift starts near 30 iterations
    x2 = np.zeros_like(x)
    p.solve(y, x2, mode=gpu.MODE_STANDARD, cgiter=it, cgeps=0.0, lam=0.0, weighted=True, toeplitz=not toeplitz)
    p.close()
    assert rel(x, x2) < 5e-2


def test_nufft_256_32coils_all_coils_full_size(gpu, oracle):
    from codeare_gb300 import synth
    cfg = synth.radial2d_256_32coils()
    k = cfg["k"]
    M, nc, N = k.shape[0], 32, 256
    rng = np.random.default_rng(20261204)
    fh = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    ys = c64(rng.standard_normal((nc, M)) + 1j * rng.standard_normal((nc, M)))
    p = gpu.Plan((N, N), M, ncoils=nc, m=4, alpha=2.0)
    p.set_kspace(k)
    p.autotune()
    f = np.zeros((nc, M), np.complex64)
    img = np.zeros((nc, N, N), np.complex64)
    p.nfft_trafo(fh, f)
    p.nfft_adjoint(ys, img)
    p.close()
    P = oracle.NFFT((N, N), M, m=4, alpha=2.0)
    P.set_x(k)
    assert rel(f, P.trafo_batch(fh)) < TOL_OP
    assert rel(img, P.adjoint_batch(ys)) < TOL_OP


def test_codeare_toeplitz_needs_an_accurate_nfft(gpu):
    from codeare_gb300 import capi, synth
    k = synth.radial2d(16, 64, golden=True)
    p = gpu.Plan((32, 32), k.shape[0], ncoils=2, m=1, alpha=1.0)
    p.set_kspace(k)
    p.set_weights(synth.ramp_weights(k))
    p.set_sensitivities(synth.coils2d(32, 2))
    y = np.ones((2, k.shape[0]), np.complex64)
    x = np.zeros((32, 32), np.complex64)
    with pytest.raises(capi.CgsError):
        p.solve(y, x, mode=gpu.MODE_CODEARE, cgiter=2, toeplitz=True)
    p.close()


def test_batch_16_of_64_uneven_problems_full_size(gpu, oracle):
    """One graph launch over 16 of the 64 uneven problems at their own sizes,
    codeare CGLS 15 iterations each, against the oracle problem by problem;
    the same batch again with the CG steps on the Toeplitz kernels."""
    from codeare_gb300 import capi, synth
    probs = synth.uneven_batch()
    sel = [probs[i] for i in BATCH_SUBSET]
    assert {c["N"] for c in sel} == set(range(96, 321, 32))
    assert {c["nc"] for c in sel} == {4, 8, 16, 32}
    assert sum(c["kind"].startswith("spiral") for c in sel) >= 4
    plans, ys, sens = [], [], []
    for c in sel:
        N, nc, k = c["N"], c["nc"], c["k"]
        p = capi.Plan((N, N), k.shape[0], ncoils=nc, m=c["m"], alpha=c["alpha"])
        p.set_kspace(k)
        p.set_weights(c["w"])
        S = synth.coils2d(N, nc)
        p.set_sensitivities(S)
        y = np.zeros((nc, k.shape[0]), np.complex64)
        p.sense_trafo(c64(synth.phantom(N)), y)
        plans.append(p)
        sens.append(S)
        ys.append(synth.add_noise(y, c["noise"], seed=c["seed"]))
    runs = []
    for toeplitz in (False, True):
        b = capi.Batch(plans, capi.solve_opts(mode=gpu.MODE_CODEARE, cgiter=15, cgeps=0.0, lam=5e-2,
                                              toeplitz=toeplitz))
        xs = [np.zeros((c["N"], c["N"]), np.complex64) for c in sel]
        reps, _ = b.solve(ys, xs)
        b.close()
        runs.append((toeplitz, xs, reps))
    for p in plans:
        p.close()
    errs = []
    for i, (c, S, y) in enumerate(zip(sel, sens, ys)):
        s = oracle.Sense(S, c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
        xo, _ = s.cgls_codeare(y, cgiter=15, cgeps=0.0, lam=5e-2)
        for toeplitz, xs, reps in runs:
            assert reps[i]["iterations"] == 15, c["name"]
            errs.append((c["name"], toeplitz, rel(xs[i], xo)))
    bad = [e for e in errs if not e[2] < TOL_IMG]
    assert not bad, bad


def test_kooshball_64cubed_downsample_matches_oracle(gpu, oracle):
    """The 64^3 downsample of the 128^3 kooshball (16 coils, 5000 x 128 spokes):
    standard CG with the Toeplitz-embedded E^H W E (128^3 FFTs) for the oracle's
    iteration count, against the oracle's FP64 NFFT-pair CG solution."""
    import sys
    sys.path.insert(0, GOLD)
    import make_kooshball64 as mk
    g = np.load(os.path.join(GOLD, "kooshball64.npz"))
    c = mk.case()
    it = int(g["iterations"])
    s = oracle.Sense(c["sens"], c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
    y = c64(s.trafo(c["image"]))
    p = gpu.Plan(c["shape"], c["k"].shape[0], ncoils=c["sens"].shape[0], m=c["m"], alpha=c["alpha"])
    p.set_kspace(c["k"])
    p.set_weights(c["w"])
    p.set_sensitivities(c64(c["sens"]))
    x = np.zeros(c["shape"], np.complex64)
    rep = p.solve(y, x, mode=gpu.MODE_STANDARD, cgiter=it, cgeps=0.0, lam=0.0, weighted=True, toeplitz=True)
    p.close()
    assert rep["iterations"] == it
    np.testing.assert_allclose(rep["res_hist"][:it + 1], g["res"][:it + 1], rtol=2e-2)
    assert rel(x, g["x"]) < TOL_IMG
