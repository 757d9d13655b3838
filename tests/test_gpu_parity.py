"""Parity of the sm_103a CUDA path (through the C ABI) with the FP64 oracle.

Tolerances: the NFFT operators run in FP32 with FP64-accumulated CG scalars,
so per-operator relative L2 errors against the FP64 oracle are held to 2e-5,
and CG-SENSE images to the 1e-4 relative L2 the parity target names.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_OP = 2e-5
TOL_IMG = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def make_plan(cg, shape, k, nc, m, alpha, w=None, S=None):
    p = cg.Plan(shape, k.shape[0], ncoils=nc, m=m, alpha=alpha)
    p.set_kspace(np.ascontiguousarray(k, dtype=np.float32))
    if w is not None:
        p.set_weights(np.ascontiguousarray(w, dtype=np.float32))
    if S is not None:
        p.set_sensitivities(c64(S))
    return p


@pytest.mark.parametrize("name", ["small2d_s2m4", "small2d_s1m1"])
def test_golden_2d_operators(gpu, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    N, nc, m, alpha = int(g["N"]), int(g["nc"]), int(g["m"]), float(g["alpha"])
    k = g["k"]
    M = k.shape[0]
    p = make_plan(gpu, (N, N), k, nc, m, alpha, w=g["w"], S=g["S"])
    out = np.zeros((nc, M), np.complex64)
    p.nfft_trafo(c64(g["fh"]), out)
    assert rel(out, g["trafo"]) < TOL_OP
    img = np.zeros((nc, N, N), np.complex64)
    p.nfft_adjoint(c64(g["ys"]), img)
    assert rel(img, g["adjoint"]) < TOL_OP
    p.nfft_itrafo(c64(g["ys"]), img, maxit=3, eps=1e-3)
    assert rel(img, g["itrafo"]) < TOL_OP
    y = np.zeros((nc, M), np.complex64)
    p.sense_trafo(c64(g["x"]), y)
    assert rel(y, g["y"]) < TOL_OP
    x = np.zeros((N, N), np.complex64)
    p.sense_adjoint_codeare(c64(g["y"]), x, ftiter=3, fteps=1e-3)
    assert rel(x, g["eh_codeare"]) < TOL_OP
    p.sense_adjoint(c64(g["y"]), x, weighted=True)
    assert rel(x, g["eh_true"]) < TOL_OP
    rep = p.solve(c64(g["y"]), x, mode=gpu.MODE_CODEARE, cgiter=5, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
    assert rel(x, g["x_cgls"]) < TOL_IMG
    assert rep["iterations"] == 5
    np.testing.assert_allclose(rep["res_hist"][:5], g["res_cgls"][:5], rtol=1e-3)
    rep = p.solve(c64(g["y"]), x, mode=gpu.MODE_STANDARD, cgiter=8, cgeps=1e-10, lam=0.0, weighted=True)
    assert rel(x, g["x_cg"]) < TOL_IMG


def test_golden_3d_operators(gpu):
    g = np.load(os.path.join(GOLD, "small3d_s2m2.npz"))
    N, nc = int(g["N"]), int(g["nc"])
    k = g["k"]
    p = make_plan(gpu, (N, N, N), k, nc, int(g["m"]), float(g["alpha"]))
    out = np.zeros((nc, k.shape[0]), np.complex64)
    p.nfft_trafo(c64(g["fh"]), out)
    assert rel(out, g["trafo"]) < TOL_OP
    img = np.zeros((nc, N, N, N), np.complex64)
    p.nfft_adjoint(c64(g["ys"]), img)
    assert rel(img, g["adjoint"]) < TOL_OP


@pytest.mark.parametrize("N,nc,alpha,m", [(32, 4, 2.0, 4), (48, 3, 2.0, 4), (40, 2, 1.0, 1), (32, 5, 1.5, 2),
                                         (96, 2, 2.0, 4), (160, 2, 2.0, 4), (224, 1, 2.0, 4), (288, 1, 2.0, 4)])
def test_nfft_vs_oracle(gpu, oracle, N, nc, alpha, m):
    """Non-power-of-two grids exercise the odd radices: 40 and 48 (alpha 1.5 on 32) the runtime-radix
    passes, 96, 192, 320, 448 and 576 (2^k times 3, 5, 7, 9) the compile-time passes."""
    from codeare_gb300 import synth
    k = synth.radial2d(30, 2 * N, golden=True)
    M = k.shape[0]
    rng = np.random.default_rng(N + nc)
    fh = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    ys = c64(rng.standard_normal((nc, M)) + 1j * rng.standard_normal((nc, M)))
    P = oracle.NFFT((N, N), M, m=m, alpha=alpha)
    P.set_x(k)
    p = make_plan(gpu, (N, N), k, nc, m, alpha)
    out = np.zeros((nc, M), np.complex64)
    p.nfft_trafo(fh, out)
    ref = np.stack([P.trafo(fh[c]) for c in range(nc)])
    assert rel(out, ref) < TOL_OP
    img = np.zeros((nc, N, N), np.complex64)
    p.nfft_adjoint(ys, img)
    ref = np.stack([P.adjoint(ys[c]) for c in range(nc)])
    assert rel(img, ref) < TOL_OP


def test_ndft_4096_points_256_32coils_size(gpu, oracle):
    """256^2 image, sigma=2, m=4: FP32 NFFT vs FP64 direct NDFT on 4096 seeded random nodes."""
    rng = np.random.default_rng(20261204)
    N = 256
    k = rng.uniform(-0.5, 0.5, (4096, 2)).astype(np.float32)
    fh = c64(rng.standard_normal((1, N, N)) + 1j * rng.standard_normal((1, N, N)))
    p = make_plan(gpu, (N, N), k, 1, 4, 2.0)
    out = np.zeros((1, 4096), np.complex64)
    p.nfft_trafo(fh, out)
    ref = oracle.ndft_trafo(k.astype(np.float64), fh[0].astype(np.complex128))
    assert rel(out[0], ref) < 1e-5
    y = c64(rng.standard_normal((1, 4096)) + 1j * rng.standard_normal((1, 4096)))
    img = np.zeros((1, N, N), np.complex64)
    p.nfft_adjoint(y, img)
    refa = oracle.ndft_adjoint(k.astype(np.float64), y[0].astype(np.complex128), (N, N))
    assert rel(img[0], refa) < 1e-5


def test_nufft_256_32coils_properties_full_size(gpu):
    """Full size (256^2, 32 coils, 403x512 golden-angle): adjointness and
    linearity, which hold at any size."""
    from codeare_gb300 import synth
    cfg = synth.radial2d_256_32coils()
    k = cfg["k"]
    M, nc, N = k.shape[0], 32, 256
    rng = np.random.default_rng(5)
    p = make_plan(gpu, (N, N), k, nc, 4, 2.0)
    a = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    b = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    y = c64(rng.standard_normal((nc, M)) + 1j * rng.standard_normal((nc, M)))
    Aa = np.zeros((nc, M), np.complex64); Ab = np.zeros_like(Aa); Aab = np.zeros_like(Aa)
    p.nfft_trafo(a, Aa); p.nfft_trafo(b, Ab); p.nfft_trafo(c64(a + 2 * b), Aab)
    assert rel(Aab, Aa + 2 * Ab) < 1e-5
    AHy = np.zeros((nc, N, N), np.complex64)
    p.nfft_adjoint(y, AHy)
    for c in (0, 17, 31):
        lhs = np.vdot(y[c].astype(np.complex128), Aa[c].astype(np.complex128))
        rhs = np.vdot(AHy[c].astype(np.complex128), a[c].astype(np.complex128))
        assert abs(lhs - rhs) < 1e-4 * abs(lhs)


def test_cgls_codeare_vs_oracle(gpu, oracle):
    """Full codeare semantics (CGLS over the CGNR-based E^H) at equal iteration count."""
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=24, nsamp=64, alpha=2.0, m=4)
    s = oracle.Sense(cfg["sens"], cfg["k"], w=cfg["w"], m=4, alpha=2.0)
    y = synth.add_noise(s.trafo(cfg["image"]), 1e-3, seed=3)
    xo, reso = s.cgls_codeare(y, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3)
    p = make_plan(gpu, (32, 32), cfg["k"], 4, 4, 2.0, w=cfg["w"], S=cfg["sens"])
    x = np.zeros((32, 32), np.complex64)
    rep = p.solve(c64(y), x, mode=gpu.MODE_CODEARE, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3)
    assert rep["iterations"] == len(reso) or rep["iterations"] == len(reso) - 1
    assert rel(x, xo) < TOL_IMG


def test_codeare_defaults_sigma1_m1(gpu, oracle):
    """The reference plugin's defaults (alpha=1, m=1, ftiter=3, fteps=1e-3): the NFFT is
    far from the NDFT here, so parity needs the exact window and CGNR semantics."""
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=1.0, m=1)
    s = oracle.Sense(cfg["sens"], cfg["k"], w=cfg["w"], m=1, alpha=1.0)
    y = s.trafo(cfg["image"])
    xo, _ = s.cgls_codeare(y, cgiter=10, cgeps=1e-7, lam=5e-2)
    p = make_plan(gpu, (32, 32), cfg["k"], 4, 1, 1.0, w=cfg["w"], S=cfg["sens"])
    x = np.zeros((32, 32), np.complex64)
    p.solve(c64(y), x, mode=gpu.MODE_CODEARE, cgiter=10, cgeps=1e-7, lam=5e-2)
    assert rel(x, xo) < TOL_IMG


def test_device_pointers_match_host(gpu):
    import torch
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4)
    k = cfg["k"]
    p = make_plan(gpu, (32, 32), k, 4, 4, 2.0, w=cfg["w"], S=cfg["sens"])
    x = c64(cfg["image"])
    yh = np.zeros((4, k.shape[0]), np.complex64)
    p.sense_trafo(x, yh)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros((4, k.shape[0]), dtype=torch.complex64, device="cuda")
    p.sense_trafo(xd, yd)
    p.sync()
    assert rel(yd.cpu().numpy(), yh) < 1e-6


def test_pinned_host_buffers_match_pageable(gpu):
    """Pinned host buffers (asynchronous copies) must give the results of
    pageable buffers, and the host output must be complete on return."""
    import torch
    from codeare_gb300 import synth
    import codeare_gb300 as cg
    cfg = synth.small_config(N=32, nc=4)
    k, M = cfg["k"], cfg["k"].shape[0]
    p = make_plan(gpu, (32, 32), k, 4, 4, 2.0, w=cfg["w"], S=cfg["sens"])

    def pinned(shape):
        return torch.zeros(shape, dtype=torch.complex64).pin_memory().numpy()

    rng = np.random.default_rng(5)
    fh = c64(rng.standard_normal((4, 32, 32)) + 1j * rng.standard_normal((4, 32, 32)))
    f_pg, f_pn = np.zeros((4, M), np.complex64), pinned((4, M))
    fh_pn = pinned((4, 32, 32))
    fh_pn[...] = fh
    p.nfft_trafo(fh, f_pg)
    p.nfft_trafo(fh_pn, f_pn)
    assert np.array_equal(f_pg, f_pn)
    a_pg, a_pn = np.zeros((4, 32, 32), np.complex64), pinned((4, 32, 32))
    p.nfft_adjoint(f_pg, a_pg)
    p.nfft_adjoint(f_pn, a_pn)
    assert np.array_equal(a_pg, a_pn)
    x = c64(cfg["image"])
    y_pg, y_pn = np.zeros((4, M), np.complex64), pinned((4, M))
    p.sense_trafo(x, y_pg)
    x_pn = pinned((32, 32))
    x_pn[...] = x
    p.sense_trafo(x_pn, y_pn)
    assert np.array_equal(y_pg, y_pn)
    s_pg, s_pn = np.zeros((32, 32), np.complex64), pinned((32, 32))
    p.solve(y_pg, s_pg, mode=cg.MODE_STANDARD, cgiter=5, cgeps=0.0, lam=0.0)
    p.solve(y_pn, s_pn, mode=cg.MODE_STANDARD, cgiter=5, cgeps=0.0, lam=0.0)
    assert np.array_equal(s_pg, s_pn)


def test_bad_arguments_return_errors(gpu):
    from codeare_gb300 import capi
    with pytest.raises(capi.CgsError) as e:
        gpu.Plan((31, 32), 100, ncoils=1)
    assert e.value.status == capi.CGS_ERR_BAD_ARG
    with pytest.raises(capi.CgsError) as e:
        gpu.Plan((22, 22), 100, ncoils=1, alpha=2.0)  # 44 = 4*11: unsupported radix
    assert e.value.status == capi.CGS_ERR_BAD_ARG
    p = gpu.Plan((16, 16), 10, ncoils=1, m=2, alpha=2.0)
    with pytest.raises(capi.CgsError) as e:
        p.set_weights(np.ones(10, np.float32))
    assert e.value.status == capi.CGS_ERR_STATE
    bad = np.full((10, 2), 0.7, np.float32)
    with pytest.raises(capi.CgsError) as e:
        p.set_kspace(bad)
    assert e.value.status == capi.CGS_ERR_BAD_ARG


def test_edge_nodes_in_one_tile_and_boundary(gpu, oracle):
    """All nodes crowded in one tile (one bin split into many work items) plus nodes at -0.5."""
    rng = np.random.default_rng(9)
    N, M = 32, 5000
    k = (rng.uniform(-0.01, 0.01, (M, 2))).astype(np.float32)
    k[:8] = -0.5
    fh = c64(rng.standard_normal((2, N, N)) + 1j * rng.standard_normal((2, N, N)))
    P = oracle.NFFT((N, N), M, m=4, alpha=2.0)
    P.set_x(k)
    p = make_plan(gpu, (N, N), k, 2, 4, 2.0)
    out = np.zeros((2, M), np.complex64)
    p.nfft_trafo(fh, out)
    assert rel(out, np.stack([P.trafo(fh[c]) for c in range(2)])) < TOL_OP
    ys = c64(rng.standard_normal((2, M)) + 1j * rng.standard_normal((2, M)))
    img = np.zeros((2, N, N), np.complex64)
    p.nfft_adjoint(ys, img)
    assert rel(img, np.stack([P.adjoint(ys[c]) for c in range(2)])) < TOL_OP


@pytest.mark.parametrize("weighted", [True, False])
def test_standard_cg_toeplitz_2d(gpu, oracle, weighted):
    """Standard-mode CG with E^H W E applied by Toeplitz embedding (2N-grid FFT
    convolution) against the oracle's NFFT-based CG at the same iteration count."""
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=40, nsamp=64, alpha=2.0, m=4)
    s = oracle.Sense(cfg["sens"], cfg["k"], w=cfg["w"], m=4, alpha=2.0)
    y = s.trafo(cfg["image"])
    xo, reso = s.cg(y, maxit=8, tol=1e-12, lam=1e-3, weighted=weighted)
    p = make_plan(gpu, (32, 32), cfg["k"], 4, 4, 2.0, w=cfg["w"], S=cfg["sens"])
    x = np.zeros((32, 32), np.complex64)
    rep = p.solve(c64(y), x, mode=gpu.MODE_STANDARD, cgiter=8, cgeps=1e-12, lam=1e-3, weighted=weighted,
                  toeplitz=True)
    assert rep["iterations"] == 8
    assert rel(x, xo) < TOL_IMG
    np.testing.assert_allclose(rep["res_hist"][:9], reso[:9], rtol=2e-3)


def test_standard_cg_toeplitz_3d(gpu, oracle):
    from codeare_gb300 import synth
    N, nc = 16, 2
    k = synth.kooshball3d(300, 32)
    w = synth.ramp_weights(k) ** 2 + 1e-3
    S = synth.coils3d(N, nc)
    s = oracle.Sense(S, k, w=w, m=3, alpha=2.0)
    xt = synth.phantom3d(N)
    y = s.trafo(xt)
    xo, _ = s.cg(y, maxit=6, tol=1e-12, lam=1e-3, weighted=True)
    p = make_plan(gpu, (N, N, N), k, nc, 3, 2.0, w=w, S=S)
    x = np.zeros((N, N, N), np.complex64)
    p.solve(c64(y), x, mode=gpu.MODE_STANDARD, cgiter=6, cgeps=1e-12, lam=1e-3, weighted=True, toeplitz=True)
    assert rel(x, xo) < TOL_IMG
    x2 = np.zeros_like(x)
    p.solve(c64(y), x2, mode=gpu.MODE_STANDARD, cgiter=6, cgeps=1e-12, lam=1e-3, weighted=True, toeplitz=False)
    assert rel(x2, xo) < TOL_IMG


def test_kooshball_reduced_toeplitz_cg_matches_oracle(gpu, oracle):
    """The 3-D kooshball case at a size the FP64 oracle finishes: |k|^2
    weights, standard CG with the Toeplitz-embedded E^H W E on the GPU against
    the oracle's CG on the NFFT pair, same iteration count (8)."""
    from codeare_gb300 import capi, synth
    import codeare_gb300 as cg
    c = synth.kooshball3d_128_16coils(N=24, nc=4, nspokes=600, nsamp=48)
    N, nc = c["shape"][0], c["sens"].shape[0]
    k, w, S = c["k"], c["w"], c["sens"]
    s = oracle.Sense(S, k, w=w, m=c["m"], alpha=c["alpha"])
    y = synth.add_noise(s.trafo(c["image"]), c["noise"], seed=c["seed"])
    xo, _ = s.cg(y, maxit=8, tol=0.0, lam=0.0, weighted=True)
    p = capi.Plan((N, N, N), k.shape[0], ncoils=nc, m=c["m"], alpha=c["alpha"])
    p.set_kspace(k)
    p.set_weights(w)
    p.set_sensitivities(np.ascontiguousarray(S))
    x = np.zeros((N, N, N), np.complex64)
    r = p.solve(y.astype(np.complex64), x, mode=cg.MODE_STANDARD, cgiter=8, cgeps=0.0, lam=0.0, weighted=True,
                toeplitz=True)
    assert r["iterations"] == 8
    assert rel(x, xo) < 1e-4
    p.close()
