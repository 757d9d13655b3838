"""NCSENSE's dim4 batch on the GPU (a plan with frames > 1): F frames with
their own trajectories and shared sensitivities and weights
(src/matrix/ft/NCSENSE.hpp:141-166, 204-348), against the FP64 restatement
(oracle.FramesSense) and against single-frame plans."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_OP = 2e-5
TOL_IMG = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def frames_case(N=32, nc=4, F=4, spokes=12, nsamp=64, m=1, alpha=1.0):
    """golden-angle radial spokes dealt into F consecutive frames, as GRASP sorts them"""
    from codeare_gb300 import synth
    k = synth.radial2d(F * spokes, nsamp, golden=True).reshape(F, spokes * nsamp, 2)
    w = synth.ramp_weights(k[0])
    S = synth.coils2d(N, nc)
    x = np.stack([synth.phantom(N) * (1.0 + 0.1 * f) for f in range(F)])
    return dict(N=N, nc=nc, F=F, k=np.ascontiguousarray(k, np.float32), w=w, S=S, x=c64(x), m=m, alpha=alpha)


def make(cg, c):
    p = cg.Plan((c["N"], c["N"]), c["k"].shape[1], ncoils=c["nc"], m=c["m"], alpha=c["alpha"], frames=c["F"])
    p.set_kspace(c["k"])
    p.set_weights(np.ascontiguousarray(c["w"], np.float32))
    p.set_sensitivities(c64(c["S"]))
    return p


def oracle_of(c):
    from oracle import oracle as O
    return O.FramesSense(c["S"], list(c["k"]), w=c["w"], m=c["m"], alpha=c["alpha"])


@pytest.mark.parametrize("m,alpha", [(1, 1.0), (4, 2.0)])
def test_frame_operators_match_oracle(gpu, m, alpha):
    c = frames_case(m=m, alpha=alpha)
    p, o = make(gpu, c), oracle_of(c)
    y = np.zeros((c["F"], c["nc"], c["k"].shape[1]), np.complex64)
    p.sense_trafo(c["x"], y)
    yo = o.trafo(c["x"])
    assert rel(y, yo) < TOL_OP
    xh = np.zeros_like(c["x"])
    p.sense_adjoint_codeare(c64(yo), xh, ftiter=3, fteps=1e-3)
    assert rel(xh, o.adjoint_codeare(yo, 3, 1e-3)) < TOL_OP


def test_frames_equal_single_frame_plans(gpu):
    """Each frame of a framed plan computes what a single-frame plan with the
    same trajectory computes (the same kernels on the same data)."""
    c = frames_case(F=3)
    p = make(gpu, c)
    M, nc, N = c["k"].shape[1], c["nc"], c["N"]
    rng = np.random.default_rng(2)
    f = c64(rng.standard_normal((c["F"], nc, M)) + 1j * rng.standard_normal((c["F"], nc, M)))
    fh = np.zeros((c["F"], nc, N, N), np.complex64)
    p.nfft_itrafo(f, fh, maxit=3, eps=1e-3)
    yk = np.zeros_like(f)
    p.nfft_trafo(fh, yk)
    for i in range(c["F"]):
        q = gpu.Plan((N, N), M, ncoils=nc, m=c["m"], alpha=c["alpha"])
        q.set_kspace(c["k"][i].copy())
        q.set_weights(np.ascontiguousarray(c["w"], np.float32))
        one = np.zeros((nc, N, N), np.complex64)
        q.nfft_itrafo(f[i].copy(), one, maxit=3, eps=1e-3)
        assert np.array_equal(one, fh[i])
        y1 = np.zeros((nc, M), np.complex64)
        q.nfft_trafo(fh[i].copy(), y1)
        assert np.array_equal(y1, yk[i])


def test_frame_cgls_matches_oracle(gpu):
    """codeare CGLS over the stacked frames (one set of CG scalars for all)."""
    from codeare_gb300 import synth
    c = frames_case()
    p, o = make(gpu, c), oracle_of(c)
    y = synth.add_noise(o.trafo(c["x"]), 1e-3, seed=9)
    xo, reso = o.cgls_codeare(y, cgiter=8, cgeps=1e-9, lam=5e-2, ftiter=3, fteps=1e-3)
    x = np.zeros_like(c["x"])
    rep = p.solve(c64(y), x, cgiter=8, cgeps=1e-9, lam=5e-2, ftiter=3, fteps=1e-3)
    assert rep["iterations"] == 8
    assert rel(x, xo) < TOL_IMG
    assert np.allclose(rep["res_hist"][:len(reso)], reso, rtol=1e-3)


def test_frame_cs_temporal_tv_matches_oracle(gpu):
    """GRASP's objective: CS over the frames with TV along the frame axis
    (tv = 0 0 1, TVOP.hpp:134-166) and the parallel line search."""
    from codeare_gb300 import synth
    from oracle import cs
    c = frames_case()
    p, o = make(gpu, c), oracle_of(c)
    y = c64(synth.add_noise(o.trafo(c["x"]), 1e-3, seed=9))
    kw = dict(tvw=(0.02, 0.0), tvdims=([0, 0, 1], None), xfmw=0.0, l1=1e-6, pnorm=1.0, csiter=2, nliter=4,
              lsiter=6, lsa=0.01, lsb=0.6, cgconv=0.0, parallel_linesearch=True, cgiter=4, cgeps=1e-6,
              lam=1e-9, ftiter=1, fteps=7e-4)
    oc = cs.CSXSense(o, **kw)
    g = gpu.CS(p, **kw)
    x0 = np.zeros_like(c["x"])
    p.solve(y, x0, cgiter=4, cgeps=1e-6, lam=1e-9, ftiter=1, fteps=7e-4)
    rng = np.random.default_rng(4)
    dx = c64(0.1 * np.abs(x0).max() * (rng.standard_normal(x0.shape) + 1j * rng.standard_normal(x0.shape)))
    oc.set_data(y)
    go = oc.df(x0)
    gg = np.zeros_like(x0)
    g.df(y, x0, gg)
    assert rel(gg, go) < 2e-4
    oc.update(dx)
    fo, _ = oc.obj(x0, dx, 0.36)
    fg, _ = g.obj(y, x0, dx, 0.36)
    assert abs(fg - fo) <= 2e-5 * abs(fo)
    oc2 = cs.CSXSense(o, **kw)
    xo = oc2.adjoint(y)
    x = np.zeros_like(x0)
    rep = gpu.CS(p, **kw).adjoint(y, x)
    assert rep["ls_index"] == [li for li, _ in oc2.log]
    assert rel(x, xo) < 2e-3


def test_frames_reject_unbuilt_paths(gpu):
    c = frames_case(F=2)
    p = make(gpu, c)
    y = np.zeros((2, c["nc"], c["k"].shape[1]), np.complex64)
    x = np.zeros_like(c["x"])
    with pytest.raises(gpu.CgsError):
        p.solve(y, x, mode=gpu.MODE_STANDARD, toeplitz=True)
    with pytest.raises(gpu.CgsError):
        p.solve_fcg(x, y=y)
    with pytest.raises(gpu.CgsError):
        gpu.CS(p, wl_family=0, wl_member=4)
    t, _ = p.autotune()
    assert p.tuning() == t
