"""2-D gridding on the 5th-generation tensor cores against the CUDA-core
kernels and the FP64 oracle: spreading (spread_block 64: tcgen05.mma
kind::tf32 over 8 x 16 grid patches) and interpolation (interp_block 64: up
to 128 nodes of an 8 x 16 footprint-start bin per CTA, one MMA per region
row with the nodes' x windows as A, the y window applied to the row results),
both with TF32-split operands, the A matrix in tensor memory and FP32
accumulation.

The two kernels compute the same 100-tap sums (m = 4) in FP32 in different
orders, so they agree to FP32 rounding (3e-6 relative, as for the mma.sync
kernels).  Cases cover coil counts that leave partial 32-coil chunks and narrow tiles (1, 3, 5, 20, 33),
oversampled sides that are not multiples of the patch (90, 96, 80), a grid
smaller than the footprint (the wrapped window sum for spreading; the
interpolation falls back to the CUDA-core kernel there), cut-offs m = 1..4,
density weights, crowded patches split over many partial slots, both output
layouts of the interpolation (the caller's coil-major one and the bin-ordered
one a solve uses), and bitwise repeatability.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def adjoint(p, ys, N):
    nc = ys.shape[0]
    img = np.zeros((nc, N, N), np.complex64)
    p.nfft_adjoint(ys, img)
    return img


def case(N, alpha, m, nc, spokes, seed, golden=True):
    from codeare_gb300 import capi, synth
    k = synth.radial2d(spokes, 2 * N, golden=golden)
    M = k.shape[0]
    p = capi.Plan((N, N), M, ncoils=nc, m=m, alpha=alpha)
    p.set_kspace(k)
    rng = np.random.default_rng(seed)
    ys = c64(rng.standard_normal((nc, M)) + 1j * rng.standard_normal((nc, M)))
    return p, k, ys


@pytest.mark.parametrize("N,alpha,m,nc", [(64, 2.0, 4, 32), (64, 2.0, 4, 3), (60, 1.5, 4, 5), (48, 2.0, 2, 20),
                                          (40, 2.0, 1, 1), (64, 2.0, 4, 33), (48, 2.0, 3, 8), (4, 2.0, 4, 3)])
def test_tcgen05_spreading_matches_cuda_cores(gpu, N, alpha, m, nc):
    p, k, ys = case(N, alpha, m, nc, spokes=max(8, N), seed=N + nc + m)
    p.set_tuning(spread_block=64)
    img_tc = adjoint(p, ys, N)
    p.set_tuning(spread_block=1)
    img_cc = adjoint(p, ys, N)
    p.close()
    assert np.all(np.isfinite(img_tc))
    assert rel(img_tc, img_cc) < 3e-6


def test_tcgen05_spreading_split_patches_weights_and_repeat(gpu):
    """Short chunks split every crowded patch over many partial slots (summed
    in slot order): the result may change only by rounding; density-weighted
    E^H matches the CUDA-core kernel; a repeat is bit-identical."""
    from codeare_gb300 import synth
    N, nc = 64, 16
    p, k, ys = case(N, 2.0, 4, nc, spokes=160, seed=7)
    p.set_weights(synth.ramp_weights(k))
    p.set_sensitivities(c64(synth.coils2d(N, nc)))
    p.set_tuning(spread_block=64)
    a0 = adjoint(p, ys, N)
    x0 = np.zeros((N, N), np.complex64)
    p.sense_adjoint(ys, x0, weighted=True)
    assert np.array_equal(adjoint(p, ys, N), a0)
    p.set_tuning(spread_block=64, spread_chunk=32)
    a1 = adjoint(p, ys, N)
    x1 = np.zeros_like(x0)
    p.sense_adjoint(ys, x1, weighted=True)
    assert rel(a1, a0) < 3e-6 and rel(x1, x0) < 3e-6
    p.set_tuning(spread_block=1, spread_chunk=0)
    x2 = np.zeros_like(x0)
    p.sense_adjoint(ys, x2, weighted=True)
    p.close()
    assert rel(x0, x2) < 3e-6


def test_tcgen05_spreading_matches_oracle(gpu, oracle):
    N, nc, m, alpha = 96, 8, 4, 2.0
    p, k, ys = case(N, alpha, m, nc, spokes=120, seed=11)
    p.set_tuning(spread_block=64)
    img = adjoint(p, ys, N)
    p.close()
    P = oracle.NFFT((N, N), k.shape[0], m=m, alpha=alpha)
    P.set_x(k)
    assert rel(img, P.adjoint_batch(ys)) < 2e-5


def forward(p, fh, M):
    nc = fh.shape[0]
    f = np.zeros((nc, M), np.complex64)
    p.nfft_trafo(fh, f)
    return f


@pytest.mark.parametrize("N,alpha,m,nc", [(64, 2.0, 4, 32), (64, 2.0, 4, 3), (60, 1.5, 4, 5), (48, 2.0, 2, 20),
                                          (40, 2.0, 1, 1), (64, 2.0, 4, 33), (48, 2.0, 3, 8), (4, 2.0, 4, 3)])
def test_tcgen05_interpolation_matches_cuda_cores(gpu, N, alpha, m, nc):
    p, k, _ = case(N, alpha, m, nc, spokes=max(8, N), seed=N + nc)
    rng = np.random.default_rng(N * nc + m)
    fh = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    p.set_tuning(interp_block=64)
    f_tc = forward(p, fh, k.shape[0])
    assert np.array_equal(forward(p, fh, k.shape[0]), f_tc)
    p.set_tuning(interp_block=1)
    f_cc = forward(p, fh, k.shape[0])
    p.close()
    assert np.all(np.isfinite(f_tc))
    assert rel(f_tc, f_cc) < 3e-6


def test_tcgen05_interpolation_in_a_solve_and_against_oracle(gpu, oracle):
    """The bin-ordered output (the CG-SENSE step's E p) through a standard CG
    solve, against the same solve on the CUDA-core kernel, and the caller-
    layout output against the FP64 oracle."""
    from codeare_gb300 import synth
    import codeare_gb300 as cg
    N, nc = 96, 8
    p, k, ys = case(N, 2.0, 4, nc, spokes=120, seed=13)
    p.set_weights(synth.ramp_weights(k))
    p.set_sensitivities(c64(synth.coils2d(N, nc)))
    xs = []
    for ib in (64, 1):
        p.set_tuning(interp_block=ib, spread_block=64 if ib == 64 else 1)
        x = np.zeros((N, N), np.complex64)
        rep = p.solve(ys, x, mode=cg.MODE_STANDARD, cgiter=8, cgeps=0.0, lam=1e-3, weighted=True, toeplitz=False)
        assert rep["iterations"] == 8
        xs.append(x)
    assert rel(xs[0], xs[1]) < 1e-5
    rng = np.random.default_rng(5)
    fh = c64(rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N)))
    p.set_tuning(interp_block=64)
    f = forward(p, fh, k.shape[0])
    p.close()
    P = oracle.NFFT((N, N), k.shape[0], m=4, alpha=2.0)
    P.set_x(k)
    assert rel(f, P.trafo_batch(fh)) < 2e-5
