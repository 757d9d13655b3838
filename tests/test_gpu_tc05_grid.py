"""2-D spreading on the 5th-generation tensor cores (spread_block 64:
tcgen05.mma kind::tf32 over 8 x 16 grid patches, TF32-split operands, FP32
accumulation in tensor memory) against the CUDA-core kernel and the FP64
oracle.

The two kernels compute the same 100-tap sums (m = 4) in FP32 in different
orders, so they agree to FP32 rounding (3e-6 relative, as for the mma.sync
kernels).  Cases cover coil counts that leave partial 32-coil chunks and narrow tiles (1, 3, 5, 20, 33),
oversampled sides that are not multiples of the patch (90, 96, 80), a grid
smaller than the footprint (the wrapped window sum), cut-offs m = 1..4,
density weights, crowded patches split over many partial slots, and
bitwise repeatability.
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
