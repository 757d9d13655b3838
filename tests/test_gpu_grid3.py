"""3-D gridding on the tensor cores against the CUDA-core kernels and the
FP64 oracle.

The default 3-D path interpolates with up to 16 nodes of one 4 x 4 x 4
footprint-start bin per warp and spreads output-stationary over 4 x 4 x 4
patches (mma.m16n8k8 with TF32-split operands, FP32 accumulation).
interp_block 1 / spread_block 1 select the CUDA-core kernels, which compute
the same sums in FP32 with another order: the two must agree to FP32
rounding (1e-5 relative for 1000-tap sums).  Cases cover grid sides that are not multiples of the patch (odd
oversampled sizes), coil counts that leave partial n-tiles and coil chunks,
cut-offs m = 1..4, density weights and crowded patches split over partial
slots.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def kooshball(nspokes, nsamp):
    from codeare_gb300 import synth
    return synth.kooshball3d(nspokes, nsamp)


def pair(p, N, nc, M, seed):
    rng = np.random.default_rng(seed)
    fh = c64(rng.standard_normal((nc, N, N, N)) + 1j * rng.standard_normal((nc, N, N, N)))
    ys = c64(rng.standard_normal((nc, M)) + 1j * rng.standard_normal((nc, M)))
    return fh, ys


def run(p, fh, ys):
    nc, M = ys.shape
    N = fh.shape[1]
    f = np.zeros((nc, M), np.complex64)
    img = np.zeros((nc, N, N, N), np.complex64)
    p.nfft_trafo(fh, f)
    p.nfft_adjoint(ys, img)
    return f, img


# oversampled sides 48, 45 (odd), 40, 42 (not a multiple of 4), 32
@pytest.mark.parametrize("N,alpha,m,nc", [(24, 2.0, 4, 16), (24, 2.0, 4, 3), (30, 1.5, 4, 5), (20, 2.0, 2, 20),
                                          (28, 1.5, 3, 1), (16, 2.0, 1, 8), (24, 2.0, 4, 33)])
def test_tensor_core_3d_gridding_matches_cuda_cores(gpu, N, alpha, m, nc):
    k = kooshball(400, 2 * N)
    M = k.shape[0]
    p = gpu.Plan((N, N, N), M, ncoils=nc, m=m, alpha=alpha)
    p.set_kspace(k)
    fh, ys = pair(p, N, nc, M, seed=N + nc + m)
    f_tc, img_tc = run(p, fh, ys)
    p.set_tuning(interp_block=1, spread_block=1)
    f_cc, img_cc = run(p, fh, ys)
    p.close()
    assert np.all(np.isfinite(f_tc)) and np.all(np.isfinite(img_tc))
    # 1000-tap FP32 sums in two different orders (the operator bar against the
    # oracle is 2e-5)
    assert rel(f_tc, f_cc) < 1e-5
    assert rel(img_tc, img_cc) < 1e-5


def test_tensor_core_3d_split_patches_and_weights(gpu):
    """A short chunk splits the crowded centre patches over many partial
    slots (reduced in slot order): the result must not depend on the split,
    and density-weighted E^H must match the CUDA-core kernels."""
    from codeare_gb300 import synth
    N, nc = 24, 8
    k = kooshball(900, 2 * N)
    M = k.shape[0]
    w = synth.ramp_weights(k)
    S = c64(synth.coils3d(N, nc))
    p = gpu.Plan((N, N, N), M, ncoils=nc, m=4, alpha=2.0)
    p.set_kspace(k)
    p.set_weights(w)
    p.set_sensitivities(S)
    fh, ys = pair(p, N, nc, M, seed=3)
    f0, img0 = run(p, fh, ys)
    x0 = np.zeros((N, N, N), np.complex64)
    p.sense_adjoint(ys, x0, weighted=True)
    p.set_tuning(spread_chunk=64)
    f1, img1 = run(p, fh, ys)
    x1 = np.zeros_like(x0)
    p.sense_adjoint(ys, x1, weighted=True)
    assert rel(img1, img0) < 1e-5 and rel(x1, x0) < 1e-5
    assert np.array_equal(f1, f0)
    p.set_tuning(interp_block=1, spread_block=1)
    x2 = np.zeros_like(x0)
    p.sense_adjoint(ys, x2, weighted=True)
    p.close()
    assert rel(x0, x2) < 1e-5


def test_tensor_core_3d_gridding_matches_oracle(gpu, oracle):
    N, nc, m, alpha = 20, 4, 4, 2.0
    k = kooshball(300, 2 * N)
    M = k.shape[0]
    p = gpu.Plan((N, N, N), M, ncoils=nc, m=m, alpha=alpha)
    p.set_kspace(k)
    fh, ys = pair(p, N, nc, M, seed=11)
    f, img = run(p, fh, ys)
    p.close()
    P = oracle.NFFT((N, N, N), M, m=m, alpha=alpha)
    P.set_x(k)
    assert rel(f, P.trafo_batch(fh)) < 2e-5
    assert rel(img, P.adjoint_batch(ys)) < 2e-5


def test_tensor_core_3d_repeat_is_bitwise(gpu):
    N, nc = 24, 16
    k = kooshball(600, 2 * N)
    M = k.shape[0]
    p = gpu.Plan((N, N, N), M, ncoils=nc, m=4, alpha=2.0)
    p.set_kspace(k)
    fh, ys = pair(p, N, nc, M, seed=5)
    a = run(p, fh, ys)
    b = run(p, fh, ys)
    p.close()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
