"""The allocation-free NFFT forward (cgs_nfft2d_trafo_noalloc).

It serves callers that may not allocate device memory while they run, such as
a real-time reconstruction loop beside an acquisition stream (cudaMalloc and
cudaFree synchronise the device) or a host with its own fixed device-memory
pool.  Its scratch is a static 4 MiB device array shared by every call.  This
test calls it through the C ABI twice in a row, with different inputs, and
checks each result against the plan-based entry point (cgs_nfft_trafo) within
the per-operator tolerance of the parity tests, on power-of-two and
mixed-radix grids, several cut-offs and the largest admitted size.  It pins
the NaN output for nodes outside [-0.5, 0.5).  It also checks that sizes
beyond the static array are rejected.  This file sorts last so that a stop at
the first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_OP = 2e-5


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


# (N, alpha, m): a power-of-two grid (n = 256), a mixed-radix grid with a
# non-integer oversampling (n = 180 = 4 * 3^2 * 5, the runtime-radix FFT) at
# two cut-offs, and the largest square image the static array admits
CASES = [(128, 2.0, 4), (120, 1.5, 2), (120, 1.5, 6), (256, 2.0, 4)]


def _call(L, N, alpha, m, k_d, fh_d, out_d):
    import ctypes as C
    return L.cgs_nfft2d_trafo_noalloc(N, alpha, m, k_d.shape[0], C.c_void_p(k_d.data_ptr()),
                                      C.c_void_p(fh_d.data_ptr()), C.c_void_p(out_d.data_ptr()), None)


@pytest.mark.parametrize("N,alpha,m", CASES)
def test_noalloc_forward_matches_plan_entry_point(gpu, N, alpha, m):
    import torch
    from codeare_gb300 import capi, synth

    L = capi.load()
    k = synth.radial2d(96, 2 * N)        # N^2 image, 96 uniform spokes x 2N samples
    M = k.shape[0]
    plan = gpu.Plan((N, N), M, ncoils=1, m=m, alpha=alpha)
    plan.set_kspace(k)
    k_d = torch.from_numpy(k).cuda()
    rng = np.random.default_rng(77 + N + m)
    for call in range(2):
        fh = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
        fh_d = torch.from_numpy(fh).cuda()
        ref = np.zeros((1, M), np.complex64)
        plan.nfft_trafo(fh[None], ref)
        out_d = torch.full((M,), float("nan"), dtype=torch.complex64, device="cuda")
        st = _call(L, N, alpha, m, k_d, fh_d, out_d)
        assert st == capi.CGS_OK, L.cgs_last_error()
        torch.cuda.synchronize()
        out = out_d.cpu().numpy()
        assert np.all(np.isfinite(out)), "call %d" % call
        assert rel(out, ref[0]) < TOL_OP, "call %d" % call
    plan.close()


def test_noalloc_node_outside_range_gives_nan(gpu):
    """A coordinate at +0.5 is outside [-0.5, 0.5): that node's value is NaN,
    the call still succeeds and every other node matches the plan path."""
    import torch
    from codeare_gb300 import capi, synth

    L = capi.load()
    N, alpha, m = 64, 2.0, 4
    k = synth.radial2d(32, 2 * N)
    M = k.shape[0]
    plan = gpu.Plan((N, N), M, ncoils=1, m=m, alpha=alpha)
    plan.set_kspace(k)
    rng = np.random.default_rng(5)
    fh = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    ref = np.zeros((1, M), np.complex64)
    plan.nfft_trafo(fh[None], ref)
    plan.close()
    bad = k.copy()
    bad[7, 0] = 0.5
    bad[11, 1] = 0.5
    out_d = torch.zeros(M, dtype=torch.complex64, device="cuda")
    st = _call(L, N, alpha, m, torch.from_numpy(bad).cuda(), torch.from_numpy(fh).cuda(), out_d)
    assert st == capi.CGS_OK, L.cgs_last_error()
    out = out_d.cpu().numpy()
    assert np.isnan(out[7]) and np.isnan(out[11])
    keep = np.ones(M, bool)
    keep[[7, 11]] = False
    assert np.all(np.isfinite(out[keep]))
    assert rel(out[keep], ref[0][keep]) < TOL_OP


def test_noalloc_rejects_sizes_beyond_the_static_array(gpu):
    import torch
    from codeare_gb300 import capi

    L = capi.load()
    dummy = torch.zeros(8, dtype=torch.complex64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    st = L.cgs_nfft2d_trafo_noalloc(512, 2.0, 4, 4, p, p, p, None)
    assert st == capi.CGS_ERR_BAD_ARG
    assert b"static scratch" in L.cgs_last_error()
    st = L.cgs_nfft2d_trafo_noalloc(128, float("inf"), 4, 4, p, p, p, None)
    assert st == capi.CGS_ERR_BAD_ARG
    assert b"2048" in L.cgs_last_error()
