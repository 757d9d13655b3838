"""The allocation-free NFFT forward (cgs_nfft2d_trafo_noalloc).

It serves callers that may not allocate device memory while they run, such as
a real-time reconstruction loop beside an acquisition stream (cudaMalloc and
cudaFree synchronise the device) or a host with its own fixed device-memory
pool.  Its scratch is a static 4 MiB device array shared by every call.  This
test calls it through the C ABI twice in a row, with different inputs, and
checks each result against the plan-based entry point (cgs_nfft_trafo) within
the per-operator tolerance of the parity tests.  It also checks that sizes
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


def test_noalloc_forward_matches_plan_entry_point(gpu):
    import torch
    from codeare_gb300 import capi, synth

    L = capi.load()
    N, alpha, m = 128, 2.0, 4
    k = synth.radial2d(96, 256)          # 128^2 image, 96 uniform spokes x 256 samples
    M = k.shape[0]
    plan = gpu.Plan((N, N), M, ncoils=1, m=m, alpha=alpha)
    plan.set_kspace(k)
    k_d = torch.from_numpy(k).cuda()
    rng = np.random.default_rng(77)
    for call in range(2):
        fh = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
        fh_d = torch.from_numpy(fh).cuda()
        ref = np.zeros((1, M), np.complex64)
        plan.nfft_trafo(fh[None], ref)
        out_d = torch.full((M,), float("nan"), dtype=torch.complex64, device="cuda")
        st = L.cgs_nfft2d_trafo_noalloc(N, alpha, m, M, C.c_void_p(k_d.data_ptr()),
                                        C.c_void_p(fh_d.data_ptr()), C.c_void_p(out_d.data_ptr()), None)
        assert st == capi.CGS_OK, L.cgs_last_error()
        torch.cuda.synchronize()
        out = out_d.cpu().numpy()
        assert np.all(np.isfinite(out)), "call %d" % call
        assert rel(out, ref[0]) < TOL_OP, "call %d" % call
    plan.close()


def test_noalloc_rejects_sizes_beyond_the_static_array(gpu):
    import torch
    from codeare_gb300 import capi

    L = capi.load()
    dummy = torch.zeros(8, dtype=torch.complex64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    st = L.cgs_nfft2d_trafo_noalloc(512, 2.0, 4, 4, p, p, p, None)
    assert st == capi.CGS_ERR_BAD_ARG
    assert b"static scratch" in L.cgs_last_error()
