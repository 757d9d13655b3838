"""Bounded device waits: the path a tensor-core kernel takes when its MMA
wait runs out, exercised without any fault.

cgs_diag_wait_timeout runs the tensor-core kernels' bounded mbarrier wait on
a barrier that nothing completes.  The wait gives up after its limit and sets
the process-wide timeout flag, and the call reports CGS_ERR_TIMEOUT.  The
flag is reported once, and the context stays usable: an NFFT through a plan
right after it matches the same NFFT before it."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _nfft(cg, synth, N=64, nc=8):
    k = synth.radial2d(48, 2 * N, golden=True)
    rng = np.random.default_rng(3)
    fh = (rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N))).astype(np.complex64)
    p = cg.Plan((N, N), k.shape[0], ncoils=nc, m=4, alpha=2.0)
    p.set_kspace(k)
    f = np.zeros((nc, k.shape[0]), np.complex64)
    p.nfft_trafo(fh, f)
    p.close()
    return f


def test_bounded_wait_runs_out_and_reports_timeout(gpu):
    from codeare_gb300 import capi, synth
    L = capi.load()
    before = _nfft(gpu, synth)
    t0 = time.perf_counter()
    st = L.cgs_diag_wait_timeout(20_000_000, None)   # 20 ms
    dt = time.perf_counter() - t0
    assert st == capi.CGS_ERR_TIMEOUT, L.cgs_last_error()
    assert b"timed out" in L.cgs_last_error()
    assert 0.015 < dt < 10.0
    # reported once: the next call of the library succeeds, with the same result
    after = _nfft(gpu, synth)
    assert np.all(np.isfinite(after))
    assert np.array_equal(after, before)


def test_diag_wait_rejects_limits_outside_one_second(gpu):
    from codeare_gb300 import capi
    L = capi.load()
    for lim in (0, -5, 2_000_000_000):
        assert L.cgs_diag_wait_timeout(lim, None) == capi.CGS_ERR_BAD_ARG
