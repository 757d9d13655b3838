"""Generate the 64^3 kooshball fixture: the FP64 oracle's standard CG-SENSE
solution of a 64^3 downsample of the 128^3 kooshball workload.

The downsample keeps the workload's construction and halves every length:
64^3 3-D Shepp-Logan (tabulated intensities), 16 Gaussian coils (sigma 0.45
FOV) on a Fibonacci sphere, 5000 kooshball spokes x 128 samples (the same
spokes per N^2 and the same 2x readout oversampling as 20000 x 256 at 128^3),
|k|^2 density weights, sigma = 2, m = 4, noise-free data.  The oracle runs
conjugate gradients on the weighted normal equations E^H W E x = E^H W y with
its FP64 NFFT pair until ||r||/||r0|| <= 1e-4.

Stored (tests/golden/kooshball64.npz): the solution x (complex64), the
iteration count and the residual history.  The data y is not stored: a test
recomputes it with the oracle's FP64 forward operator (a few seconds), so the
fixture stays small.  The run takes a few minutes on 8 host cores.

Run:  python tests/golden/make_kooshball64.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from codeare_gb300 import synth  # noqa: E402

N, NC, SPOKES, SAMPLES = 64, 16, 5000, 128
TOL = 1e-4
OUT = os.path.join(HERE, "kooshball64.npz")


def case():
    """The downsampled workload (shared with the test that reads the fixture)."""
    c = synth.kooshball3d_64_downsample()
    assert c["shape"] == (N, N, N) and c["sens"].shape[0] == NC and c["k"].shape[0] == SPOKES * SAMPLES
    return c


def main():
    c = case()
    t0 = time.time()
    s = O.Sense(c["sens"], c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
    y = s.trafo(c["image"]).astype(np.complex64)
    x, res = s.cg(y, maxit=200, tol=TOL, lam=0.0, weighted=True)
    it = len(res) - 1
    print("oracle CG: %d iterations, final %.3e, %.1f s" % (it, res[-1], time.time() - t0))
    np.savez_compressed(OUT, x=x.astype(np.complex64), iterations=it, res=res, N=N, nc=NC,
                        spokes=SPOKES, samples=SAMPLES, tol=TOL)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
