"""Generate the small golden fixtures of the CG-SENSE path.

The reference cannot run here (it needs NFFT3, FFTW, Boost, ...; see the
oracle header), so these vectors come from the FP64 oracle restatement and are
cross-checked at generation time against a dense numpy NDFT (exact operator,
sigma=2, m=4) and against the oracle's own adjointness.  They pin the oracle
and the CUDA path against regressions; they do not pin either to NFFT3.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from codeare_gb300 import synth  # noqa: E402


def case2d(name, N, nc, nspokes, nsamp, alpha, m, seed):
    rng = np.random.default_rng(seed)
    k = synth.radial2d(nspokes, nsamp, golden=True)
    w = synth.ramp_weights(k)
    S = synth.coils2d(N, nc)
    x = synth.phantom(N) * np.exp(1j * 0.3).astype(np.complex64)
    fh = (rng.standard_normal((nc, N, N)) + 1j * rng.standard_normal((nc, N, N))).astype(np.complex64)
    ys = (rng.standard_normal((nc, k.shape[0])) + 1j * rng.standard_normal((nc, k.shape[0]))).astype(np.complex64)
    sense = O.Sense(S, k, w=w, m=m, alpha=alpha, threads=1)
    P = sense.nfft
    trafo = np.stack([P.trafo(fh[c]) for c in range(nc)])
    adjoint = np.stack([P.adjoint(ys[c]) for c in range(nc)])
    itrafo = np.stack([P.itrafo(ys[c], w, sense.what, 3, 1e-3)[0] for c in range(nc)])
    y = sense.trafo(x)
    eh_codeare = sense.adjoint_codeare(y, 3, 1e-3)
    eh_true = sense.adjoint(y, weighted=True)
    x_cgls, res = sense.cgls_codeare(y, cgiter=5, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
    x_cg, res_cg = sense.cg(y, maxit=8, tol=1e-10, lam=0.0, weighted=True)
    if alpha >= 2.0 and m >= 4:
        A = O.ndft_matrix(k, (N, N))
        ref = A @ fh[0].reshape(-1)
        err = np.linalg.norm(trafo[0] - ref) / np.linalg.norm(ref)
        assert err < 1e-6, err
    np.savez_compressed(os.path.join(HERE, name + ".npz"), N=N, nc=nc, alpha=alpha, m=m, k=k, w=w, S=S,
                        x=x, fh=fh, ys=ys, trafo=trafo, adjoint=adjoint, itrafo=itrafo, y=y,
                        eh_codeare=eh_codeare, eh_true=eh_true, x_cgls=x_cgls, res_cgls=res,
                        x_cg=x_cg, res_cg=res_cg, what=sense.what, imap=sense.I)


def case3d(name, N, nc, nspokes, nsamp, alpha, m, seed):
    rng = np.random.default_rng(seed)
    k = synth.kooshball3d(nspokes, nsamp)
    fh = (rng.standard_normal((nc, N, N, N)) + 1j * rng.standard_normal((nc, N, N, N))).astype(np.complex64)
    ys = (rng.standard_normal((nc, k.shape[0])) + 1j * rng.standard_normal((nc, k.shape[0]))).astype(np.complex64)
    P = O.NFFT((N, N, N), k.shape[0], m=m, alpha=alpha)
    P.set_x(k)
    trafo = np.stack([P.trafo(fh[c]) for c in range(nc)])
    adjoint = np.stack([P.adjoint(ys[c]) for c in range(nc)])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), N=N, nc=nc, alpha=alpha, m=m, k=k, fh=fh, ys=ys,
                        trafo=trafo, adjoint=adjoint)


if __name__ == "__main__":
    case2d("small2d_s2m4", N=16, nc=2, nspokes=12, nsamp=32, alpha=2.0, m=4, seed=1)
    case2d("small2d_s1m1", N=16, nc=2, nspokes=12, nsamp=32, alpha=1.0, m=1, seed=2)
    case3d("small3d_s2m2", N=8, nc=2, nspokes=40, nsamp=16, alpha=2.0, m=2, seed=3)
    print("written to", HERE)
