"""Learned preconditioner for flexible CG-SENSE (configuration 4 workload).

Problem family: 2-D radial, 256^2 image, 16 coils, golden-angle radial with
32-100 spokes of 512 samples, random phantoms of 8-20 ellipses with uniform
complex intensities.  The normal equations are the standard-mode ones,
(E^H W E + lambda I) x = E^H W y, applied by Toeplitz embedding.

Training pairs (residual r, correction e): r is a plain-CG residual
b - A x_k at a random iteration k of a random problem, e = CG_20(A, r) is the
20-iteration plain-CG solution of A e = r from zero.  The preconditioner is
z = C r + d . net(t), t = d . r, with d = diag(A)^-1/2 (exact: sum_c |S_c|^2
sum_j w_j + lambda) and C the circulant of cgs_precond_apply (a global step:
the inverse of the floored T. Chan spectrum of the point-spread function,
between coil-energy scalings).  The network corrects the circulant step
locally, so its pairs are (t, (e - C r) / d), both divided by the RMS of t
(the network is positively homogeneous, so the scale is exact) and stored as
[H][W][2] float.  With base="jacobi" the older form z = d . (t + net(t))
(pairs (t, e / d - t)) is trained instead.  The network is include/cgs.h's
cgs_net_*; cgs_solve_fcg applies the scaling.

All compute runs in libcgs.so; torch only holds device buffers and slices
random training crops.
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np

from . import capi, synth

WEIGHTS_MAGIC = b"CGSN"


def ellipse_phantom(n: int, rng) -> np.ndarray:
    """8-20 random ellipses with uniform complex intensities (|v| <= 1)."""
    img = np.zeros((n, n), np.complex64)
    yy, xx = np.meshgrid((np.arange(n) - n / 2) / (n / 2), (np.arange(n) - n / 2) / (n / 2), indexing="ij")
    for _ in range(int(rng.integers(8, 21))):
        a, b = rng.uniform(0.05, 0.6, 2)
        cy, cx = rng.uniform(-0.6, 0.6, 2)
        th = rng.uniform(0, math.pi)
        v = complex(rng.uniform(-1, 1), rng.uniform(-1, 1))
        xr = (xx - cx) * math.cos(th) + (yy - cy) * math.sin(th)
        yr = -(xx - cx) * math.sin(th) + (yy - cy) * math.cos(th)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += v
    return img


def density(k):
    """ramp density compensation with a floor so the k-space centre keeps weight"""
    w = synth.ramp_weights(k)
    return (w + 0.5 / 512.0).astype(np.float32)


class Problem:
    """One configuration-4 instance on the GPU (plan, data, normal-equation rhs)."""

    def __init__(self, seed: int, N: int = 256, nc: int = 16, nsamp: int = 512, spokes=None,
                 sens=None, lam_rel: float = 1e-3, noise: float = 1e-3):
        import torch
        rng = np.random.default_rng(seed)
        self.N, self.nc = N, nc
        self.spokes = int(spokes if spokes is not None else rng.integers(32, 101))
        self.k = synth.radial2d(self.spokes, nsamp, golden=True)
        self.w = density(self.k)
        self.S = sens if sens is not None else synth.coils2d(N, nc)
        self.x_true = ellipse_phantom(N, rng)
        M = self.k.shape[0]
        self.plan = capi.Plan((N, N), M, ncoils=nc, m=4, alpha=2.0)
        self.plan.set_kspace(self.k)
        self.plan.set_weights(self.w)
        self.plan.set_sensitivities(np.ascontiguousarray(self.S))
        y = np.zeros((nc, M), np.complex64)
        self.plan.sense_trafo(self.x_true, y)
        self.y = synth.add_noise(y, noise, seed=seed + 7)
        # Tikhonov weight relative to the mean diagonal of E^H W E
        diag = float(np.sum(self.w)) * float(np.mean(np.sum(np.abs(self.S) ** 2, axis=0)))
        self.diag = diag
        self.lam = lam_rel * diag
        ssq = np.sum(np.abs(self.S) ** 2, axis=0)
        self.d = torch.from_numpy((1.0 / np.sqrt(ssq * float(np.sum(self.w, dtype=np.float64)) + self.lam))
                                  .astype(np.float32)).cuda()
        self.y_d = torch.from_numpy(self.y).cuda()
        b = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
        self.plan.sense_adjoint(self.y_d, b, weighted=True)
        self.b = b

    def solve(self, x, rhs=None, net=None, cgiter=500, cgeps=1e-4, jacobi=False, circulant=False):
        return self.plan.solve_fcg(x, rhs=self.b if rhs is None else rhs, net=net, cgiter=cgiter, cgeps=cgeps,
                                   lam=self.lam, weighted=True, toeplitz=True, jacobi=jacobi,
                                   circulant=circulant)

    def precond(self, r, out):
        return self.plan.precond_apply(r, out, lam=self.lam, weighted=True)

    def apply(self, x, out):
        return self.plan.normal_apply(x, out, lam=self.lam, weighted=True, toeplitz=True)

    def close(self):
        self.plan.close()


def as_channels(z):
    """complex [H][W] tensor -> float [H][W][2]"""
    import torch
    return torch.view_as_real(z).contiguous()


def generate_pairs(n_pairs: int, seed: int = 20261207, per_problem: int = 8, N: int = 256, nc: int = 16,
                   k_max: int = 60, corr_iters: int = 20, base: str = "circulant", log=None):
    """(t = d . residual, (correction - C residual) / d) pairs on the GPU (with
    base="jacobi": (t, correction / d - t)), each divided by the RMS of t."""
    import torch
    X = torch.empty((n_pairs, N, N, 2), dtype=torch.float32, device="cuda")
    T = torch.empty_like(X)
    rng = np.random.default_rng(seed)
    S = synth.coils2d(N, nc)
    i = 0
    prob_id = 0
    while i < n_pairs:
        pr = Problem(seed + 1000 * prob_id, N=N, nc=nc, sens=S)
        prob_id += 1
        x = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
        Ax = torch.zeros_like(x)
        e = torch.zeros_like(x)
        for _ in range(per_problem):
            if i >= n_pairs:
                break
            kk = int(rng.integers(0, k_max + 1))
            if kk == 0:
                r = pr.b.clone()
            else:
                pr.solve(x, cgiter=kk, cgeps=0.0)
                pr.apply(x, Ax)
                r = pr.b - Ax
            r = r.contiguous()
            pr.solve(e, rhs=r, cgiter=corr_iters, cgeps=0.0)
            rs = r * pr.d
            s = torch.sqrt(torch.mean(torch.view_as_real(rs) ** 2)).clamp_min(1e-30)
            X[i] = as_channels(rs / s)
            if base == "circulant":
                cr = torch.zeros_like(r)
                pr.precond(r, cr)
                T[i] = as_channels((e - cr) / pr.d / s)
            else:
                T[i] = as_channels((e / pr.d - rs) / s)
            i += 1
        pr.close()
        if log and prob_id % 16 == 0:
            log("pairs %d / %d" % (i, n_pairs))
    return X, T


def train(net, X, T, steps: int = 2000, batch: int = 32, crop: int = 64, lr: float = 1e-3, seed: int = 3,
          log=None):
    """Adam on random crops; returns the loss history."""
    import torch
    P, N = X.shape[0], X.shape[1]
    g = torch.Generator(device="cpu").manual_seed(seed)
    xb = torch.empty((batch, crop, crop, 2), dtype=torch.float32, device="cuda")
    tb = torch.empty_like(xb)
    hist = []
    for it in range(steps):
        idx = torch.randint(0, P, (batch,), generator=g)
        oy = torch.randint(0, N - crop + 1, (batch,), generator=g)
        ox = torch.randint(0, N - crop + 1, (batch,), generator=g)
        for b in range(batch):
            xb[b] = X[idx[b], oy[b]:oy[b] + crop, ox[b]:ox[b] + crop]
            tb[b] = T[idx[b], oy[b]:oy[b] + crop, ox[b]:ox[b] + crop]
        step_lr = lr * (0.5 * (1 + math.cos(math.pi * it / steps)))
        want = (it % 50 == 0) or it == steps - 1
        loss = net.train_step(xb, tb, lr=step_lr, want_loss=want)
        if want:
            hist.append((it, loss))
            if log:
                log("step %d loss %.4e" % (it, loss))
    return hist


def save_weights(path: str, w: np.ndarray, meta: str = ""):
    w = np.ascontiguousarray(w, dtype=np.float32)
    mb = meta.encode()
    with open(path, "wb") as f:
        f.write(WEIGHTS_MAGIC)
        f.write(struct.pack("<II", w.size, len(mb)))
        f.write(mb)
        f.write(w.tobytes())


def load_weights(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        assert f.read(4) == WEIGHTS_MAGIC
        n, lm = struct.unpack("<II", f.read(8))
        f.read(lm)
        return np.frombuffer(f.read(4 * n), dtype=np.float32).copy()


WEIGHTS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "precond_weights.bin")


def load_net(path: str = WEIGHTS_FILE):
    """the trained network from `path`, or None when there is no weights file"""
    if not os.path.exists(path):
        return None
    net = capi.Net(max_batch=1, max_h=256, max_w=256)
    net.set_weights(load_weights(path))
    return net


def compare(net, seed: int, cgeps: float = 1e-4, ref_eps: float = 1e-6, repeats: int = 2, spokes=None):
    """Plain CG, Jacobi-preconditioned CG, circulant-preconditioned CG and
    learned flexible CG (the circulant step plus the network's correction) on
    one held-out problem to relative residual `cgeps` (the second of `repeats`
    timed solves is kept: the first builds the solve graph), each image's
    relative L2 error against the plain solve converged to `ref_eps`."""
    import torch
    pr = Problem(seed, spokes=spokes)
    N = pr.N
    ref = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    pr.solve(ref, cgiter=2000, cgeps=ref_eps)
    out = {"seed": seed, "spokes": pr.spokes}
    arms = [("plain", {}), ("jacobi", {"jacobi": True}), ("circulant", {"circulant": True})]
    if net is not None:
        arms.append(("learned", {"net": net, "circulant": True}))
    for name, kw in arms:
        x = torch.zeros_like(ref)
        for _ in range(repeats):
            rep = pr.solve(x, cgiter=2000, cgeps=cgeps, **kw)
        err = float(torch.linalg.vector_norm(x - ref) / torch.linalg.vector_norm(ref))
        out[name] = {"iterations": rep["iterations"], "ms": 1e3 * rep["seconds"], "res": rep["res_last"],
                     "fallback_at": rep["fallback_at"], "image_err": err}
    pr.close()
    return out


HELD_OUT = [(9001, 32), (9002, 40), (9003, 50), (9004, 60), (9005, 70), (9006, 80), (9007, 90), (9008, 100)]


def compare_many(net, problems=HELD_OUT, cgeps: float = 1e-4):
    """compare() over held-out problems spread over 32-100 spokes; per arm the
    median speed-up against plain CG and the worst image error."""
    rows = [compare(net, seed, cgeps=cgeps, spokes=sp) for seed, sp in problems]
    arms = [a for a in ("jacobi", "circulant", "learned") if a in rows[0]]
    summary = {}
    for a in arms:
        sp = [r["plain"]["ms"] / r[a]["ms"] for r in rows]
        it = [r["plain"]["iterations"] / max(1, r[a]["iterations"]) for r in rows]
        summary[a] = {"median_speedup_vs_plain": float(np.median(sp)), "min_speedup": float(np.min(sp)),
                      "median_iteration_ratio": float(np.median(it)),
                      "max_image_err": float(max(r[a]["image_err"] for r in rows))}
    summary["plain_max_image_err"] = float(max(r["plain"]["image_err"] for r in rows))
    return rows, summary


def main(argv=None):
    """python -m codeare_gb300.learned [--pairs P] [--steps S] [--lr LR] [--out FILE]:
    generate pairs with the plain solver, train on the GPU, write the weights."""
    import argparse
    import time
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=WEIGHTS_FILE)
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    t0 = time.time()
    X, T = generate_pairs(a.pairs, log=log)
    torch.cuda.synchronize()
    ms = float((T ** 2).mean())
    log("pairs %d in %.1f s, target mean square %.4g" % (a.pairs, time.time() - t0, ms))
    net = capi.Net(max_batch=32, max_h=256, max_w=256)
    t0 = time.time()
    hist = train(net, X, T, steps=a.steps, lr=a.lr)
    torch.cuda.synchronize()
    last = float(np.mean([h[1] for h in hist[-5:]]))
    log("trained %d steps in %.1f s, relative loss %.3f -> %.3f" % (a.steps, time.time() - t0, hist[0][1] / ms,
                                                                    last / ms))
    save_weights(a.out, net.weights(), "pairs=%d steps=%d lr=%g rel_loss=%.4f" % (a.pairs, a.steps, a.lr,
                                                                                   last / ms))
    del X, T
    rows, summary = compare_many(net)
    for r in rows:
        log(str(r))
    log(str(summary))


if __name__ == "__main__":
    main()
