#!/usr/bin/env python
"""Benchmark of the NuFFT operator on the 256^2, 32-coil golden-angle radial workload.

Workload (one "step"): the per-coil NFFT forward (32 coil images -> k-space)
followed by the per-coil adjoint (k-space -> 32 coil images) of a 256^2 image,
32 coils, golden-angle radial trajectory of 403 spokes x 512 samples, sigma=2
(512^2 oversampled grid), Kaiser-Bessel m=4.  Seeded synthetic inputs stand in
for scanner data (none is published for this path).

Metric: NuFFT GB/s = algorithmic bytes of one forward+adjoint (per-pass model:
deapodise/pad, FFT, interpolation; spreading, FFT, crop/deapodise) / time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device-resident (inputs already in HBM, device pointers through the
C ABI, L2 flushed before each timed step); `e2e` is the same metric through
the C ABI with pinned HOST buffers, host<->device copies inside the timed
region.  The reference arm times the FP64 CPU restatement of the reference's
NFFT3 path (oracle/): the reference itself needs NFFT3, FFTW, Boost and its
CMake build, none of which this image has.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NuFFT GB/s (per-coil NFFT forward + adjoint)"
UNIT = "GB/s"
N, NC, SPOKES, SAMPLES, SIGMA, M_KB = 256, 32, 403, 512, 2.0, 4
WORKLOAD = ("NuFFT forward+adjoint, 256^2 image x 32 coils, golden-angle radial "
            "403x512 (M=206336), sigma=2 (512^2 grid), KB m=4")


def algorithmic_bytes(N, n, M, d, nc):
    """Per-pass byte model (complex64 = 8 B, coordinates float32)."""
    img = nc * N ** d * 8
    grid = nc * n ** d * 8
    ks = nc * M * 8
    coords = M * d * 4
    b = {
        "pad_deapod": img + grid,
        "fft": 2 * grid,                 # per transform
        "interp": grid + coords + ks,
        "spread": coords + ks + grid,
        "crop_deapod": grid + img,
    }
    b["forward"] = b["pad_deapod"] + b["fft"] + b["interp"]
    b["adjoint"] = b["spread"] + b["fft"] + b["crop_deapod"]
    b["step"] = b["forward"] + b["adjoint"]
    return b


def pruned_fft_bytes(N, n, nc):
    """Bytes the four 2-D FFT passes of a forward + adjoint step must move
    when the zero rows of the padded image are neither read nor transformed
    and the cropped rows are not written: forward along x (N rows: image in,
    N x n out), forward along y (N x n in, n x n out), inverse along y (n x n
    in, N x n out), inverse along x (N x n in, image out)."""
    img, mid, grid = nc * N * N * 8, nc * N * n * 8, nc * n * n * 8
    return 2 * (img + mid) + 2 * (mid + grid)


def workload_data(seed=20261204):
    from codeare_gb300 import synth
    k = synth.radial2d(SPOKES, SAMPLES, golden=True)
    rng = np.random.default_rng(seed)
    fh = (rng.standard_normal((NC, N, N)) + 1j * rng.standard_normal((NC, N, N))).astype(np.complex64)
    return k, fh


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [q.strip() for q in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo) and core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                name = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith(("model name", "cpu model")):
                    name = ln.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"model": name or "unknown", "nproc": os.cpu_count() or 1}


class CpuNfftStep:
    """FP64 CPU restatement of the reference's per-coil NFFT3 trafo+adjoint
    (oracle/), one coil per host thread as NCSENSE runs one plan per thread.
    The window values are precomputed once per trajectory (NFFT3's PRE_PSI,
    which codeare sets) outside the timed call."""

    def __init__(self, k, fh, threads):
        from oracle import oracle as O
        O.build()
        self.P = O.NFFT((N, N), k.shape[0], m=M_KB, alpha=SIGMA)
        self.P.set_x(k.astype(np.float64))
        self.fh64 = fh.astype(np.complex128)
        self.threads = threads

    def __call__(self):
        t0 = time.perf_counter()
        f = self.P.trafo_batch(self.fh64, threads=self.threads)
        self.P.adjoint_batch(f, threads=self.threads)
        return time.perf_counter() - t0


def cpu_baseline_leg(k, fh, warmup=1, runs=5):
    """The CPU baseline protocol: all 32 coils, `warmup` untimed steps, then the
    median of `runs` timed steps, with the host's core count and CPU model."""
    cpu = cpu_model()
    threads = cpu["nproc"]
    step = CpuNfftStep(k, fh, threads)
    for _ in range(warmup):
        step()
    times = [step() for _ in range(runs)]
    t = statistics.median(times)
    b = algorithmic_bytes(N, int(N * SIGMA), k.shape[0], 2, fh.shape[0])["step"]
    return {"value": b / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu["model"],
            "seconds": t, "runs_s": times,
            "sample": "all %d coils, one forward+adjoint per run, %d warm-up + median of %d; one coil per "
                      "thread; FP64 C restatement of the NFFT3 path with the project's own FFT (the "
                      "reference needs NFFT3/FFTW/Boost, absent here)" % (fh.shape[0], warmup, runs)}


def run_reference(args):
    ws, rank, local = dist_setup()
    if rank != 0:
        return 0
    k, fh = workload_data()
    cpu = cpu_model()
    threads = cpu["nproc"]
    step = CpuNfftStep(k, fh, threads)      # every step: all 32 coils, as the GPU arm
    b = algorithmic_bytes(N, int(N * SIGMA), k.shape[0], 2, NC)["step"]
    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    t = sum(times) / len(times)
    v = b / t / 1e9
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": WORKLOAD, "N": N, "n": int(N * SIGMA), "M": int(k.shape[0]), "ncoils": NC,
                   "m": M_KB, "alg_bytes_per_step": b},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu["model"],
                         "sample": "all 32 coils per step, one forward+adjoint, one coil per host thread; "
                                   "FP64 C restatement of the NFFT3 path with the project's own FFT "
                                   "(the reference needs NFFT3/FFTW/Boost, absent here)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def rel_l2(a, b):
    a = np.ravel(np.asarray(a)); b = np.ravel(np.asarray(b))
    return float(np.linalg.norm(a - b) / max(float(np.linalg.norm(b)), 1e-300))


def cgsense_section(cpu_too: bool):
    """CG-SENSE on 128^2 Shepp-Logan, 8 coils, 96 uniform spokes x 256, sigma=2, m=4.
    Times (GPU, inputs already on the device through the C ABI):
      - codeare mode (CGLS over the CGNR-based E^H), 10 iterations, lambda = 5e-2;
      - standard mode (true adjoint) to ||r||/||r0|| = 1e-4, with E^H W E applied by the
        NFFT pair and by the Toeplitz embedding.
    The CPU leg runs the FP64 oracle's codeare-mode solve on the same input."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import synth
    c = synth.radial2d_128_8coils()
    N, nc = c["shape"][0], c["sens"].shape[0]
    k, w, S = c["k"], c["w"], c["sens"]
    M = k.shape[0]
    p = cg.Plan((N, N), M, ncoils=nc, m=c["m"], alpha=c["alpha"])
    p.set_kspace(k)
    p.set_weights(w)
    p.set_sensitivities(S)
    p.autotune()
    y = np.zeros((nc, M), np.complex64)
    p.sense_trafo(np.ascontiguousarray(c["image"]), y)
    y = synth.add_noise(y, c["noise"], seed=c["seed"])
    yd = torch.from_numpy(y).cuda()
    xd = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    out = {"workload": "128^2, 8 coils, 96x256 uniform radial, sigma=2, m=4, 1e-3 noise"}

    def timed(**kw):
        p.solve(yd, xd, **kw)  # warm-up (and Toeplitz kernel build)
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rep = p.solve(yd, xd, **kw)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            if best is None or wall < best[0]:
                best = (wall, rep)
        wall, rep = best
        return {"iterations": rep["iterations"], "wall_ms": wall * 1e3, "device_ms": rep["seconds"] * 1e3,
                "res_last": rep["res_last"]}

    out["codeare_10it"] = timed(mode=cg.MODE_CODEARE, cgiter=10, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
    x_codeare = xd.cpu().numpy()
    # the same CGLS with every CG step's E^H(E p) on the Toeplitz kernel (inner CGNR in image space)
    out["codeare_10it_toeplitz"] = timed(mode=cg.MODE_CODEARE, cgiter=10, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3,
                                         toeplitz=True)
    x_codeare_t = xd.cpu().numpy()
    # standard mode to ||r||/||r0|| = 1e-4 (the cap is far above the ~250 iterations it takes)
    out["standard_to_1e-4_nfft"] = timed(mode=cg.MODE_STANDARD, cgiter=1000, cgeps=1e-4, lam=0.0, weighted=True)
    out["standard_to_1e-4_toeplitz"] = timed(mode=cg.MODE_STANDARD, cgiter=1000, cgeps=1e-4, lam=0.0,
                                             weighted=True, toeplitz=True)
    x_std = xd.cpu().numpy()
    for key in ("standard_to_1e-4_nfft", "standard_to_1e-4_toeplitz"):
        out[key]["reached_1e-4"] = bool(out[key]["res_last"] <= 1e-4)
    p.solve(yd, xd, mode=cg.MODE_STANDARD, cgiter=20, cgeps=0.0, lam=0.0, weighted=True, toeplitz=True)
    x_std20 = xd.cpu().numpy()
    p.close()
    # the FP64 oracle on the same data, at the same iteration counts
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    s = O.Sense(S, k, w=w, m=c["m"], alpha=c["alpha"], threads=threads)
    xo, _ = s.cgls_codeare(y, cgiter=10, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)   # also the warm-up
    runs = []
    for _ in range(5 if cpu_too else 0):   # the CPU protocol: 1 warm-up, median of 5
        t0 = time.perf_counter()
        s.cgls_codeare(y, cgiter=10, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
        runs.append(time.perf_counter() - t0)
    out["codeare_10it"]["rel_l2_vs_oracle"] = rel_l2(x_codeare, xo)
    out["codeare_10it_toeplitz"]["rel_l2_vs_oracle"] = rel_l2(x_codeare_t, xo)
    it = out["standard_to_1e-4_toeplitz"]["iterations"]
    xs, _ = s.cg(y, maxit=20, tol=0.0, lam=0.0, weighted=True)
    out["standard_to_1e-4_toeplitz"]["rel_l2_vs_oracle_20it"] = rel_l2(x_std20, xs)
    xs, _ = s.cg(y, maxit=it, tol=0.0, lam=0.0, weighted=True)
    out["standard_to_1e-4_toeplitz"]["rel_l2_vs_oracle_same_iterations"] = rel_l2(x_std, xs)
    out["standard_to_1e-4_toeplitz"]["note"] = (
        "lambda 0 is ill-conditioned (ramp weight 0 at the k-space centre): FP32 and FP64 CG drift apart "
        "(~1e-3 by 40 iterations) and reach 1e-4 along different paths, so the oracle error is also given at "
        "20 iterations")
    if cpu_too:
        out["cpu_codeare_10it"] = {"wall_ms": statistics.median(runs) * 1e3, "cores": threads, "kind": "port",
                                   "runs_ms": [r * 1e3 for r in runs],
                                   "note": "FP64 oracle restatement, one coil per thread; 1 warm-up, median of 5"}
    return out


def cs_section(cpu_too: bool):
    """Compressed sensing over NCSENSE (the CompressedSensing module, ft = 3) on
    the 128^2 radial input: 128^2, 8 coils, 96x256 uniform spokes, sigma=2, m=4,
    with the reference's example CS settings (csiter 2, 8 NLCG iterations,
    10 line-search steps, lsa 0.01, lsb 0.6, TV 0.002, L1 0.005, p = 1,
    l1 1e-15, Daubechies 4) and a 10-iteration codeare CGLS inside every
    gradient.  Times one whole reconstruction on the GPU (device-resident
    data, best of 3).  The CPU leg times one gradient evaluation (E, a CGLS
    solve, the wavelet) of the FP64 oracle on the same input, the unit of
    work a reconstruction repeats once per NLCG iteration."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import synth
    c = synth.radial2d_128_8coils()
    N, nc = c["shape"][0], c["sens"].shape[0]
    k, w, S = c["k"], c["w"], c["sens"]
    M = k.shape[0]
    p = cg.Plan((N, N), M, ncoils=nc, m=c["m"], alpha=c["alpha"])
    p.set_kspace(k)
    p.set_weights(w)
    p.set_sensitivities(S)
    p.autotune()
    y = np.zeros((nc, M), np.complex64)
    p.sense_trafo(np.ascontiguousarray(c["image"]), y)
    y = synth.add_noise(y, c["noise"], seed=c["seed"])
    yd = torch.from_numpy(y).cuda()
    xd = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    kw = dict(tvw=(0.002, 0.0), xfmw=0.005, l1=1e-15, pnorm=1.0, csiter=2, nliter=8, lsiter=10, lsa=0.01,
              lsb=0.6, cgconv=5e-3, wl_family=0, wl_member=4, cgiter=10, cgeps=1e-7, lam=5e-2, ftiter=3,
              fteps=1e-3)
    best = None
    for _ in range(4):  # the first run also captures the solve graph
        h = cg.CS(p, **kw)  # a fresh handle: the TV weight scaling is per call, as in the module
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rep = h.adjoint(yd, xd)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        h.close()
        if best is None or wall < best[0]:
            best = (wall, rep)
    wall, rep = best
    out = {"workload": "CompressedSensing ft=3 on the 128^2 radial case (128^2, 8 coils, 96x256 radial, sigma=2, m=4), "
                       "reference example settings, Daubechies 4",
           "wall_ms": wall * 1e3, "device_ms": rep["seconds"] * 1e3, "nlcg_iterations": rep["iterations"],
           "solves": rep["solves"], "cg_iterations": rep["solve_iterations"],
           "ms_per_solve": wall * 1e3 / max(1, rep["solves"]), "ls_index": rep["ls_index"]}
    p.close()
    if cpu_too:
        from oracle import oracle as O, cs
        threads = os.cpu_count() or 1
        sn = O.Sense(S, k, w=w, m=c["m"], alpha=c["alpha"], threads=threads)
        o = cs.CSXSense(sn, **kw)
        o.set_data(y)
        x0 = xd.cpu().numpy()
        t0 = time.perf_counter()
        o.df(o.W(x0))
        t = time.perf_counter() - t0
        out["cpu_gradient"] = {"wall_ms": t * 1e3, "cores": threads, "kind": "port",
                               "sample": "one CS gradient (E, 10-iteration CGLS, wavelet) of the FP64 oracle",
                               "gpu_ms_per_solve": out["ms_per_solve"]}
    return out


def batch_section():
    """Batch of 64 uneven CG-SENSE problems (N 96..320, 4-32 coils, radial and
    spiral trajectories), codeare-mode CGLS with 15 iterations each, as one
    graph launch (cgs_batch) and as 64 consecutive per-plan solves; the
    autotuner runs on every plan first."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import capi, synth
    probs = synth.uneven_batch()
    t0 = time.perf_counter()
    plans, ys, xs = [], [], []
    for c in probs:
        N, nc, k = c["N"], c["nc"], c["k"]
        p = capi.Plan((N, N), k.shape[0], ncoils=nc, m=c["m"], alpha=c["alpha"])
        p.set_kspace(k)
        p.set_weights(c["w"])
        p.set_sensitivities(synth.coils2d(N, nc))
        y = np.zeros((nc, k.shape[0]), np.complex64)
        p.sense_trafo(np.ascontiguousarray(synth.phantom(N)), y)
        plans.append(p)
        ys.append(torch.from_numpy(synth.add_noise(y, c["noise"], seed=c["seed"])).cuda())
        xs.append(torch.zeros((N, N), dtype=torch.complex64, device="cuda"))
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    for p in plans:
        p.autotune()
    t_tune = time.perf_counter() - t0
    kw = dict(mode=cg.MODE_CODEARE, cgiter=15, cgeps=0.0, lam=5e-2)

    def sequential(**extra):
        return sum(p.solve(y, x, **kw, **extra)["seconds"] for p, y, x in zip(plans, ys, xs))

    sequential()
    t_seq = min(sequential() for _ in range(2))
    b = capi.Batch(plans, capi.solve_opts(**kw))
    b.solve(ys, xs)
    t_batch = min(b.solve(ys, xs)[1] for _ in range(3))
    b.close()
    # every CG step's E^H(E p) on the Toeplitz kernels (the data's E^H y still through the NFFT)
    sequential(toeplitz=True)
    t_seq_t = min(sequential(toeplitz=True) for _ in range(2))
    b = capi.Batch(plans, capi.solve_opts(toeplitz=True, **kw))
    b.solve(ys, xs)
    t_batch_t = min(b.solve(ys, xs)[1] for _ in range(3))
    b.close()
    # the FP64 oracle on four of the problems (the smallest, a spiral among them), same data and iterations
    from oracle import oracle as O
    cost = sorted(range(len(probs)), key=lambda i: probs[i]["nc"] * probs[i]["k"].shape[0])
    check = cost[:3] + [next(i for i in cost if probs[i]["kind"].startswith("spiral"))]
    errs = {}
    for i in dict.fromkeys(check):
        c = probs[i]
        s = O.Sense(synth.coils2d(c["N"], c["nc"]), c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
        xo, _ = s.cgls_codeare(ys[i].cpu().numpy(), cgiter=15, cgeps=0.0, lam=5e-2)
        errs[c["name"]] = rel_l2(xs[i].cpu().numpy(), xo)
    out = {"workload": "64 uneven problems, N 96..320, 4/8/16/32 coils, golden-angle radial 32..400 x 512 "
                       "or VD spiral 16 x 4096, codeare CGLS 15 iterations (lambda 5e-2, 3 inner steps)",
           "problems": len(plans), "coil_samples": int(sum(c["k"].shape[0] * c["nc"] for c in probs)),
           "batch_ms": t_batch * 1e3, "sequential_ms": t_seq * 1e3, "problems_per_s": len(plans) / t_batch,
           "toeplitz": {"batch_ms": t_batch_t * 1e3, "sequential_ms": t_seq_t * 1e3,
                        "problems_per_s": len(plans) / t_batch_t},
           "setup_s": t_setup, "autotune_s": t_tune, "rel_l2_vs_oracle_of": "the Toeplitz batch's images",
           "rel_l2_vs_oracle": errs,
           "rel_l2_vs_oracle_max": max(errs.values())}
    for p in plans:
        p.close()
    return out


def kooshball_section():
    """3-D kooshball CG-SENSE, 128^3, 16 coils, 20000 x 256 spokes,
    standard CG with the Toeplitz-embedded E^H W E (256^3 FFTs) to
    ||r||/||r0|| = 1e-4.  Reports the one-off costs (binning, E^H y, the
    Toeplitz kernel) apart from the iterations."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import capi, synth
    c = synth.kooshball3d_128_16coils()
    N, nc = c["shape"][0], c["sens"].shape[0]
    k = c["k"]
    M = k.shape[0]
    t0 = time.perf_counter()
    p = capi.Plan(c["shape"], M, ncoils=nc, m=c["m"], alpha=c["alpha"])
    p.set_kspace(k)
    p.set_weights(c["w"])
    p.set_sensitivities(np.ascontiguousarray(c["sens"]))
    torch.cuda.synchronize()
    t_plan = time.perf_counter() - t0
    y = torch.zeros((nc, M), dtype=torch.complex64, device="cuda")
    p.sense_trafo(torch.from_numpy(np.ascontiguousarray(c["image"])).cuda(), y)
    y = torch.from_numpy(synth.add_noise(y.cpu().numpy(), c["noise"], seed=c["seed"])).cuda()
    x = torch.zeros(c["shape"], dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p.sense_adjoint(y, x, weighted=True)
    torch.cuda.synchronize()
    t_eh = time.perf_counter() - t0
    # per-kernel CUDA-event times of one E (interpolation) and one E^H W (spreading), 16 coils
    capi.profile_enable(True)
    yk = torch.empty_like(y)
    for _ in range(2):
        p.sense_trafo(x, yk)
        p.sense_adjoint(y, x, weighted=True)
    torch.cuda.synchronize()
    prof = capi.profile_collect()
    capi.profile_enable(False)
    n3 = 2 * N
    kern = {}
    for cat, (ms, cnt) in prof.items():
        if cnt:
            kern[cat] = {"launches": cnt, "avg_ms": ms / cnt}
    gbytes = (M * 3 * 4 + nc * M * 8 + nc * n3 ** 3 * 8)     # coordinates, samples, grid
    for cat in ("interp", "spread"):
        if cat in kern:
            kern[cat]["alg_GBps"] = gbytes / (kern[cat]["avg_ms"] * 1e-3) / 1e9
            kern[cat]["tap_coil_macs_per_s"] = M * nc * 1000.0 / (kern[cat]["avg_ms"] * 1e-3)
    kw = dict(mode=cg.MODE_STANDARD, cgeps=c["cgeps"], lam=0.0, weighted=True, toeplitz=True)
    t0 = time.perf_counter()
    p.solve(y, x, cgiter=1, **kw)   # builds the Toeplitz kernel
    torch.cuda.synchronize()
    t_first = time.perf_counter() - t0
    best = None
    for _ in range(2):
        r = p.solve(y, x, cgiter=300, **kw)
        if best is None or r["seconds"] < best["seconds"]:
            best = r
    p.close()
    it = best["iterations"]
    out = {"workload": "3-D kooshball 128^3, 16 coils, kooshball 20000 x 256, |k|^2 weights, sigma=2, m=4, "
                       "Toeplitz 256^3, standard CG to 1e-4",
           "M": M, "plan_s": t_plan, "eh_y_ms": t_eh * 1e3, "toeplitz_build_and_first_solve_ms": t_first * 1e3,
           "iterations": it, "res_last": best["res_last"], "solve_ms": best["seconds"] * 1e3,
           "ms_per_iteration": (best["seconds"] - t_eh) * 1e3 / max(it, 1), "kernels": kern}
    out["downsample_64"] = kooshball64_check()
    return out


def kooshball64_check():
    """The 64^3 downsample of the kooshball workload against the FP64 oracle's
    CG solution committed in tests/golden/kooshball64.npz (the data y is
    recomputed with the oracle's FP64 forward operator): the same iteration
    count, standard CG with the Toeplitz-embedded E^H W E on 128^3 FFTs."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import capi, synth
    from oracle import oracle as O
    path = os.path.join(ROOT, "tests", "golden", "kooshball64.npz")
    if not os.path.exists(path):
        return None
    g = np.load(path)
    c = synth.kooshball3d_64_downsample()
    it = int(g["iterations"])
    s = O.Sense(c["sens"], c["k"], w=c["w"], m=c["m"], alpha=c["alpha"])
    y = np.ascontiguousarray(s.trafo(c["image"]), dtype=np.complex64)
    p = capi.Plan(c["shape"], c["k"].shape[0], ncoils=c["sens"].shape[0], m=c["m"], alpha=c["alpha"])
    p.set_kspace(c["k"])
    p.set_weights(c["w"])
    p.set_sensitivities(np.ascontiguousarray(c["sens"]))
    yd = torch.from_numpy(y).cuda()
    xd = torch.zeros(c["shape"], dtype=torch.complex64, device="cuda")
    kw = dict(mode=cg.MODE_STANDARD, cgiter=it, cgeps=0.0, lam=0.0, weighted=True, toeplitz=True)
    p.solve(yd, xd, **kw)
    rep = p.solve(yd, xd, **kw)
    p.close()
    return {"workload": "64^3 downsample: 16 coils, kooshball 5000 x 128, Toeplitz 128^3", "iterations": it,
            "solve_ms": rep["seconds"] * 1e3, "rel_l2_vs_oracle": rel_l2(xd.cpu().numpy(), g["x"])}


def learned_section():
    """Learned-preconditioned flexible CG against plain GPU CG (and Jacobi and
    circulant-preconditioned CG) to relative residual 1e-4 on eight held-out
    256^2, 16-coil golden-angle problems spread over 32-100 spokes, with each
    image's error against the converged plain solve.  The learned arm is the
    circulant step plus the network's local correction.  Uses the committed
    trained weights; null when they are absent."""
    from codeare_gb300 import learned
    net = learned.load_net()
    if net is None:
        return None
    rows, summary = learned.compare_many(net)
    net.close()
    return {"workload": ("learned preconditioner: 256^2, 16 coils, golden-angle radial 32..100 spokes x 512, "
                         "random-ellipse phantoms, Toeplitz E^H W E, lambda = 1e-3 mean diagonal, to "
                         "||r||/||r0|| = 1e-4; eight held-out problems"),
            "problems": rows, "summary": summary,
            "speedup_vs_plain": summary["learned"]["median_speedup_vs_plain"],
            "circulant_speedup_vs_plain": summary["circulant"]["median_speedup_vs_plain"]}


def run_ours(args):
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import capi

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_over_ranks(x):
        if ws == 1:
            return x
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    k, fh = workload_data()
    M = k.shape[0]
    n = int(N * SIGMA)
    bytes_model = algorithmic_bytes(N, n, M, 2, NC)
    plan = cg.Plan((N, N), M, ncoils=NC, m=M_KB, alpha=SIGMA)
    plan.set_kspace(k)
    # the library's autotuner picks the gridding bins and coil blocks (untimed set-up)
    tuning = plan.autotune()[0] if not args.no_autotune else plan.tuning()
    # a dedicated stream: torch's default stream has handle 0, which the C ABI
    # reads as "the plan's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    fh_d = torch.from_numpy(fh).cuda()
    f_d = torch.empty((NC, M), dtype=torch.complex64, device="cuda")
    img_d = torch.empty((NC, N, N), dtype=torch.complex64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 126 MB L2

    def step():
        plan.nfft_trafo(fh_d, f_d, stream=stream)
        plan.nfft_adjoint(f_d, img_d, stream=stream)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # ---- timed region: K steps, L2 flushed before each, CUDA events on the launching stream
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    l0 = cg.kernel_launches()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = cg.kernel_launches() - l0
    clk = clocks.stop()
    t_step = sum(a.elapsed_time(b) for a, b in ev) / args.steps * 1e-3
    t_step = max_over_ranks(t_step)
    value = ws * bytes_model["step"] / t_step / 1e9

    # ---- per-kernel CUDA-event profile over the same steps
    capi.profile_enable(True)
    for i in range(args.steps):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    prof = capi.profile_collect()
    capi.profile_enable(False)
    per_kernel = {}
    kb = {"interp": bytes_model["interp"], "spread": bytes_model["spread"],
          # FFT passes: 2 launches per transform; model bytes per transform include pad/crop
          "fft": (bytes_model["pad_deapod"] + bytes_model["fft"] + bytes_model["fft"] +
                  bytes_model["crop_deapod"]) / 4.0}
    for cat, (ms, cnt) in prof.items():
        if cnt:
            avg = ms / cnt * 1e-3
            per_kernel[cat] = {"launches": cnt, "avg_ms": avg * 1e3, "alg_bytes_per_launch": kb[cat],
                               "GBps": kb[cat] / avg / 1e9}
    dom = max(per_kernel, key=lambda c: prof[c][0]) if per_kernel else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    traffic = None
    try:
        tj = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = tj.get(dom)
    except Exception:
        pass
    for v in per_kernel.values():  # each kernel against the same HBM denominator
        v["frac_of_hbm"] = v["GBps"] / hbm
    if "fft" in per_kernel:  # the same passes on the bytes a pruned transform must move
        f = per_kernel["fft"]
        f["pruned_bytes_per_launch"] = pruned_fft_bytes(N, n, NC) / 4.0
        f["GBps_pruned"] = f["pruned_bytes_per_launch"] / (f["avg_ms"] * 1e-3) / 1e9
        f["frac_of_hbm_pruned"] = f["GBps_pruned"] / hbm
    roofline = None
    if dom:
        a = per_kernel[dom]["GBps"]
        roofline = {"bound": "hbm", "kernel": dom, "achieved": a, "peak": hbm, "peak_source": peak_src,
                    "unit": "GB/s", "frac": a / hbm, "traffic": traffic,
                    "alg_bytes_per_launch": per_kernel[dom]["alg_bytes_per_launch"]}

    # ---- e2e through the C ABI with pinned host buffers
    fh_h = torch.from_numpy(fh).pin_memory().numpy()
    f_h = torch.empty((NC, M), dtype=torch.complex64).pin_memory().numpy()
    img_h = torch.empty((NC, N, N), dtype=torch.complex64).pin_memory().numpy()

    def step_host():
        plan.nfft_trafo(fh_h, f_h)
        plan.nfft_adjoint(f_h, img_h)

    for _ in range(2):
        step_host()
    tt = 0.0
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_host()
        tt += time.perf_counter() - t0
    t_e2e = max_over_ranks(tt / args.steps)
    h2d = fh_h.nbytes + f_h.nbytes
    d2h = f_h.nbytes + img_h.nbytes
    e2e = {"value": ws * bytes_model["step"] / t_e2e / 1e9, "unit": UNIT, "ms_per_step": t_e2e * 1e3,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    # ---- CPU baseline (rank 0, N = 1): bounded sample, one coil per host thread
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline_leg(k, fh)

    plan.close()
    cgs_part = None
    learned_part = None
    batch_part = None
    kooshball_part = None
    cs_part = None
    if rank == 0 and not args.no_cgsense:
        cgs_part = cgsense_section(cpu_too=(ws == 1 and not args.no_cpu))
        cs_part = cs_section(cpu_too=(ws == 1 and not args.no_cpu))
        learned_part = learned_section()
        batch_part = batch_section()
        kooshball_part = kooshball_section()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "N": N, "n": n, "M": M, "ncoils": NC, "m": M_KB,
                       "alg_bytes_per_step": bytes_model["step"], "tuning": tuning,
                       "l2": "flushed before every timed step (512 MiB write, untimed)",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "roofline": roofline, "kernels": per_kernel, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk, "gpu_launches": launches, "cgsense": cgs_part, "learned_fcg": learned_part,
            "batch": batch_part, "kooshball3d": kooshball_part, "compressed_sensing": cs_part,
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """Forward + adjoint steps of one workload and nothing else, for profiler
    captures (prints one summary line, no JSON contract):
      nufft256    -- the 256^2, 32-coil NuFFT of the headline (default tuning);
      kooshball64 -- the 64^3 downsample of the kooshball, 16 coils, E and E^H W;
      cnn256      -- the learned preconditioner's network on one 256^2 image;
      cg256       -- 10 iterations each of plain, circulant-preconditioned and
                     learned flexible CG on one 256^2, 16-coil, 32-spoke problem
                     (Toeplitz normal operator), then the normal operator and
                     the circulant step as ordinary launches."""
    import torch
    import codeare_gb300 as cg
    from codeare_gb300 import capi, synth
    torch.cuda.set_device(0)
    if args.profile_case == "cg256":
        from codeare_gb300 import learned
        net = learned.load_net()
        pr = learned.Problem(9001, spokes=32)
        x = torch.zeros((pr.N, pr.N), dtype=torch.complex64, device="cuda")
        q = torch.empty_like(x)
        for _ in range(args.warmup + args.steps):
            for kw in ({}, {"circulant": True}, {"net": net, "circulant": True}):
                x.zero_()
                pr.solve(x, cgiter=10, cgeps=1e-12, **kw)
            # the loops run inside CUDA graphs; the normal operator and the
            # circulant step once more as ordinary launches, so a launch list
            # shows their kernels
            pr.apply(pr.b, q)
            pr.precond(pr.b, q)
        torch.cuda.synchronize()
        pr.close()
        if net is not None:
            net.close()
        print("profile case cg256: %d steps" % (args.warmup + args.steps))
        return 0
    if args.profile_case == "cnn256":
        from codeare_gb300 import learned
        net = learned.load_net() or capi.Net(max_batch=1, max_h=256, max_w=256)
        x = torch.randn((1, 256, 256, 2), device="cuda")
        y = torch.empty_like(x)
        for _ in range(args.warmup + args.steps):
            net.forward(x, y)
        torch.cuda.synchronize()
        net.close()
        print("profile case cnn256: %d steps" % (args.warmup + args.steps))
        return 0
    if args.profile_case == "nufft256":
        k, fh = workload_data()
        p = cg.Plan((N, N), k.shape[0], ncoils=NC, m=M_KB, alpha=SIGMA)
        p.set_kspace(k)
        a = torch.from_numpy(fh).cuda()
        b = torch.empty((NC, k.shape[0]), dtype=torch.complex64, device="cuda")

        def step():
            p.nfft_trafo(a, b)
            p.nfft_adjoint(b, a)
    else:
        c = synth.kooshball3d_64_downsample()
        k = c["k"]
        p = capi.Plan(c["shape"], k.shape[0], ncoils=c["sens"].shape[0], m=c["m"], alpha=c["alpha"])
        p.set_kspace(k)
        p.set_weights(c["w"])
        p.set_sensitivities(np.ascontiguousarray(c["sens"]))
        a = torch.from_numpy(np.ascontiguousarray(c["image"])).cuda()
        b = torch.empty((c["sens"].shape[0], k.shape[0]), dtype=torch.complex64, device="cuda")

        def step():
            p.sense_trafo(a, b)
            p.sense_adjoint(b, a, weighted=True)
    for _ in range(args.warmup + args.steps):
        step()
    torch.cuda.synchronize()
    p.close()
    print("profile case %s: %d steps" % (args.profile_case, args.warmup + args.steps))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default gridding decomposition (profiling runs: no candidate launches)")
    ap.add_argument("--no-cgsense", action="store_true", help="skip the CG-SENSE, batch, kooshball, learned-preconditioner and CS sections")
    ap.add_argument("--profile-case", choices=["nufft256", "kooshball64", "cnn256", "cg256"],
                    help="run only this workload's forward+adjoint steps (profiler captures; no JSON line)")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
