"""ctypes binding of libcgs.so (include/cgs.h).

The product path is the CUDA library; there is no CPU fallback.  Loading fails
loudly when libcgs.so is missing or was built for another machine.

Arrays may be numpy (host) or torch CUDA tensors (device); both are passed as
raw pointers and the library stages host data itself.  Layouts are the C-order
views of codeare's column-major matrices (see codeare_gb300/synth.py).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcgs.so")

CGS_OK, CGS_ERR_BAD_ARG, CGS_ERR_OOM, CGS_ERR_CUDA, CGS_ERR_TIMEOUT, CGS_ERR_NAN, CGS_ERR_STATE = range(7)
MODE_CODEARE, MODE_STANDARD = 0, 1

EXPORTED = [
    "cgs_plan_create", "cgs_plan_destroy", "cgs_set_kspace", "cgs_set_weights",
    "cgs_set_sensitivities", "cgs_nfft_trafo", "cgs_nfft_adjoint", "cgs_nfft_itrafo",
    "cgs_sense_trafo", "cgs_sense_adjoint_codeare", "cgs_sense_adjoint", "cgs_solve",
    "cgs_plan_info", "cgs_sync", "cgs_kernel_launches", "cgs_last_error",
    "cgs_profile_enable", "cgs_profile_collect", "cgs_nfft2d_trafo_noalloc",
    "cgs_net_num_params", "cgs_net_create", "cgs_net_destroy", "cgs_net_set_weights", "cgs_net_get_weights",
    "cgs_net_forward", "cgs_net_gradients", "cgs_net_train_step", "cgs_solve_fcg", "cgs_normal_apply", "cgs_precond_apply", "cgs_set_frame_sensitivities", "cgs_net_set_conv_kernel",
    "cgs_get_tuning", "cgs_set_tuning", "cgs_autotune", "cgs_autotune_cache", "cgs_batch_create", "cgs_batch_solve",
    "cgs_batch_destroy", "cgs_cs_create", "cgs_cs_destroy", "cgs_cs_adjoint", "cgs_cs_df", "cgs_cs_obj",
    "cgs_cs_wavelet", "cgs_diag_wait_timeout",
]
PROFILE_CATEGORIES = ("fft", "interp", "spread")


class PlanDesc(C.Structure):
    _fields_ = [("rank", C.c_int), ("N", C.c_int * 3), ("alpha", C.c_double), ("m", C.c_int),
                ("M", C.c_int64), ("ncoils", C.c_int), ("frames", C.c_int)]


class SolveOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("cgiter", C.c_int), ("cgeps", C.c_double),
                ("lam", C.c_double), ("ftiter", C.c_int), ("fteps", C.c_double),
                ("weighted", C.c_int), ("toeplitz", C.c_int), ("jacobi", C.c_int)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("res_first", C.c_double), ("res_last", C.c_double),
                ("seconds", C.c_double), ("res_hist", C.c_double * 256), ("fallback_at", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("tile", C.c_int), ("work_slice", C.c_int), ("spread_chunk", C.c_int),
                ("interp_coils", C.c_int), ("spread_coils", C.c_int), ("spread_block", C.c_int),
                ("interp_block", C.c_int), ("host_chunks", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CsOpts(C.Structure):
    _fields_ = [("cgiter", C.c_int), ("cgeps", C.c_double), ("lambda_", C.c_double), ("ftiter", C.c_int),
                ("fteps", C.c_double), ("nlopt", C.c_int), ("csiter", C.c_int), ("nliter", C.c_int),
                ("lsiter", C.c_int), ("lsa", C.c_float), ("lsb", C.c_float), ("cgconv", C.c_float),
                ("parallel_linesearch", C.c_int), ("tvw", C.c_float * 2), ("tvdims", (C.c_int * 3) * 2),
                ("ntvdims", C.c_int * 2), ("xfmw", C.c_float), ("l1", C.c_float), ("pnorm", C.c_float),
                ("wl_family", C.c_int), ("wl_member", C.c_int), ("ft", C.c_int)]


class CsReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("ls_index", C.c_int * 256), ("rmse", C.c_double * 256),
                ("solves", C.c_int), ("solve_iterations", C.c_int), ("tvw_used", C.c_float * 2),
                ("seconds", C.c_double)]


class CgsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("cgs status %d: %s" % (status, msg))
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load libcgs.so (raises if absent: the CUDA library is the only path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libcgs.so not built (run __graft_entry__.build()): %s" % path)
    L = C.CDLL(path)
    vp = C.c_void_p
    L.cgs_plan_create.argtypes = [C.POINTER(vp), C.POINTER(PlanDesc)]
    L.cgs_plan_destroy.argtypes = [vp]
    L.cgs_set_kspace.argtypes = [vp, vp]
    L.cgs_set_weights.argtypes = [vp, vp]
    L.cgs_set_sensitivities.argtypes = [vp, vp]
    L.cgs_nfft_trafo.argtypes = [vp, vp, vp, vp]
    L.cgs_nfft_adjoint.argtypes = [vp, vp, vp, vp]
    L.cgs_nfft_itrafo.argtypes = [vp, vp, vp, C.c_int, C.c_double, vp]
    L.cgs_sense_trafo.argtypes = [vp, vp, vp, vp]
    L.cgs_sense_adjoint_codeare.argtypes = [vp, vp, vp, C.c_int, C.c_double, vp]
    L.cgs_sense_adjoint.argtypes = [vp, vp, vp, C.c_int, vp]
    L.cgs_solve.argtypes = [vp, vp, vp, C.POINTER(SolveOpts), C.POINTER(SolveReport), vp]
    L.cgs_plan_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int64), C.POINTER(C.c_int)]
    L.cgs_sync.argtypes = [vp]
    L.cgs_kernel_launches.restype = C.c_int64
    L.cgs_last_error.restype = C.c_char_p
    L.cgs_profile_enable.argtypes = [C.c_int]
    L.cgs_profile_enable.restype = None
    L.cgs_profile_collect.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.cgs_profile_collect.restype = None
    L.cgs_nfft2d_trafo_noalloc.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int64, vp, vp, vp, vp]
    L.cgs_solve_fcg.argtypes = [vp, vp, vp, vp, C.POINTER(SolveOpts), vp, C.POINTER(SolveReport), vp]
    L.cgs_normal_apply.argtypes = [vp, vp, vp, C.POINTER(SolveOpts), vp]
    L.cgs_precond_apply.argtypes = [vp, vp, vp, C.POINTER(SolveOpts), vp]
    L.cgs_set_frame_sensitivities.argtypes = [vp, C.c_int, vp]
    L.cgs_net_set_conv_kernel.argtypes = [vp, C.c_int]
    L.cgs_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.cgs_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.cgs_autotune.argtypes = [vp, C.POINTER(Tuning), C.POINTER(C.c_double), vp]
    L.cgs_autotune_cache.argtypes = [C.c_int]
    L.cgs_diag_wait_timeout.argtypes = [C.c_int64, vp]
    L.cgs_batch_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.POINTER(SolveOpts), C.c_int, vp]
    L.cgs_batch_solve.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(SolveReport),
                                  C.POINTER(C.c_double)]
    L.cgs_batch_destroy.argtypes = [vp]
    L.cgs_net_num_params.restype = C.c_int64
    L.cgs_net_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int]
    L.cgs_net_destroy.argtypes = [vp]
    L.cgs_net_set_weights.argtypes = [vp, vp]
    L.cgs_net_get_weights.argtypes = [vp, vp]
    L.cgs_net_forward.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp]
    L.cgs_net_gradients.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
    L.cgs_net_train_step.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, vp, vp]
    L.cgs_cs_create.argtypes = [C.POINTER(vp), vp, C.POINTER(CsOpts)]
    L.cgs_cs_destroy.argtypes = [vp]
    L.cgs_cs_adjoint.argtypes = [vp, vp, vp, C.POINTER(CsReport), vp]
    L.cgs_cs_df.argtypes = [vp, vp, vp, vp, vp]
    L.cgs_cs_obj.argtypes = [vp, vp, vp, vp, C.c_float, C.POINTER(C.c_double), C.POINTER(C.c_double), vp]
    L.cgs_cs_wavelet.argtypes = [vp, vp, vp, C.c_int, vp]
    for name in EXPORTED:
        if name not in ("cgs_kernel_launches", "cgs_last_error", "cgs_profile_enable",
                        "cgs_profile_collect", "cgs_net_num_params"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(status):
    if status != CGS_OK:
        raise CgsError(status, load().cgs_last_error().decode())


def _ptr(a):
    """raw pointer of a numpy array or torch tensor (no copy)"""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return C.c_void_p(a.data_ptr())
    raise TypeError("expected numpy array or torch tensor")


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return C.c_void_p(s.cuda_stream)
    return C.c_void_p(int(s))


def _resolve_stream(stream):
    """Stream for a plan call and whether to wait for the plan's own stream
    afterwards.  An explicit stream is used as given.  Otherwise torch's current
    stream is used when it is a real stream, so device tensors are ordered with
    torch's own work; on the legacy default stream (handle 0) the library runs
    on the plan's stream and the call waits for it, so a device result is ready
    for torch when the call returns."""
    if stream is not None:
        return _stream(stream), False
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            h = torch.cuda.current_stream().cuda_stream
            if h:
                return C.c_void_p(h), False
    except ImportError:
        pass
    return None, True


def kernel_launches() -> int:
    return int(load().cgs_kernel_launches())


def autotune_cache(mode: int):
    """cgs_autotune_cache: 0 off (cleared), 1 on (cleared; the default), 2 clear"""
    _check(load().cgs_autotune_cache(int(mode)))


def profile_enable(on: bool = True):
    load().cgs_profile_enable(int(bool(on)))


def profile_collect():
    """{category: (total ms, launches)} accumulated since the last collect"""
    ms = (C.c_double * 3)()
    cnt = (C.c_int64 * 3)()
    load().cgs_profile_collect(ms, cnt)
    return {PROFILE_CATEGORIES[i]: (ms[i], cnt[i]) for i in range(3)}


def _report(rep):
    n = rep.iterations
    hist = [rep.res_hist[i] for i in range(min(256, n + 1))]
    return dict(iterations=n, res_first=rep.res_first, res_last=rep.res_last, seconds=rep.seconds,
                res_hist=hist, fallback_at=rep.fallback_at)


class Plan:
    """One NFFT / NCSENSE operator on the current CUDA device.  With frames > 1
    it is NCSENSE's dim4 batch: `shape` and `M` are per frame, k-space is
    (F, M, d), signals (F, NC, M) and images (F, *shape) (C order)."""

    def _go(self, fn, *args, stream=None):
        st, wait = _resolve_stream(stream)
        _check(fn(self._h, *args, st))
        if wait:
            _check(load().cgs_sync(self._h))

    def __init__(self, shape, M, ncoils=1, m=1, alpha=1.0, frames=1):
        L = load()
        self.shape = tuple(int(s) for s in shape)
        self.d = len(self.shape)
        self.M = int(M)
        self.nc = int(ncoils)
        self.frames = int(frames)
        desc = PlanDesc(self.d, (C.c_int * 3)(*self.shape, *([1] * (3 - self.d))), float(alpha), int(m),
                        self.M, self.nc, self.frames)
        h = C.c_void_p()
        _check(L.cgs_plan_create(C.byref(h), C.byref(desc)))
        self._h = h
        N = (C.c_int * 3)(); n = (C.c_int * 3)(); r = C.c_int(); Mo = C.c_int64(); nc = C.c_int()
        _check(L.cgs_plan_info(h, C.byref(r), N, n, C.byref(Mo), C.byref(nc)))
        self.n = tuple(n[i] for i in range(self.d))

    def close(self):
        if getattr(self, "_h", None):
            load().cgs_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup -------------------------------------------------------------
    def set_kspace(self, k):
        _check(load().cgs_set_kspace(self._h, _ptr(k)))

    def set_weights(self, w):
        _check(load().cgs_set_weights(self._h, _ptr(w)))

    def set_frame_sensitivities(self, frame, s):
        """the sensitivities (NC, N..) of one frame of a framed plan"""
        _check(load().cgs_set_frame_sensitivities(self._h, int(frame), _ptr(s)))

    def set_sensitivities(self, s):
        _check(load().cgs_set_sensitivities(self._h, _ptr(s)))

    def sync(self):
        _check(load().cgs_sync(self._h))

    # -- operators (out must be preallocated, same memory kind as in) -------
    def nfft_trafo(self, fhat, out, stream=None):
        self._go(load().cgs_nfft_trafo, _ptr(fhat), _ptr(out), stream=stream)
        return out

    def nfft_adjoint(self, f, out, stream=None):
        self._go(load().cgs_nfft_adjoint, _ptr(f), _ptr(out), stream=stream)
        return out

    def nfft_itrafo(self, f, out, maxit=3, eps=1e-3, stream=None):
        self._go(load().cgs_nfft_itrafo, _ptr(f), _ptr(out), int(maxit), float(eps), stream=stream)
        return out

    def sense_trafo(self, x, out, stream=None):
        self._go(load().cgs_sense_trafo, _ptr(x), _ptr(out), stream=stream)
        return out

    def sense_adjoint_codeare(self, y, out, ftiter=3, fteps=1e-3, stream=None):
        self._go(load().cgs_sense_adjoint_codeare, _ptr(y), _ptr(out), int(ftiter), float(fteps), stream=stream)
        return out

    def sense_adjoint(self, y, out, weighted=True, stream=None):
        self._go(load().cgs_sense_adjoint, _ptr(y), _ptr(out), int(bool(weighted)), stream=stream)
        return out

    def solve(self, y, out, mode=MODE_CODEARE, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3,
              weighted=True, toeplitz=False, stream=None):
        o = SolveOpts(int(mode), int(cgiter), float(cgeps), float(lam), int(ftiter), float(fteps),
                      int(bool(weighted)), int(bool(toeplitz)))
        rep = SolveReport()
        self._go(load().cgs_solve, _ptr(y), _ptr(out), C.byref(o), C.byref(rep), stream=stream)
        return _report(rep)

    def tuning(self):
        t = Tuning()
        _check(load().cgs_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        t = Tuning()
        _check(load().cgs_get_tuning(self._h, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        _check(load().cgs_set_tuning(self._h, C.byref(t)))

    def autotune(self, stream=None):
        """times candidate gridding decompositions, applies the fastest; returns
        (tuning dict, interpolation + spreading milliseconds)"""
        t = Tuning()
        ms = C.c_double()
        _check(load().cgs_autotune(self._h, C.byref(t), C.byref(ms), _stream(stream)))
        return t.as_dict(), ms.value

    def solve_fcg(self, out, y=None, rhs=None, net=None, cgiter=200, cgeps=1e-4, lam=0.0, weighted=True,
                  toeplitz=True, jacobi=False, circulant=False, stream=None):
        """flexible CG with the learned preconditioner `net`; without one, plain CG,
        (jacobi=True) CG preconditioned by the exact diagonal of the normal
        operator or (circulant=True) by the circulant of precond_apply.  With a
        net, circulant=True makes the net correct the circulant step."""
        kind = 2 if circulant else (1 if jacobi else 0)
        o = SolveOpts(MODE_STANDARD, int(cgiter), float(cgeps), float(lam), 0, 0.0, int(bool(weighted)),
                      int(bool(toeplitz)), kind)
        rep = SolveReport()
        self._go(load().cgs_solve_fcg, None if y is None else _ptr(y), None if rhs is None else _ptr(rhs),
                 _ptr(out), C.byref(o), None if net is None else net._h, C.byref(rep), stream=stream)
        return _report(rep)

    def precond_apply(self, r, out, lam=0.0, weighted=True, stream=None):
        """out = C r, the circulant preconditioner of the normal equations"""
        o = SolveOpts(MODE_STANDARD, 0, 0.0, float(lam), 0, 0.0, int(bool(weighted)), 1, 2)
        self._go(load().cgs_precond_apply, _ptr(r), _ptr(out), C.byref(o), stream=stream)

    def normal_apply(self, x, out, lam=0.0, weighted=True, toeplitz=True, stream=None):
        o = SolveOpts(MODE_STANDARD, 0, 0.0, float(lam), 0, 0.0, int(bool(weighted)), int(bool(toeplitz)))
        self._go(load().cgs_normal_apply, _ptr(x), _ptr(out), C.byref(o), stream=stream)
        return out


class CS:
    """Compressed sensing over a plan's NCSENSE operator (codeare's CS_XSENSE
    with ft = 3, minimised by NLCG), or with ft = 2 over a single-coil plan's
    NFFT (its inverse by CGNR with ftiter steps and threshold fteps).  The plan needs k-space, weights and
    sensitivities and must not be used elsewhere while a CS call runs.
    tvdims: per TV term the list of TV'ed axes in codeare order (None: all)."""

    def __init__(self, plan, tvw=(0.0, 0.0), tvdims=(None, None), xfmw=0.0, l1=0.0, pnorm=0.0, nlopt=0,
                 csiter=1, nliter=4, lsiter=8, lsa=0.01, lsb=0.6, cgconv=1e-4, parallel_linesearch=False,
                 cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3, wl_family=-1, wl_member=0, ft=3):
        o = CsOpts()
        o.cgiter, o.cgeps, o.lambda_, o.ftiter, o.fteps = int(cgiter), float(cgeps), float(lam), int(ftiter), float(fteps)
        o.nlopt, o.csiter, o.nliter, o.lsiter = int(nlopt), int(csiter), int(nliter), int(lsiter)
        o.lsa, o.lsb, o.cgconv = float(lsa), float(lsb), float(cgconv)
        o.parallel_linesearch = int(bool(parallel_linesearch))
        for i in range(2):
            o.tvw[i] = float(tvw[i])
            dims = list(tvdims[i] or [])[:3]
            o.ntvdims[i] = len(dims)
            for j, v in enumerate(dims):
                o.tvdims[i][j] = int(v)
        o.xfmw, o.l1, o.pnorm = float(xfmw), float(l1), float(pnorm)
        o.wl_family, o.wl_member, o.ft = int(wl_family), int(wl_member), int(ft)
        self.plan = plan
        h = C.c_void_p()
        _check(load().cgs_cs_create(C.byref(h), plan._h, C.byref(o)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().cgs_cs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _go(self, fn, *args, stream=None):
        st, wait = _resolve_stream(stream)
        _check(fn(self._h, *args, st))
        if wait:
            _check(load().cgs_sync(self.plan._h))

    def adjoint(self, y, out, stream=None):
        rep = CsReport()
        self._go(load().cgs_cs_adjoint, _ptr(y), _ptr(out), C.byref(rep), stream=stream)
        n = min(256, rep.iterations)
        return dict(iterations=rep.iterations, ls_index=[rep.ls_index[i] for i in range(n)],
                    rmse=[rep.rmse[i] for i in range(n)], solves=rep.solves,
                    solve_iterations=rep.solve_iterations, tvw_used=(rep.tvw_used[0], rep.tvw_used[1]),
                    seconds=rep.seconds)

    def wavelet(self, x, out, inverse=False, stream=None):
        """out = W x (or W^-1 x), the handle's wavelet transform"""
        self._go(load().cgs_cs_wavelet, _ptr(x), _ptr(out), int(bool(inverse)), stream=stream)
        return out

    def df(self, y, x, out, stream=None):
        self._go(load().cgs_cs_df, _ptr(y), _ptr(x), _ptr(out), stream=stream)
        return out

    def obj(self, y, x, dx, t, stream=None):
        o, r = C.c_double(), C.c_double()
        self._go(load().cgs_cs_obj, _ptr(y), _ptr(x), _ptr(dx), float(t), C.byref(o), C.byref(r), stream=stream)
        return o.value, r.value


class Net:
    """The learned preconditioner's CNN (2 -> 32 -> 32 -> 32 -> 32 -> 2, 3x3)."""

    def __init__(self, max_batch=1, max_h=256, max_w=256):
        L = load()
        h = C.c_void_p()
        _check(L.cgs_net_create(C.byref(h), int(max_batch), int(max_h), int(max_w)))
        self._h = h
        self.nparams = int(L.cgs_net_num_params())

    def close(self):
        if getattr(self, "_h", None):
            load().cgs_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def weights(self):
        w = np.zeros(self.nparams, np.float32)
        _check(load().cgs_net_get_weights(self._h, _ptr(w)))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _check(load().cgs_net_set_weights(self._h, _ptr(w)))

    def set_conv_kernel(self, kind):
        """32 -> 32 layers on tcgen05 (1, default) or mma.sync (0)"""
        _check(load().cgs_net_set_conv_kernel(self._h, int(kind)))

    def forward(self, x, out=None, stream=None):
        B, H, W, _ = x.shape
        if out is None:
            out = np.zeros_like(x) if isinstance(x, np.ndarray) else x.new_empty(x.shape)
        _check(load().cgs_net_forward(self._h, _ptr(x), _ptr(out), B, H, W, _stream(stream)))
        return out

    def gradients(self, x, t, stream=None):
        B, H, W, _ = x.shape
        g = np.zeros(self.nparams, np.float32)
        loss = np.zeros(1, np.float32)
        _check(load().cgs_net_gradients(self._h, _ptr(x), _ptr(t), B, H, W, _ptr(g), _ptr(loss),
                                        _stream(stream)))
        return float(loss[0]), g

    def train_step(self, x, t, lr=1e-3, stream=None, want_loss=True):
        B, H, W, _ = x.shape
        loss = np.zeros(1, np.float32)
        _check(load().cgs_net_train_step(self._h, _ptr(x), _ptr(t), B, H, W, float(lr),
                                         _ptr(loss) if want_loss else None, _stream(stream)))
        return float(loss[0]) if want_loss else None


def solve_opts(mode=MODE_CODEARE, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3, weighted=True,
               toeplitz=False):
    return SolveOpts(int(mode), int(cgiter), float(cgeps), float(lam), int(ftiter), float(fteps),
                     int(bool(weighted)), int(bool(toeplitz)), 0)


class Batch:
    """Solves of several plans in one CUDA graph (include/cgs.h, cgs_batch_*).
    `opts` is one solve_opts(...) per plan, or one for all."""

    def __init__(self, plans, opts, stream=None):
        L = load()
        n = len(plans)
        if isinstance(opts, SolveOpts):
            opts = [opts] * n
        self.plans = list(plans)
        self._ph = (C.c_void_p * n)(*[p._h.value for p in plans])
        self._opts = (SolveOpts * n)(*opts)
        h = C.c_void_p()
        _check(L.cgs_batch_create(C.byref(h), self._ph, self._opts, n, _stream(stream)))
        self._h = h

    def solve(self, ys, xs):
        """ys[i] -> xs[i]; returns (reports, device seconds of the graph launch)"""
        n = len(self.plans)
        yp = (C.c_void_p * n)(*[_ptr(y).value for y in ys])
        xp = (C.c_void_p * n)(*[_ptr(x).value for x in xs])
        reps = (SolveReport * n)()
        sec = C.c_double()
        _check(load().cgs_batch_solve(self._h, yp, xp, reps, C.byref(sec)))
        return [_report(r) for r in reps], sec.value

    def close(self):
        if getattr(self, "_h", None):
            load().cgs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
