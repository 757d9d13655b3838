"""The CGSENSE.so plugin driven through its ReconStrategy lifecycle by a dlopen
host (cgsense_run), as codeare's ReconContext loads modules, compared with the
FP64 oracle of the reference semantics (CGLS over the CGNR-based E^H)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_IMG = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def run_plugin(tmp_path, mats, attrs):
    from codeare_gb300 import build, cgsm
    build.build()
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), mats)
    xml.write_text("<CGSENSE " + " ".join('%s="%s"' % kv for kv in attrs.items()) + "/>\n")
    r = subprocess.run([build.DRIVER, build.PLUGIN, str(xml), str(inp), str(out), "image"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return cgsm.read(str(out))["image"], r.stdout


@pytest.mark.parametrize("alpha,m", [(2.0, 4), (1.0, 1)])
def test_plugin_matches_reference_semantics(gpu, oracle, tmp_path, alpha, m):
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=alpha, m=m)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = oracle.Sense(S, k, w=w, m=m, alpha=alpha)
    y = synth.add_noise(s.trafo(cfg["image"]), 1e-3, seed=4)
    xo, _ = s.cgls_codeare(y, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3)
    mats = {"sensitivities": S, "kspace": k, "weights": w, "signals": y.astype(np.complex64)}
    attrs = dict(nk=k.shape[0], lambda_=0.05, m=m, cgeps=1e-6, cgmaxit=10, ftmaxit=3, fteps=0.001,
                 noise=0, testcase=0, threads=1, verbose=0)
    attrs["lambda"] = attrs.pop("lambda_")
    if alpha != 1.0:
        attrs["alpha"] = alpha
    img, log = run_plugin(tmp_path, mats, attrs)
    assert img.shape == (32, 32)
    assert rel(img, xo) < TOL_IMG, log


def test_plugin_toeplitz_key(gpu, oracle, tmp_path):
    """toeplitz="1": codeare's CGLS with each step's inner CGNR run in image
    space on the Toeplitz kernel; same result as the NFFT pair (sigma 2, m 4)."""
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=2.0, m=4)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = oracle.Sense(S, k, w=w, m=4, alpha=2.0)
    y = synth.add_noise(s.trafo(cfg["image"]), 1e-3, seed=4)
    xo, _ = s.cgls_codeare(y, cgiter=10, cgeps=1e-6, lam=5e-2, ftiter=3, fteps=1e-3)
    mats = {"sensitivities": S, "kspace": k, "weights": w, "signals": y.astype(np.complex64)}
    attrs = {"nk": k.shape[0], "lambda": 0.05, "m": 4, "alpha": 2.0, "cgeps": 1e-6, "cgmaxit": 10,
             "ftmaxit": 3, "fteps": 0.001, "noise": 0, "testcase": 0, "toeplitz": 1}
    img, log = run_plugin(tmp_path, mats, attrs)
    assert rel(img, xo) < TOL_IMG, log


def test_plugin_testcase_mode(gpu, oracle, tmp_path):
    """testcase=1: the plugin encodes its own Shepp-Logan phantom (CGSENSE.cpp:171-172)."""
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=2.0, m=4)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = oracle.Sense(S, k, w=w, m=4, alpha=2.0)
    xo, _ = s.cgls_codeare(s.trafo(synth.phantom(32)), cgiter=6, cgeps=1e-7, lam=5e-2)
    mats = {"sensitivities": S, "kspace": k, "weights": w}
    attrs = {"nk": k.shape[0], "lambda": 0.05, "m": 4, "alpha": 2.0, "cgeps": 1e-7, "cgmaxit": 6,
             "ftmaxit": 3, "fteps": 0.001, "noise": 0, "testcase": 1, "threads": 1, "verbose": 1}
    img, log = run_plugin(tmp_path, mats, attrs)
    assert rel(img, xo) < TOL_IMG, log


def test_plugin_standard_mode(gpu, oracle, tmp_path):
    from codeare_gb300 import synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=2.0, m=4)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = oracle.Sense(S, k, w=w, m=4, alpha=2.0)
    y = s.trafo(cfg["image"])
    xo, _ = s.cg(y, maxit=12, tol=1e-12, lam=0.0, weighted=True)
    mats = {"sensitivities": S, "kspace": k, "weights": w, "signals": y.astype(np.complex64)}
    attrs = {"nk": k.shape[0], "lambda": 0.0, "m": 4, "alpha": 2.0, "cgeps": 1e-12, "cgmaxit": 12,
             "ftmaxit": 3, "fteps": 0.001, "noise": 0, "testcase": 0, "mode": "standard"}
    img, log = run_plugin(tmp_path, mats, attrs)
    assert rel(img, xo) < TOL_IMG, log


def test_nufft_plugin_matches_reference_semantics(gpu, oracle, tmp_path):
    """NuFFT.so: img = NFFT ->* data, the CGNR inverse NFFT with the reference's
    unforwarded defaults (3 steps, epsilon 7e-4) whatever maxit/epsilon say
    (src/modules/NuFFT.cpp:74-75 vs :99-108)."""
    from codeare_gb300 import build, cgsm, synth
    build.build()
    N = 32
    k = synth.radial2d(24, 64, golden=True)
    w = synth.ramp_weights(k)
    M = k.shape[0]
    P = oracle.NFFT((N, N), M, m=2, alpha=1.5)
    P.set_x(k)
    data = P.trafo(synth.phantom(N)).astype(np.complex64)
    ref, _, _ = P.itrafo(data, w, oracle.damp_mask((N, N)), maxit=3, eps=7e-4)
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"kspace": k, "weights": w, "data": data[None, :]})
    xml.write_text('<NuFFT dim="2" nx="%d" ny="%d" M="%d" shots="1" maxit="20" epsilon="1e-9" m="2" '
                   'alpha="1.5" dft_3rd_dim="0" test_case="0"/>\n' % (N, N, M))
    r = subprocess.run([build.DRIVER, build.PLUGIN_NUFFT, str(xml), str(inp), str(out), "img"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    img = cgsm.read(str(out))["img"]
    assert img.shape == (N, N)
    assert rel(img, ref) < TOL_IMG, r.stdout


def golden_radial_from_raster(raster, nk, nv, golden_deg=111.246117975):
    """The EstimateSensitivities trajectory: the raster spoke linearly
    interpolated to 10x its samples and cut to nk, rotated by v golden angles,
    scaled to |k| <= 1/2, +0.5 wrapped to -0.5; (M, 2) with row order
    (sample fastest, then volume), columns (kx, ky) as codeare's kspace rows."""
    n = raster.shape[0]
    xi = np.linspace(0.0, 1.0, n)
    XI = np.linspace(0.0, 1.0, 10 * n)[:nk]
    kx = np.interp(XI, xi, raster[:, 0].astype(np.float64))
    ky = np.interp(XI, xi, raster[:, 1].astype(np.float64))
    spoke = kx + 1j * ky
    k = np.concatenate([spoke * np.exp(1j * np.deg2rad(v * golden_deg)) for v in range(nv)])
    k = k / (2.0 * np.abs(k).max())
    out = np.stack([k.real, k.imag], axis=1)
    out[out >= 0.5] -= 1.0
    return out.astype(np.float32)


def test_estimate_sensitivities_matches_oracle(gpu, oracle, tmp_path):
    """EstimateSensitivities.so (src/modules/EstimateSensitivities.cpp:53-182):
    golden-angle spokes from a raster trajectory and the per-coil inverse NFFT
    (unit weights, 3 CGNR steps) of 1e6-scaled data, against the FP64 oracle's
    inverse NFFT on the same nodes."""
    from codeare_gb300 import build, cgsm, synth
    build.build()
    N, nc, nk, nv, n = 48, 4, 96, 40, 12
    raster = np.stack([np.linspace(-1.0, 1.0, n), np.zeros(n)], axis=1).astype(np.float32)
    k = golden_radial_from_raster(raster, nk, nv)
    M = k.shape[0]
    S = synth.coils2d(N, nc)
    img = synth.phantom(N)
    P = oracle.NFFT((N, N), M, m=2, alpha=2.0)
    P.set_x(k)
    y = np.stack([P.trafo(S[c] * img) for c in range(nc)]).astype(np.complex64)   # (nc, M)
    meas = np.ascontiguousarray(y.reshape(nc, nv, nk).transpose(1, 0, 2))        # codeare (nk, nc, nv)
    sync = raster.reshape(-1)                                                    # (2n) interleaved (kx, ky)
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"meas": meas, "sync": sync.astype(np.float32)})
    xml.write_text('<EstimateSensitivities ftalpha="2.0" ftm="2" nk="%d" nl="1" cart_3rd_dim="0" '
                   'image_size="%d %d" ftiter="3"/>\n' % (nk, N, N))
    r = subprocess.run([build.DRIVER, build.PLUGIN_ESTSENS, str(xml), str(inp), str(out), "sensitivities"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    sens = cgsm.read(str(out))["sensitivities"]
    assert sens.shape == (nc, N, N)
    what = oracle.damp_mask((N, N))
    w = np.ones(M, np.float32)
    ref = np.stack([P.itrafo(y[c].astype(np.complex128) * 1e6, w, what, maxit=3, eps=7e-4)[0] for c in range(nc)])
    assert rel(sens, ref) < TOL_IMG, r.stdout


def test_plugin_from_cod_files(gpu, tmp_path):
    """The same CGSENSE run fed from codeare .cod files (double-precision
    weights, converted on read) and writing a .cod image gives the image of
    the container-fed run."""
    from codeare_gb300 import build, cod, synth
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=2.0, m=4)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    from oracle import oracle as O
    y = synth.add_noise(O.Sense(S, k, w=w, m=4, alpha=2.0).trafo(cfg["image"]), 1e-3, seed=5)
    mats = {"sensitivities": S, "kspace": k, "weights": w, "signals": y.astype(np.complex64)}
    attrs = {"nk": k.shape[0], "lambda": 0.05, "m": 4, "alpha": 2.0, "cgeps": 1e-6, "cgmaxit": 8,
             "ftmaxit": 3, "fteps": 0.001, "noise": 0, "testcase": 0, "threads": 1, "verbose": 0}
    ref, _ = run_plugin(tmp_path, mats, attrs)
    files = []
    for name, a in mats.items():
        a = np.asarray(a)
        a = a.astype(np.complex64 if np.iscomplexobj(a) else (np.float64 if name == "weights" else np.float32))
        p = tmp_path / (name + ".cod")
        cod.write(str(p), a, name)
        files.append("%s=%s" % (name, p))
    out = tmp_path / "image.cod"
    r = subprocess.run([build.DRIVER, build.PLUGIN, str(tmp_path / "cfg.xml"), ",".join(files), str(out), "image"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    img, name, _ = cod.read(str(out))
    assert name == "image" and img.dtype == np.complex64 and img.shape == ref.shape
    assert np.array_equal(img, ref)


def test_compressed_sensing_plugin_matches_oracle(gpu, tmp_path):
    """CompressedSensing.so with ft = 3 through the plugin host: the keys of
    src/modules/CompressedSensing.cpp:31-136, compared with the FP64
    restatement of CS_XSENSE + NLCG."""
    from codeare_gb300 import build, cgsm, synth
    from oracle import oracle as O, cs
    cfg = synth.small_config(N=32, nc=4, nspokes=32, nsamp=64, alpha=1.0, m=1)
    k, w, S = cfg["k"], cfg["w"], cfg["sens"]
    s = O.Sense(S, k, w=w, m=1, alpha=1.0)
    y = synth.add_noise(s.trafo(cfg["image"]), 1e-3, seed=4)
    o = cs.CSXSense(s, tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-15, pnorm=1.0, csiter=2, nliter=4, lsiter=10,
                    lsa=1e-3, lsb=0.6, cgconv=1e-5, cgiter=6, cgeps=1e-7, lam=5e-2, ftiter=3, fteps=1e-3)
    xo = o.adjoint(y)
    attrs = {"ftdims": "32 32", "ft": 3, "test_case": 0, "noise": 0, "verbose": 1, "nk": k.shape[0],
             "ftmaxit": 3, "fteps": 1e-3, "cgmaxit": 6, "cgeps": 1e-7, "lambda": 5e-2, "ftalpha": 1.0,
             "cart_3rd_dim": 0, "threads": 1, "nlopt": 0, "parallel_linesearch": 0, "tvw1": 2e-3, "tvw2": 0,
             "tv1": "1 1", "xfmw": 5e-3, "l1": 1e-15, "lsa": 1e-3, "lsb": 0.6, "pnorm": 1, "wl_family": -1,
             "wl_member": 0, "csiter": 2, "cgiter": 4, "cgconv": 1e-5, "lsiter": 10}
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"sensitivities": S, "kspace": k, "weights": w, "data": y.astype(np.complex64)})
    xml.write_text("<CompressedSensing " + " ".join('%s="%s"' % kv for kv in attrs.items()) + "/>\n")
    r = subprocess.run([build.DRIVER, build.PLUGIN_CS, str(xml), str(inp), str(out), "im_dc"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    img = cgsm.read(str(out))["im_dc"]
    assert img.shape == (32, 32)
    assert rel(img, xo) < 2e-3, r.stdout
    assert "%d NLCG iterations" % len(o.log) in r.stdout


def grasp_weights(nx, nv):
    """GRASP.cpp:158-162 with codeare's float linspace (Creators.hpp:573-590)"""
    def linspace(a, b, n):
        r = np.full(n, np.float32(a), np.float32)
        gap = np.float32((np.float32(b) - np.float32(a)) / np.float32(n - 1))
        for i in range(1, n - 1):
            r[i] = np.float32(r[i - 1] + gap)
        r[n - 1] = np.float32(b)
        return r
    half = np.concatenate([linspace(1.0, 0.002, nx // 2), linspace(0.002, 1.0, nx // 2)])
    w = (half.astype(np.float64) ** 0.75).astype(np.float32)
    return np.tile(w, nv)


def test_grasp_plugin_matches_oracle(gpu, tmp_path):
    """GRASP.so: stack-of-stars data sorted into frames (GRASP.cpp:129-170),
    one CS over NCSENSE with dim4 = frames per slice inside the margins,
    against the FP64 restatement slice by slice."""
    from codeare_gb300 import build, cgsm, synth
    from oracle import oracle as O, cs
    N, nc, nz, nx, nt, nv = 32, 3, 3, 64, 4, 10
    NV = nt * nv + 2                                   # two views past the last frame are dropped
    k = synth.radial2d(NV, nx, golden=True).reshape(NV, nx, 2).astype(np.float32)
    sens = np.stack([synth.coils2d(N, nc) * (1.0 + 0.2 * z) for z in range(nz)], axis=1)  # (nc, nz, N, N)
    w = grasp_weights(nx, nv)
    ks = list(k[:nt * nv].reshape(nt, nv * nx, 2))
    rng = np.random.default_rng(3)
    meas = (rng.standard_normal((nc, nz, NV, nx)) + 1j * rng.standard_normal((nc, nz, NV, nx))).astype(np.complex64)
    kw = dict(tvw=(0.02, 0.0), tvdims=([0, 0, 1], None), xfmw=0.0, l1=1e-6, pnorm=1.0, csiter=3, nliter=6,
              lsiter=6, lsa=0.01, lsb=0.6, cgconv=0.0, parallel_linesearch=True, cgiter=0, cgeps=1e-6, lam=1e-9,
              ftiter=1, fteps=7e-4)
    expect = {}
    for z in (1, 2):                                   # margin_top = 1
        fs = O.FramesSense(sens[:, z], ks, w=w, m=1, alpha=1.0)
        x = np.stack([synth.phantom(N) * (1.0 + 0.15 * t + 0.1 * z) for t in range(nt)])
        y = synth.add_noise(fs.trafo(x), 1e-3, seed=10 + z)   # (nt, nc, nv nx)
        meas[:, z, :nt * nv, :] = y.transpose(1, 0, 2).reshape(nc, nt * nv, nx)
        expect[z] = cs.CSXSense(fs, **kw).adjoint(meas[:, z, :nt * nv, :].reshape(nc, nt, nv * nx).transpose(1, 0, 2))
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"meas": meas, "kspace": k, "sensitivities": sens.astype(np.complex64)})
    attrs = {"ta": 40.0, "frame_duration": 10, "margin_top": 1, "margin_bottom": 0, "tv": "0 0 1", "l1": 1e-6,
             "verbose": 1}
    xml.write_text("<GRASP " + " ".join('%s="%s"' % kv for kv in attrs.items()) + "/>\n")
    r = subprocess.run([build.DRIVER, build.PLUGIN_GRASP, str(xml), str(inp), str(out), "im_xd"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    im = cgsm.read(str(out))["im_xd"]                  # codeare (N, N, nz', nt)
    assert im.shape == (nt, 2, N, N)
    for i, z in enumerate((1, 2)):
        assert rel(im[:, i], expect[z]) < 2e-3, (z, r.stdout)


def test_compressed_sensing_plugin_nfft(gpu, tmp_path):
    """CompressedSensing.so with ft = 2: CS over the plain NFFT (the
    reference's nufft_cs configurations), keys of CompressedSensing.cpp:73-85."""
    from codeare_gb300 import build, cgsm, synth
    from oracle import cs
    k = synth.radial2d(24, 64, golden=True)
    w = synth.ramp_weights(k)
    op = cs.NFFTOp((32, 32), k, w=w, m=1, alpha=1.0)
    y = synth.add_noise(op.trafo(synth.phantom(32)), 1e-3, seed=6).astype(np.complex64)
    kw = dict(tvw=(2e-3, 0.0), xfmw=5e-3, l1=1e-6, pnorm=1.0, csiter=2, nliter=5, lsiter=8, lsa=1e-3, lsb=0.6,
              cgconv=1e-5, ftiter=3, fteps=7e-4, ft=2)
    xo = cs.CSXSense(op, **kw).adjoint(y)
    attrs = {"ftdims": "32 32", "ft": 2, "test_case": 0, "noise": 0, "verbose": 0, "ftnk": k.shape[0], "ftiter": 3,
             "fteps": 7e-4, "ftalpha": 1.0, "ftm": 1, "nlopt": 0, "parallel_linesearch": 0, "tvw1": 2e-3, "tvw2": 0,
             "xfmw": 5e-3, "l1": 1e-6, "lsa": 1e-3, "lsb": 0.6, "pnorm": 1, "wl_family": -1, "wl_member": 0,
             "csiter": 2, "cgiter": 5, "cgconv": 1e-5, "lsiter": 8}
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"kspace": k, "weights": w, "data": y})
    xml.write_text("<CompressedSensing " + " ".join('%s="%s"' % kv for kv in attrs.items()) + "/>\n")
    r = subprocess.run([build.DRIVER, build.PLUGIN_CS, str(xml), str(inp), str(out), "im_dc"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert rel(cgsm.read(str(out))["im_dc"], xo) < 2e-3, r.stdout


def test_plugin_cartesian_third_dimension(gpu, oracle, tmp_path):
    """CGSENSE with dft_3rd_dim (NCSENSE's 3rd_dim_cart): sensitivities
    (N, N, slices, NC), signals (nk, slices, NC), one trajectory for every
    slice; the CGLS over the whole stack against the oracle's slice stack."""
    from codeare_gb300 import synth
    N, nz, nc, m, alpha = 32, 3, 4, 4, 2.0
    k = synth.radial2d(32, 64, golden=True)
    w = synth.ramp_weights(k)
    S3 = synth.coils3d(N, nc)[:, N // 2 - 1:N // 2 - 1 + nz]          # (nc, slices, N, N)
    x3 = synth.phantom3d(N)[N // 2 - 1:N // 2 - 1 + nz]                 # (slices, N, N)
    fs = oracle.FramesSense([S3[:, z] for z in range(nz)], [k] * nz, w=w, m=m, alpha=alpha)
    y = synth.add_noise(fs.trafo(x3), 1e-3, seed=6)                      # (slices, nc, nk)
    xo, _ = fs.cgls_codeare(y, cgiter=8, cgeps=1e-9, lam=5e-2)
    mats = {"sensitivities": np.ascontiguousarray(S3, dtype=np.complex64), "kspace": k, "weights": w,
            "signals": np.ascontiguousarray(y.transpose(1, 0, 2), dtype=np.complex64)}
    attrs = {"nk": k.shape[0], "lambda": 0.05, "m": m, "alpha": alpha, "cgeps": 1e-9, "cgmaxit": 8,
             "ftmaxit": 3, "fteps": 0.001, "noise": 0, "testcase": 0, "dft_3rd_dim": 1}
    img, log = run_plugin(tmp_path, mats, attrs)
    assert img.shape == (nz, N, N)
    assert rel(img, xo) < TOL_IMG, log


def test_nfft_cartesian_third_dimension(gpu, oracle, tmp_path):
    """NuFFT with dft_3rd_dim (NFFT's 3rd_dim_cart): a stack of 2-D inverse
    NFFTs over the slices, one trajectory; each slice against the oracle's
    CGNR (the NuFFT module's 3 steps, epsilon 7e-4)."""
    from codeare_gb300 import build, cgsm, synth
    N, nz = 32, 3
    k = synth.radial2d(24, 64, golden=True)
    w = synth.ramp_weights(k)
    rng = np.random.default_rng(12)
    data = (rng.standard_normal((nz, k.shape[0])) + 1j * rng.standard_normal((nz, k.shape[0]))).astype(np.complex64)
    P = oracle.NFFT((N, N), k.shape[0], m=1, alpha=1.0)
    P.set_x(k)
    what = oracle.damp_mask((N, N))
    ref = np.stack([P.itrafo(data[z], w, what, 3, 7e-4)[0] for z in range(nz)])
    build.build()
    inp, out, xml = tmp_path / "in.cgsm", tmp_path / "out.cgsm", tmp_path / "cfg.xml"
    cgsm.write(str(inp), {"kspace": k, "weights": w, "data": data})
    xml.write_text('<NuFFT dim="3" nx="%d" ny="%d" nz="%d" M="%d" shots="1" maxit="3" epsilon="7e-4" '
                   'dft_3rd_dim="1"/>\n' % (N, N, nz, k.shape[0]))
    r = subprocess.run([build.DRIVER, build.PLUGIN_NUFFT, str(xml), str(inp), str(out), "img"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    img = cgsm.read(str(out))["img"]
    assert img.shape == (nz, N, N)
    assert rel(img, ref) < 2e-5
