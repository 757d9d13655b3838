"""CPU-only checks of the C ABI library and the host-side helpers (no GPU calls)."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(cgs_[a-z_0-9]+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_library_builds_and_exports_every_declared_symbol():
    from codeare_gb300 import build, capi
    build.build()
    L = capi.load()
    names = declared_functions()
    assert len(names) >= 16
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(capi.EXPORTED) <= set(names)


def test_plugin_exports_reconstrategy_factories():
    import ctypes
    from codeare_gb300 import build
    build.build()
    for so in (build.PLUGIN, build.PLUGIN_NUFFT, build.PLUGIN_ESTSENS, build.PLUGIN_CS, build.PLUGIN_GRASP):
        P = ctypes.CDLL(so)
        assert hasattr(P, "create") and hasattr(P, "destroy"), so
    assert os.access(build.DRIVER, os.X_OK)


def test_synthetic_configs_shapes_and_ranges():
    from codeare_gb300 import synth
    c0 = synth.radial2d_128_8coils()
    assert c0["k"].shape == (96 * 256, 2) and c0["k"].dtype == np.float32
    assert c0["sens"].shape == (8, 128, 128)
    assert np.all(c0["k"] >= -0.5) and np.all(c0["k"] < 0.5)
    c1 = synth.radial2d_256_32coils()
    assert c1["k"].shape == (403 * 512, 2)
    assert c1["sens"].shape == (32, 256, 256)
    k3 = synth.kooshball3d(100, 64)
    assert k3.shape == (6400, 3) and np.all(k3 < 0.5) and np.all(k3 >= -0.5)
    sp = synth.spiral2d(16, 4096)
    assert sp.shape == (65536, 2)


def test_phantom_values():
    from codeare_gb300 import synth
    p = synth.phantom(128)
    vals = set(np.round(np.unique(p.real), 4).tolist())
    # every pixel is a sum of tabulated intensities; background is 0, skull 1.0
    assert 0.0 in vals and 1.0 in vals
    assert abs(p[64, 64].real - 0.2) < 1e-6 or p[64, 64].real > 0
    assert np.all(p.imag == 0)
    p3 = synth.phantom3d(32)
    assert p3.shape == (32, 32, 32) and p3.max().real <= 2.0 + 1e-6


def header_struct_fields(name):
    """(field, C type, array length) of `typedef struct {...} name;` in include/cgs.h, in order"""
    txt = open(os.path.join(ROOT, "include", "cgs.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    m = re.search(r"typedef struct \{([^}]*)\}\s*" + name + r"\s*;", txt)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        t, rest = re.match(r"((?:unsigned )?[a-z_0-9]+)\s+(.*)", decl).groups()
        for var in rest.split(","):
            v = re.match(r"\s*([A-Za-z_0-9]+)((?:\[\d+\])*)", var)
            dims = [int(d) for d in re.findall(r"\[(\d+)\]", v.group(2))]
            fields.append((v.group(1), t, dims))
    return fields


def test_ctypes_structures_mirror_the_header():
    """Every ctypes structure of the Python binding lists the header's fields
    in the header's order with the same C types (a missing field would shift
    every later one across the boundary)."""
    import ctypes as C
    from codeare_gb300 import capi
    ctype = {"int": C.c_int, "double": C.c_double, "float": C.c_float, "int64_t": C.c_int64}
    pairs = [(capi.PlanDesc, "cgs_plan_desc"), (capi.SolveOpts, "cgs_solve_opts"),
             (capi.SolveReport, "cgs_solve_report"), (capi.Tuning, "cgs_tuning"),
             (capi.CsOpts, "cgs_cs_opts"), (capi.CsReport, "cgs_cs_report")]
    for cls, name in pairs:
        hdr = header_struct_fields(name)
        py = cls._fields_
        assert len(py) == len(hdr), (name, [f for f, _ in py], [f for f, _, _ in hdr])
        for (pf, pt), (hf, ht, dims) in zip(py, hdr):
            # `lambda` is a Python keyword: the binding spells it lam or lambda_
            assert {"lam": "lambda"}.get(pf, pf.rstrip("_")) == hf, (name, pf, hf)
            want = ctype[ht]
            for d in reversed(dims):
                want = want * d
            assert C.sizeof(pt) == C.sizeof(want), (name, hf)
            base = pt
            while hasattr(base, "_type_") and hasattr(base, "_length_"):
                base = base._type_
            assert base == ctype[ht], (name, hf, base, ht)
