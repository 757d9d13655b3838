"""Build libcgs.so (sm_103a) in-tree with nvcc.

Each .cu translation unit compiles in parallel, then one shared link.  Output:
codeare_gb300/lib/libcgs.so.  The build never reads anything outside this
repository.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libcgs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]

SOURCES = ["cgs_fft.cu", "cgs_grid.cu", "cgs_vec.cu", "cgs_plan.cu", "cgs_static.cu", "cgs_cnn.cu", "cgs_cs.cu"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    t = 0.0
    for f in os.listdir(CSRC):
        t = max(t, os.path.getmtime(os.path.join(CSRC, f)))
    t = max(t, os.path.getmtime(os.path.join(ROOT, "include", "cgs.h")))
    return t


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime() and not extra:
        build_host()
        return LIB
    extra = list(extra or [])
    cc = nvcc()

    def one(src):
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_host(force=True)
    return LIB


HOST = os.path.join(HERE, "host")
PLUGIN = os.path.join(LIBDIR, "CGSENSE.so")
PLUGIN_NUFFT = os.path.join(LIBDIR, "NuFFT.so")
PLUGIN_ESTSENS = os.path.join(LIBDIR, "EstimateSensitivities.so")
PLUGIN_CS = os.path.join(LIBDIR, "CompressedSensing.so")
PLUGIN_GRASP = os.path.join(LIBDIR, "GRASP.so")
DRIVER = os.path.join(LIBDIR, "cgsense_run")


def build_host(force: bool = False) -> str:
    """The C++ drop-in layer: CGSENSE.so, NuFFT.so, EstimateSensitivities.so,
    CompressedSensing.so and GRASP.so (ReconStrategy plugins over libcgs.so)
    and cgsense_run (a dlopen host that drives a plugin)."""
    srcs = [os.path.join(HOST, f) for f in ("CGSENSE.cpp", "cgsense_run.cpp", "NuFFT.cpp",
                                            "EstimateSensitivities.cpp", "CompressedSensing.cpp", "GRASP.cpp")]
    hdrs = [os.path.join(HOST, "codeare", f) for f in os.listdir(os.path.join(HOST, "codeare"))]
    newest = max(os.path.getmtime(f) for f in srcs + hdrs + [LIB])
    outs = (PLUGIN, DRIVER, PLUGIN_NUFFT, PLUGIN_ESTSENS, PLUGIN_CS, PLUGIN_GRASP)
    if not force and all(os.path.exists(o) for o in outs) and min(os.path.getmtime(o) for o in outs) >= newest:
        return PLUGIN
    common = ["g++", "-O2", "-std=c++17", "-Wall", "-I" + HOST, "-I" + os.path.join(ROOT, "include")]
    cmds = [
        common + ["-fPIC", "-shared", srcs[0], "-o", PLUGIN + ".tmp", "-L" + LIBDIR, "-lcgs",
                  "-Wl,-rpath,$ORIGIN"],
        common + [srcs[1], "-o", DRIVER + ".tmp", "-ldl", "-rdynamic"],
        common + ["-fPIC", "-shared", srcs[2], "-o", PLUGIN_NUFFT + ".tmp", "-L" + LIBDIR, "-lcgs",
                  "-Wl,-rpath,$ORIGIN"],
        common + ["-fPIC", "-shared", srcs[3], "-o", PLUGIN_ESTSENS + ".tmp", "-L" + LIBDIR, "-lcgs",
                  "-Wl,-rpath,$ORIGIN"],
        common + ["-fPIC", "-shared", srcs[4], "-o", PLUGIN_CS + ".tmp", "-L" + LIBDIR, "-lcgs",
                  "-Wl,-rpath,$ORIGIN"],
        common + ["-fPIC", "-shared", srcs[5], "-o", PLUGIN_GRASP + ".tmp", "-L" + LIBDIR, "-lcgs",
                  "-Wl,-rpath,$ORIGIN"],
    ]
    for cmd in cmds:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    for o in outs:
        os.replace(o + ".tmp", o)
    return PLUGIN


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
