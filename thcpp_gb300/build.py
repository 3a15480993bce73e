"""In-tree build of libthc_gb300.so (nvcc, sm_103a) and of the C++ host tools.

Each CUDA translation unit compiles in parallel into ``thcpp_gb300/_build``; the shared
library lands in ``thcpp_gb300/lib``.  Rebuilds happen only when a source or header is
newer than its object.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libthc_gb300.so")

CUDA_SOURCES = ["capi.cu", "kmeans.cu", "dense64.cu", "isdf.cu", "mixed.cu", "ozgemm.cu",
                "ozgemm_tc.cu", "noalloc.cu", "synthgen.cu", "qrcp.cu", "halfc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST = os.path.join(PKG, "host")
HOST_SOURCES = ["h5lite.cpp", "h5lite_capi.cpp", "gpu_context.cpp", "kmeans.cpp", "qrcp.cpp", "interpolating_points.cpp",
                "interpolating_vectors.cpp"]
HOST_LIB = os.path.join(LIBDIR, "libthcpp_host.so")
BINDIR = os.path.join(PKG, "bin")
DRIVER = os.path.join(BINDIR, "thcpp_gb300.x")


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libthc_gb300")
    return cand


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, verbose):
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link libthc_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for name in CUDA_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs]):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_compile, s, o, verbose) for s, o in jobs]:
                f.result()
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    build_host(force=force, verbose=verbose)
    return LIB


def _have_zlib() -> bool:
    return os.path.exists("/usr/include/zlib.h")


def build_host(force: bool = False, verbose: bool = False) -> str:
    """The C++ drop-in layer (solver classes + HDF5 I/O) and the thcpp_gb300.x driver."""
    os.makedirs(BINDIR, exist_ok=True)
    srcs = [os.path.join(HOST, f) for f in HOST_SOURCES]
    hdrs = glob.glob(os.path.join(HOST, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    zlib = ["-lz"] if _have_zlib() else []
    gxx = shutil.which("g++") or "g++"
    if force or _stale(HOST_LIB, srcs + hdrs + [LIB]):
        tmp = HOST_LIB + f".tmp{os.getpid()}"
        cmd = [gxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-o", tmp, *srcs, "-L", LIBDIR,
               "-lthc_gb300", "-Wl,-rpath,$ORIGIN", *zlib]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host library build failed:\n{r.stderr}")
        os.replace(tmp, HOST_LIB)
    main = os.path.join(HOST, "main.cpp")
    if force or _stale(DRIVER, [main, HOST_LIB] + hdrs):
        tmp = DRIVER + f".tmp{os.getpid()}"
        cmd = [gxx, "-O2", "-std=c++17", "-o", tmp, main, "-L", LIBDIR, "-lthcpp_host",
               "-lthc_gb300", "-Wl,-rpath,$ORIGIN/../lib", *zlib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stderr}")
        os.replace(tmp, DRIVER)
    return HOST_LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
