"""CPU oracle for thcpp's ISDF hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg (and its
``--impl reference`` arm) may import this package.  It is the checker of the CUDA path,
never the thing shipped or measured as the product.

Contents
--------
``kmeans_oracle.cpp``  single-rank C++ restatement of ``src/kmeans.cpp`` (k-means points),
                       compiled by :func:`build` into ``oracle/_build/libkmeans_oracle.so``.
``isdf.py``            numpy/scipy restatement of ``src/interpolating_vectors.cpp``
                       (plain and half-rotated):
                       the literal complex form (zgels QR, C2C FFT, herk, zpotrf) and the
                       regularised real form (Cholesky, R2C) used as the parity target.
``qrcp.py``            numpy/scipy restatement of ``src/qrcp.cpp`` (QRCP points): the
                       literal Z^T + pivoted Householder QR, and the pivoted Cholesky of
                       Z Z^T that the CUDA path implements.

Parity pinning
--------------
The reference's own tests hold no golden vector for this path (its Catch2 tests cover
only real ``d``-routines and the molecular LS-THC path), and the reference cannot be
built here (MPI, BLACS/ScaLAPACK, FFTW3 and the HDF5 C++ API are absent), so parity is
pinned by known-answer tests written for this project (constructed k-means ties,
delta/plane-wave FFTs, analytic Gaussian Coulomb integrals, L L^T = M) and by
cross-checking the two oracle formulations against each other.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
KMEANS_SO = os.path.join(BUILD, "libkmeans_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C++ k-means oracle (g++, OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "kmeans_oracle.cpp")
    if force or not os.path.exists(KMEANS_SO) or os.path.getmtime(KMEANS_SO) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = KMEANS_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC",
                               "-shared", "-o", tmp, src])
        os.replace(tmp, KMEANS_SO)
    return KMEANS_SO


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(KMEANS_SO)
        vp, i64, ci, cu, cd = (ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                               ctypes.c_uint, ctypes.c_double)
        lib.orc_initial_indices.argtypes = [i64, ci, cu, vp]
        lib.orc_initial_indices.restype = ci
        lib.orc_classify.argtypes = [vp, i64, vp, ci, vp, ci]
        lib.orc_classify.restype = None
        lib.orc_kmeans.argtypes = [vp, vp, i64, ci, vp, ci, cd, ci, vp, vp, vp, vp, vp]
        lib.orc_kmeans.restype = ci
        lib.orc_num_threads.argtypes = []
        lib.orc_num_threads.restype = ci
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def initial_indices(ng: int, nmu: int, seed: int) -> np.ndarray:
    """mt19937 + std::shuffle initial points (src/kmeans.cpp:159-168)."""
    out = np.zeros(nmu, np.int32)
    st = _load().orc_initial_indices(ng, nmu, seed, _p(out))
    if st:
        raise ValueError("bad arguments")
    return out


def classify(grid: np.ndarray, centroids: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """classify_grid_points (src/kmeans.cpp:88-106)."""
    g = np.ascontiguousarray(grid, np.float64)
    c = np.ascontiguousarray(centroids, np.float64)
    out = np.zeros(g.shape[0], np.int32)
    _load().orc_classify(_p(g), g.shape[0], _p(c), c.shape[0], _p(out),
                         nthreads or os.cpu_count() or 1)
    return out


class KMeansResult:
    def __init__(self, status, idx, iters, diff, centroids, labels):
        self.status = status
        self.idx = idx
        self.iters = iters
        self.diff = diff
        self.centroids = centroids
        self.labels = labels


def kmeans(grid, rho, nmu, init_idx, max_it, threshold, nthreads: int = 0) -> KMeansResult:
    """Single-rank KMeansSolver::kernel (src/kmeans.cpp:187-264)."""
    g = np.ascontiguousarray(grid, np.float64)
    r = np.ascontiguousarray(rho, np.float64).reshape(-1)
    init = np.ascontiguousarray(init_idx, np.int32)
    ng = g.shape[0]
    idx = np.zeros(nmu, np.int32)
    cen = np.zeros((nmu, 3))
    labels = np.zeros(ng, np.int32)
    iters = ctypes.c_int()
    diff = ctypes.c_double()
    st = _load().orc_kmeans(_p(g), _p(r), ng, nmu, _p(init), max_it, threshold,
                            nthreads or os.cpu_count() or 1, _p(idx), ctypes.byref(iters),
                            ctypes.byref(diff), _p(cen), _p(labels))
    return KMeansResult(st, idx, iters.value, diff.value, cen, labels)


def kmeans_system(system, nthreads: int = 0) -> KMeansResult:
    init = initial_indices(system.ng, system.nmu, system.rng_seed)
    return kmeans(system.grid, system.density, system.nmu, init, system.max_it,
                  system.threshold, nthreads)


from .isdf import (isdf_reference, isdf_real, half_spectrum_weights,  # noqa: E402,F401
                   pair_coulomb_exact, thc_pair_coulomb, isdf_half_reference)
from .qrcp import qrcp_reference, qrcp_gram, z_transpose  # noqa: E402,F401
