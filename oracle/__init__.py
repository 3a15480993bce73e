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

``reference.py``       runs the reference's OWN ``src/kmeans.cpp``, compiled unmodified by
                       ``ref/Makefile`` into ``_ref/kmeans_ref`` (one-rank MPI stand-in,
                       in-memory datasets in place of the HDF5 file).

Parity pinning
--------------
k-means is pinned to the reference itself: ``reference.py`` runs its ``KMeansSolver`` and
the tests compare the restatement (and the GPU) with it, live where the reference tree is
present and through fixtures it generated (``tests/golden/ref_kmeans.npz``) elsewhere.
The ISDF half needs MPI, BLACS/ScaLAPACK, FFTW3 and the HDF5 C++ API, none of which is
installed, so it cannot be built; its restatement is pinned by known-answer tests written
for this project (delta/plane-wave FFTs, analytic Gaussian Coulomb integrals, L L^T = M)
and by cross-checking the two oracle formulations against each other.
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
        lib.orc_kmeans.argtypes = [vp, vp, i64, ci, vp, ci, cd, ci, vp, vp, vp, vp, vp, vp,
                                   vp]
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
    def __init__(self, status, idx, iters, diff, centroids, labels, diffs=None, pct=None):
        self.status = status
        self.idx = idx
        self.iters = iters
        self.diff = diff
        self.centroids = centroids
        self.labels = labels
        self.diffs = diffs      # normed difference of every completed iteration
        self.pct = pct          # percentage_change of every completed iteration


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
    diffs = np.zeros(max_it)
    pct = np.zeros(max_it)
    st = _load().orc_kmeans(_p(g), _p(r), ng, nmu, _p(init), max_it, threshold,
                            nthreads or os.cpu_count() or 1, _p(idx), ctypes.byref(iters),
                            ctypes.byref(diff), _p(cen), _p(labels), _p(diffs), _p(pct))
    n = iters.value
    return KMeansResult(st, idx, n, diff.value, cen, labels, diffs[:n], pct[:n])


def kmeans_system(system, nthreads: int = 0) -> KMeansResult:
    init = initial_indices(system.ng, system.nmu, system.rng_seed)
    return kmeans(system.grid, system.density, system.nmu, init, system.max_it,
                  system.threshold, nthreads)


from .isdf import (isdf_reference, isdf_real, half_spectrum_weights,  # noqa: E402,F401
                   pair_coulomb_exact, thc_pair_coulomb, isdf_half_reference)
from .qrcp import qrcp_reference, qrcp_gram, z_transpose  # noqa: E402,F401
