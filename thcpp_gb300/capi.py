"""ctypes binding of libthc_gb300.so (the C ABI declared in include/thc_gb300.h).

Arrays may be numpy arrays (host memory: the library copies them to the device) or
CUDA tensors / any object with ``data_ptr()`` (device memory: used in place).  Loading
fails loudly when the shared library is missing -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

THC_OK = 0
THC_ERR_ARG = 1
THC_ERR_CUDA = 2
THC_ERR_EMPTY_CLUSTER = 3
THC_ERR_NOT_PD = 4
THC_ERR_SHAPE = 5
THC_ERR_IO = 6
THC_ERR_TIMEOUT = 7
THC_ERR_NOMEM = 8
THC_ERR_CUFFT = 9

THC_PREC_FP64 = 0
THC_PREC_MIXED = 1

# Every symbol include/thc_gb300.h declares.
EXPORTS = [
    "thc_ctx_create", "thc_ctx_destroy", "thc_ctx_set_stream", "thc_ctx_set_option",
    "thc_ctx_last_error", "thc_status_string", "thc_ctx_kernel_launches",
    "thc_kmeans_initial_indices", "thc_kmeans", "thc_isdf", "thc_ctx_kernel_time",
    "thc_kmeans_history", "thc_factorize_batched", "thc_kmeans_noalloc",
    "thc_synth_gaussian_basis", "thc_isdf_half", "thc_qrcp", "thc_isdf_complex",
    "thc_qrcp_complex", "thc_isdf_interpolating_vectors", "thc_isdf_half_complex",
    "thc_ctx_autotune_log",
]


class KMeansStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("zero_filled", ctypes.c_int), ("duplicates", ctypes.c_int),
                ("final_diff", ctypes.c_double), ("pct_changed", ctypes.c_double),
                ("rechecked", ctypes.c_longlong), ("device_ms", ctypes.c_double)]


class IsdfStats(ctypes.Structure):
    _fields_ = [("chol_c_info", ctypes.c_int), ("chol_m_info", ctypes.c_int),
                ("rank_deficient", ctypes.c_int), ("n_anti", ctypes.c_int),
                ("shift_used", ctypes.c_double), ("c_min_pivot", ctypes.c_double),
                ("device_ms", ctypes.c_double)]


class QrcpStats(ctypes.Structure):
    _fields_ = [("numerical_rank", ctypes.c_int), ("device_ms", ctypes.c_double)]


class System(ctypes.Structure):
    """One system of thc_factorize_batched (include/thc_gb300.h: thc_system)."""
    _fields_ = [("grid", ctypes.c_void_p), ("rho", ctypes.c_void_p), ("ng", ctypes.c_longlong),
                ("nmu", ctypes.c_int), ("init_idx", ctypes.c_void_p), ("max_it", ctypes.c_int),
                ("threshold", ctypes.c_double), ("phi", ctypes.c_void_p),
                ("norb", ctypes.c_int), ("mesh", ctypes.c_void_p), ("coulG", ctypes.c_void_p),
                ("shift_rel", ctypes.c_double), ("out_idx", ctypes.c_void_p),
                ("out_orbitals", ctypes.c_void_p), ("out_M", ctypes.c_void_p),
                ("out_L", ctypes.c_void_p), ("status", ctypes.c_int),
                ("kmeans_stats", KMeansStats), ("isdf_stats", IsdfStats),
                ("error", ctypes.c_char * 192)]


class ThcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libthc_gb300.so; raise if it is absent (unless asked to build it)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; "
                               f"g.build()'` (no CPU fallback exists)")
        _build.build()
    lib = ctypes.CDLL(path)
    vp, ci, cll, cd, cu = (ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double,
                           ctypes.c_uint)
    lib.thc_ctx_create.argtypes = [ci, ci, ctypes.POINTER(vp)]
    lib.thc_ctx_destroy.argtypes = [vp]
    lib.thc_ctx_set_stream.argtypes = [vp, vp]
    lib.thc_ctx_set_option.argtypes = [vp, ctypes.c_char_p, cd]
    lib.thc_ctx_last_error.argtypes = [vp]
    lib.thc_ctx_last_error.restype = ctypes.c_char_p
    lib.thc_ctx_autotune_log.argtypes = [vp]
    lib.thc_ctx_autotune_log.restype = ctypes.c_char_p
    lib.thc_status_string.argtypes = [ci]
    lib.thc_status_string.restype = ctypes.c_char_p
    lib.thc_ctx_kernel_launches.argtypes = [vp]
    lib.thc_ctx_kernel_launches.restype = cll
    lib.thc_ctx_kernel_time.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(cd),
                                        ctypes.POINTER(cll)]
    lib.thc_ctx_kernel_time.restype = ci
    lib.thc_factorize_batched.argtypes = [ci, ci, ctypes.POINTER(System), ci, ci]
    lib.thc_factorize_batched.restype = ci
    lib.thc_kmeans_history.argtypes = [vp, vp, vp, ci]
    lib.thc_kmeans_history.restype = ci
    lib.thc_kmeans_initial_indices.argtypes = [cll, ci, cu, vp]
    lib.thc_kmeans.argtypes = [vp, vp, vp, cll, ci, vp, ci, cd, vp, ctypes.POINTER(KMeansStats)]
    lib.thc_kmeans_noalloc.argtypes = lib.thc_kmeans.argtypes
    lib.thc_synth_gaussian_basis.argtypes = [vp, vp, vp, vp, vp, ci, vp, ci, cd, vp]
    lib.thc_synth_gaussian_basis.restype = ci
    lib.thc_isdf.argtypes = [vp, vp, cll, ci, vp, ci, vp, vp, cd, vp, vp, vp,
                             ctypes.POINTER(IsdfStats)]
    lib.thc_isdf_half.argtypes = [vp, vp, cll, ci, vp, ci, vp, ci, vp, vp, cd, vp, vp, vp,
                                  ctypes.POINTER(IsdfStats)]
    lib.thc_isdf_complex.argtypes = lib.thc_isdf.argtypes
    lib.thc_qrcp_complex.argtypes = [vp, vp, cll, ci, ci, vp, vp, vp, ctypes.POINTER(QrcpStats)]
    lib.thc_qrcp.argtypes = [vp, vp, cll, ci, vp, ci, ci, vp, vp, vp, ctypes.POINTER(QrcpStats)]
    lib.thc_isdf_interpolating_vectors.argtypes = [vp, cll, ci, vp]
    lib.thc_isdf_half_complex.argtypes = [vp, vp, cll, ci, vp, ci, vp, ci, vp, vp, vp, vp, vp,
                                          ctypes.POINTER(IsdfStats)]
    for f in ("thc_ctx_create", "thc_ctx_destroy", "thc_ctx_set_stream", "thc_ctx_set_option",
              "thc_kmeans_initial_indices", "thc_kmeans", "thc_isdf", "thc_kmeans_noalloc",
              "thc_isdf_half", "thc_qrcp", "thc_isdf_complex", "thc_qrcp_complex",
              "thc_isdf_interpolating_vectors", "thc_isdf_half_complex"):
        getattr(lib, f).restype = ci
    _lib = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data_as(ctypes.c_void_p)
    raise TypeError(f"unsupported array type {type(a)}")


def _is_complex(a) -> bool:
    """Whether ``a`` holds complex values, without converting it (device tensors stay put)."""
    if hasattr(a, "is_complex"):
        return bool(a.is_complex())
    return bool(np.iscomplexobj(a))


def _complex_pairs(a):
    """A complex array as its (re, im) float64 pairs, shape ``a.shape + (2,)``.

    Tensors (any device) go through ``torch.view_as_real`` and keep their device; numpy
    arrays through a float64 view.
    """
    if hasattr(a, "is_complex"):
        import torch
        if a.dtype != torch.complex128:
            raise TypeError(f"complex orbitals must be complex128, not {a.dtype}")
        return torch.view_as_real(a.contiguous())
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a.view(np.float64).reshape(a.shape + (2,))


def factorize_batched(systems, device=0, precision=THC_PREC_MIXED, nstreams=8):
    """Run thc_factorize_batched on a list of dicts with the thc_system fields.

    Array fields hold numpy arrays or device tensors (kept alive by the caller).
    Returns (status, array of System).
    """
    arr = (System * len(systems))()
    for i, d in enumerate(systems):
        for k, v in d.items():
            if hasattr(v, "data_ptr") or isinstance(v, np.ndarray):
                setattr(arr[i], k, _ptr(v).value if _ptr(v) is not None else None)
            else:
                setattr(arr[i], k, v)
    st = load().thc_factorize_batched(device, precision, arr, len(systems), nstreams)
    return st, arr


def initial_indices(ng: int, nmu: int, seed: int) -> np.ndarray:
    out = np.zeros(nmu, np.int32)
    st = load().thc_kmeans_initial_indices(ng, nmu, seed, _ptr(out))
    if st:
        raise ThcError(st, "thc_kmeans_initial_indices failed")
    return out


class Context:
    """One GPU context (device, precision, stream, workspace)."""

    def __init__(self, device: int = 0, precision: int = THC_PREC_FP64):
        self.lib = load()
        h = ctypes.c_void_p()
        st = self.lib.thc_ctx_create(device, precision, ctypes.byref(h))
        if st:
            raise ThcError(st, "thc_ctx_create failed: "
                           + self.lib.thc_status_string(st).decode())
        self.h = h
        self.precision = precision

    def close(self):
        if getattr(self, "h", None):
            self.lib.thc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st:
            raise ThcError(st, f"{what}: {self.lib.thc_ctx_last_error(self.h).decode()}")

    def set_option(self, key: str, value: float):
        self._check(self.lib.thc_ctx_set_option(self.h, key.encode(), float(value)), key)

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.thc_ctx_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)),
                    "set_stream")

    def kernel_time(self, name: str):
        """(total ms, launches) of the profiled kernel `name`."""
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        self._check(self.lib.thc_ctx_kernel_time(self.h, name.encode(), ctypes.byref(ms),
                                                 ctypes.byref(n)), "kernel_time")
        return ms.value, n.value

    def autotune_log(self):
        """The autotuner's decisions on this device, one string per shape class."""
        txt = self.lib.thc_ctx_autotune_log(self.h).decode()
        return [ln for ln in txt.splitlines() if ln]

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.thc_ctx_kernel_launches(self.h))

    def kmeans(self, grid, rho, nmu, init_idx, max_it, threshold, out_idx=None,
               raise_on_error=True):
        ng = int(grid.shape[0])
        if out_idx is None:
            out_idx = np.zeros(nmu, np.int32)
        stats = KMeansStats()
        st = self.lib.thc_kmeans(self.h, _ptr(grid), _ptr(rho), ng, nmu, _ptr(init_idx), max_it,
                                 threshold, _ptr(out_idx), ctypes.byref(stats))
        if raise_on_error:
            self._check(st, "thc_kmeans")
        return out_idx, stats, st

    def kmeans_noalloc(self, grid, rho, nmu, init_idx, max_it, threshold, out_idx=None,
                       raise_on_error=True):
        """thc_kmeans_noalloc: thc_kmeans on a fixed device scratch (no allocation)."""
        ng = int(grid.shape[0])
        if out_idx is None:
            out_idx = np.zeros(nmu, np.int32)
        stats = KMeansStats()
        st = self.lib.thc_kmeans_noalloc(self.h, _ptr(grid), _ptr(rho), ng, nmu, _ptr(init_idx),
                                         max_it, threshold, _ptr(out_idx), ctypes.byref(stats))
        if raise_on_error:
            self._check(st, "thc_kmeans_noalloc")
        return out_idx, stats, st

    def gaussian_basis(self, grid, mesh, centres, centre_atom, alphas, nfunc, rcut, out):
        """thc_synth_gaussian_basis: periodised Gaussian s/p functions into ``out`` (device)."""
        mesh_a = np.ascontiguousarray(np.asarray(mesh, dtype=np.int32).reshape(3))
        st = self.lib.thc_synth_gaussian_basis(self.h, _ptr(grid), _ptr(mesh_a), _ptr(centres),
                                               _ptr(centre_atom), int(centre_atom.shape[0]),
                                               _ptr(alphas), int(nfunc), float(rcut), _ptr(out))
        self._check(st, "thc_synth_gaussian_basis")
        return out

    def kmeans_history(self, n):
        diff = np.zeros(n)
        pct = np.zeros(n)
        self._check(self.lib.thc_kmeans_history(self.h, _ptr(diff), _ptr(pct), n), "history")
        return diff, pct

    def isdf(self, phi, idx, mesh, coulG, shift_rel=-1.0, out_orbitals=None, out_M=None,
             out_L=None, raise_on_error=True, want=("M", "L", "orbitals")):
        ng, no = int(phi.shape[0]), int(phi.shape[1])
        nmu = int(idx.shape[0])
        mesh_a = np.ascontiguousarray(np.asarray(mesh, dtype=np.int32).reshape(3))
        if out_M is None and "M" in want:
            out_M = np.zeros((nmu, nmu, 2))
        if out_L is None and "L" in want:
            out_L = np.zeros((nmu, nmu, 2))
        if out_orbitals is None and "orbitals" in want:
            out_orbitals = np.zeros((no, nmu, 2))
        stats = IsdfStats()
        st = self.lib.thc_isdf(self.h, _ptr(phi), ng, no, _ptr(idx), nmu, _ptr(mesh_a),
                               _ptr(coulG), float(shift_rel), _ptr(out_orbitals), _ptr(out_M),
                               _ptr(out_L), ctypes.byref(stats))
        if raise_on_error and st not in (THC_OK, THC_ERR_NOT_PD):
            self._check(st, "thc_isdf")
        return dict(M=out_M, L=out_L, orbitals=out_orbitals, stats=stats, status=st)

    def interpolating_vectors(self, ng, nmu, out=None):
        """thc_isdf_interpolating_vectors: zeta^T (N_mu x N_g float64) of the last ISDF call;
        into ``out`` (host array or device tensor) when given."""
        if out is None:
            out = np.zeros((nmu, ng))
        self._check(self.lib.thc_isdf_interpolating_vectors(self.h, int(ng), int(nmu),
                                                            _ptr(out)),
                    "thc_isdf_interpolating_vectors")
        return out

    def isdf_complex(self, phi, idx, mesh, coulG, shift_rel=-1.0):
        """thc_isdf_complex: ``phi`` complex128 (N_g, N_o) or float64 (N_g, N_o, 2)."""
        if _is_complex(phi):
            phi = _complex_pairs(phi)
        ng, no = int(phi.shape[0]), int(phi.shape[1])
        nmu = int(idx.shape[0])
        mesh_a = np.ascontiguousarray(np.asarray(mesh, dtype=np.int32).reshape(3))
        out_M = np.zeros((nmu, nmu, 2))
        out_L = np.zeros((nmu, nmu, 2))
        out_orb = np.zeros((no, nmu, 2))
        stats = IsdfStats()
        st = self.lib.thc_isdf_complex(self.h, _ptr(phi), ng, no, _ptr(idx), nmu, _ptr(mesh_a),
                                       _ptr(coulG), float(shift_rel), _ptr(out_orb),
                                       _ptr(out_M), _ptr(out_L), ctypes.byref(stats))
        if st not in (THC_OK, THC_ERR_NOT_PD):
            self._check(st, "thc_isdf_complex")
        return dict(M=out_M, L=out_L, orbitals=out_orb, stats=stats, status=st)

    def qrcp(self, phi, npts, phi_occ=None):
        """thc_qrcp: QRCP interpolating points (sorted), pivot order and |R_kk|."""
        ng, no = int(phi.shape[0]), int(phi.shape[1])
        nocc = 0 if phi_occ is None else int(phi_occ.shape[1])
        idx = np.zeros(npts, np.int32)
        order = np.zeros(npts, np.int32)
        diag = np.zeros(npts)
        stats = QrcpStats()
        if _is_complex(phi):
            if phi_occ is not None:
                raise ValueError("the half-rotated QRCP takes real orbitals")
            pr = _complex_pairs(phi)
            st = self.lib.thc_qrcp_complex(self.h, _ptr(pr), ng, no, int(npts), _ptr(idx),
                                           _ptr(order), _ptr(diag), ctypes.byref(stats))
        else:
            st = self.lib.thc_qrcp(self.h, _ptr(phi), ng, no, _ptr(phi_occ), nocc, int(npts),
                                   _ptr(idx), _ptr(order), _ptr(diag), ctypes.byref(stats))
        self._check(st, "thc_qrcp")
        return dict(idx=idx, order=order, diag=diag, stats=stats)

    def isdf_half_complex(self, phi, phi_occ, idx, mesh, coulG):
        """thc_isdf_half_complex: complex128 (N_g, N_o) / (N_g, N_occ) orbitals, or their
        float64 (..., 2) pairs; returns M, the complex orbitals at the points and stats."""
        if _is_complex(phi):
            phi = _complex_pairs(phi)
        if _is_complex(phi_occ):
            phi_occ = _complex_pairs(phi_occ)
        ng, no, nocc = int(phi.shape[0]), int(phi.shape[1]), int(phi_occ.shape[1])
        nmu = int(idx.shape[0])
        mesh_a = np.ascontiguousarray(np.asarray(mesh, dtype=np.int32).reshape(3))
        out_M = np.zeros((nmu, nmu, 2))
        out_orb = np.zeros((no, nmu, 2))
        out_occ = np.zeros((nocc, nmu, 2))
        stats = IsdfStats()
        st = self.lib.thc_isdf_half_complex(self.h, _ptr(phi), ng, no, _ptr(phi_occ), nocc,
                                            _ptr(idx), nmu, _ptr(mesh_a), _ptr(coulG),
                                            _ptr(out_orb), _ptr(out_occ), _ptr(out_M),
                                            ctypes.byref(stats))
        self._check(st, "thc_isdf_half_complex")
        return dict(M=out_M, orbitals=out_orb, occ_orbitals=out_occ, stats=stats, status=st)

    def isdf_half(self, phi, phi_occ, idx, mesh, coulG, shift_rel=-1.0):
        """thc_isdf_half: half-rotated interpolating vectors and M (no Cholesky factor)."""
        ng, no = int(phi.shape[0]), int(phi.shape[1])
        nocc = int(phi_occ.shape[1])
        if int(phi_occ.shape[0]) != ng:
            raise ValueError("phi_occ must have N_g rows")
        nmu = int(idx.shape[0])
        mesh_a = np.ascontiguousarray(np.asarray(mesh, dtype=np.int32).reshape(3))
        out_M = np.zeros((nmu, nmu, 2))
        out_orb = np.zeros((no, nmu, 2))
        out_occ = np.zeros((nocc, nmu, 2))
        stats = IsdfStats()
        st = self.lib.thc_isdf_half(self.h, _ptr(phi), ng, no, _ptr(phi_occ), nocc, _ptr(idx),
                                    nmu, _ptr(mesh_a), _ptr(coulG), float(shift_rel),
                                    _ptr(out_orb), _ptr(out_occ), _ptr(out_M),
                                    ctypes.byref(stats))
        self._check(st, "thc_isdf_half")
        return dict(M=out_M, orbitals=out_orb, occ_orbitals=out_occ, stats=stats, status=st)
