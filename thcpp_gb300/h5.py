"""Python access to the HDF5 subset of thcpp's files through h5lite (libthcpp_host.so).

h5py is not available on the build or GPU hosts; these helpers read and write the same
files as the C++ solver classes: f64 / i32 datasets and complex128 as h5py's {r, i}
compound (orbital files) or as a trailing dimension of 2 (QMCPACK output).
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
KIND_INT, KIND_FLOAT, KIND_COMPLEX = 0, 1, 2


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.HOST_LIB):
            raise RuntimeError(f"{_build.HOST_LIB} missing: build the package first")
        lib = ctypes.CDLL(_build.HOST_LIB)
        vp, ci, cc = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p
        lib.h5l_last_error.restype = cc
        lib.h5l_writer_open.argtypes = [cc, ci]
        lib.h5l_writer_open.restype = vp
        lib.h5l_writer_write.argtypes = [vp, cc, ci, ci, ctypes.POINTER(ctypes.c_ulonglong), vp]
        lib.h5l_writer_write.restype = ci
        lib.h5l_writer_close.argtypes = [vp]
        lib.h5l_reader_open.argtypes = [cc]
        lib.h5l_reader_open.restype = vp
        lib.h5l_reader_close.argtypes = [vp]
        lib.h5l_reader_info.argtypes = [vp, cc, ctypes.POINTER(ci), ctypes.POINTER(ci),
                                        ctypes.POINTER(ctypes.c_ulonglong)]
        lib.h5l_reader_info.restype = ci
        lib.h5l_reader_read.argtypes = [vp, cc, ci, vp, ctypes.c_ulonglong]
        lib.h5l_reader_read.restype = ci
        _lib = lib
    return _lib


def _err():
    return _load().h5l_last_error().decode()


class Writer:
    def __init__(self, path: str, truncate: bool = True):
        self.h = _load().h5l_writer_open(path.encode(), 1 if truncate else 0)
        if not self.h:
            raise OSError(_err())

    def write(self, name: str, data, complex_compound: bool = False):
        a = np.asarray(data)
        if complex_compound or np.iscomplexobj(a):
            kind = 2
            buf = np.ascontiguousarray(a.astype(np.complex128)).view(np.float64)
            dims = a.shape
        elif np.issubdtype(a.dtype, np.integer):
            kind = 1
            buf = np.ascontiguousarray(a, dtype=np.int32)
            dims = a.shape
        else:
            kind = 0
            buf = np.ascontiguousarray(a, dtype=np.float64)
            dims = a.shape
        d = (ctypes.c_ulonglong * max(len(dims), 1))(*dims)
        st = _load().h5l_writer_write(self.h, name.encode(), kind, len(dims), d,
                                      buf.ctypes.data_as(ctypes.c_void_p))
        if st:
            raise OSError(_err())

    def close(self):
        if self.h:
            _load().h5l_writer_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Reader:
    def __init__(self, path: str):
        self.h = _load().h5l_reader_open(path.encode())
        if not self.h:
            raise OSError(_err())

    def info(self, name: str):
        kind, rank = ctypes.c_int(), ctypes.c_int()
        dims = (ctypes.c_ulonglong * 8)()
        if _load().h5l_reader_info(self.h, name.encode(), ctypes.byref(kind), ctypes.byref(rank),
                                   dims):
            raise OSError(_err())
        return kind.value, tuple(dims[i] for i in range(rank.value))

    def exists(self, name: str) -> bool:
        return self.info(name)[0] >= 0

    def read(self, name: str, as_complex: bool | None = None):
        kind, shape = self.info(name)
        if kind < 0:
            raise KeyError(name)
        cplx = (kind == KIND_COMPLEX) if as_complex is None else as_complex
        n = int(np.prod(shape)) if shape else 1
        out = np.zeros(2 * n if cplx else n)
        if _load().h5l_reader_read(self.h, name.encode(), 1 if cplx else 0,
                                   out.ctypes.data_as(ctypes.c_void_p), out.size):
            raise OSError(_err())
        if cplx:
            return out.view(np.complex128).reshape(shape)
        if kind == KIND_INT:
            return out.astype(np.int64).reshape(shape)
        return out.reshape(shape)

    def close(self):
        if self.h:
            _load().h5l_reader_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
