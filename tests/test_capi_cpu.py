"""The C ABI library loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

import numpy as np

import oracle
from thcpp_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(thc_[a-z0-9_]+)\s*\(", text))
    return names


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert {"thc_kmeans", "thc_isdf", "thc_ctx_create"} <= names
    for n in names:
        assert hasattr(lib, n), f"{n} missing from libthc_gb300.so"
    assert names == set(capi.EXPORTS), "capi.EXPORTS out of sync with the header"


def test_status_strings(lib):
    for st in range(10):
        assert lib.thc_status_string(st)
    assert lib.thc_status_string(capi.THC_ERR_EMPTY_CLUSTER) == b"empty k-means cluster"


def test_initial_indices_match_oracle(lib):
    for ng, nmu, seed in [(13824, 64, 18), (110592, 256, 19), (70000, 5, 4294967295)]:
        assert np.array_equal(capi.initial_indices(ng, nmu, seed),
                              oracle.initial_indices(ng, nmu, seed))


def test_initial_indices_bad_args(lib):
    out = np.zeros(4, np.int32)
    p = out.ctypes.data_as(ctypes.c_void_p)
    assert lib.thc_kmeans_initial_indices(3, 4, 1, p) == capi.THC_ERR_ARG
    assert lib.thc_kmeans_initial_indices(10, 0, 1, p) == capi.THC_ERR_ARG


def test_null_context_rejected(lib):
    assert lib.thc_kmeans(None, None, None, 0, 0, None, 0, 0.0, None, None) == capi.THC_ERR_ARG
    assert lib.thc_isdf(None, None, 0, 0, None, 0, None, None, 0.0, None, None, None,
                        None) == capi.THC_ERR_ARG
