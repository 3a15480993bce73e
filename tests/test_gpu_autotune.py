"""The sliced-GEMM autotuner: decisions are logged per shape class, shared by every context
of the process (so two contexts produce the same bits), and any decision gives the same
result to within the mixed path's rounding."""
import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu


def _cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def test_autotune_shared_and_logged():
    s = system("c2")
    idx = oracle.kmeans_system(s).idx
    with capi.Context(0, capi.THC_PREC_MIXED) as a, capi.Context(0, capi.THC_PREC_MIXED) as b:
        ra = a.isdf(s.phi, idx, s.mesh, s.coulG)
        rb = b.isdf(s.phi, idx, s.mesh, s.coulG)
        log = a.autotune_log()
        assert log and all("bk=" in ln and "split=" in ln for ln in log)
        assert b.autotune_log() == log
    assert np.array_equal(ra["M"], rb["M"])
    # The same product with the tuner off (default k-step, tile order and split).
    with capi.Context(0, capi.THC_PREC_MIXED) as c:
        c.set_option("autotune", 0)
        rc = c.isdf(s.phi, idx, s.mesh, s.coulG)
    # The choices change the summation order of the inexact level >= 3 accumulator and of the
    # split-K partials, and zeta is rounded to FP32 after them: agreement at the path's own
    # accuracy (~1e-7 against the FP64 oracle).
    Ma, Mc = _cplx(ra["M"]), _cplx(rc["M"])
    assert np.linalg.norm(Ma - Mc) <= 1e-7 * np.linalg.norm(Mc)
