"""Error paths of the C ABI on the GPU, made without faulting anything.

* A bounded device wait that runs out: the context option "spin_limit" = 0 makes every
  mbarrier wait of the tensor-core GEMM give up at once (before any copy or MMA is issued);
  the call returns THC_ERR_TIMEOUT and the next call on the same context is exact again.
* Cholesky breakdowns reported the way the reference reports them: THC_ERR_NOT_PD for M
  (the reference prints the failed minor and still writes Luv,
  src/interpolating_vectors.cpp:296-304) and for a singular C solved without a shift.
"""
import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu


def _cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_device_wait_timeout_is_reported_and_context_stays_usable(gpu_ctx_mixed):
    s = system("tiny")
    idx = oracle.kmeans_system(s).idx
    gpu_ctx_mixed.set_option("spin_limit", 0)
    try:
        r = gpu_ctx_mixed.isdf(s.phi, idx, s.mesh, s.coulG, raise_on_error=False)
        assert r["status"] == capi.THC_ERR_TIMEOUT
        assert "timed out" in gpu_ctx_mixed.lib.thc_ctx_last_error(gpu_ctx_mixed.h).decode()
    finally:
        gpu_ctx_mixed.set_option("spin_limit", 1 << 24)
    r = gpu_ctx_mixed.isdf(s.phi, idx, s.mesh, s.coulG)
    assert r["status"] == capi.THC_OK
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    assert _rel(_cplx(r["M"]), ref["M"]) < 1e-6


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_m_not_positive_definite(gpu_ctx_fp64, gpu_ctx_mixed, prec):
    """A negative Coulomb kernel makes M negative definite: THC_ERR_NOT_PD with the failed
    leading minor, and M and Luv are still written."""
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system("tiny")
    idx = oracle.kmeans_system(s).idx
    r = ctx.isdf(s.phi, idx, s.mesh, -s.coulG, raise_on_error=False)
    assert r["status"] == capi.THC_ERR_NOT_PD
    assert r["stats"].chol_m_info == 1
    ref = oracle.isdf_real(s.phi, idx, s.mesh, -s.coulG)
    assert _rel(_cplx(r["M"]), ref["M"]) < 1e-6
    assert np.isfinite(r["L"]).all()
    ok = ctx.isdf(s.phi, idx, s.mesh, s.coulG)
    assert ok["status"] == capi.THC_OK


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_singular_c_without_shift(gpu_ctx_fp64, gpu_ctx_mixed, prec):
    """C1's C is singular (N_mu 64 > 36 pair products); shift_rel = 0 forbids the shift, so
    the Cholesky of C breaks down: THC_ERR_NOT_PD, and the automatic policy still works."""
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system("c1")
    idx = oracle.kmeans_system(s).idx
    r = ctx.isdf(s.phi, idx, s.mesh, s.coulG, 0.0, raise_on_error=False)
    assert r["status"] == capi.THC_ERR_NOT_PD
    assert "Cholesky of C failed" in ctx.lib.thc_ctx_last_error(ctx.h).decode()
    r = ctx.isdf(s.phi, idx, s.mesh, s.coulG)
    assert r["status"] == capi.THC_OK and r["stats"].rank_deficient == 1
