"""GPU QRCP interpolating points (thc_qrcp) against the oracle's pivots."""
import os

import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "qrcp.npz"))


def _check(r, key, exact=True):
    """exact: the pivots themselves; otherwise (a symmetric cell, where equivalent points
    tie up to rounding and either choice is a valid pivot) the |R_kk| sequence, which the
    symmetry leaves unchanged."""
    order = GOLDEN[key + "_order"]
    d = GOLDEN[key + "_diag"]
    if exact:
        assert np.array_equal(r["order"], order)
    assert np.array_equal(r["idx"], np.sort(r["order"]))
    assert len(set(r["order"].tolist())) == len(order)
    assert np.max(np.abs(r["diag"] - d)) <= 1e-10 * d[0]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_qrcp_c2_matches_householder(gpu_ctx_fp64, gpu_ctx_mixed, prec):
    """256 pivots over 110,592 grid points, identical to the literal QRCP of the 1024-row
    Z^T (the computation runs in FP64 in both precisions)."""
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system("c2")
    r = ctx.qrcp(s.phi, 256)
    _check(r, "c2")
    assert r["stats"].numerical_rank == 256


def test_qrcp_tiny_full_and_half(gpu_ctx_fp64):
    """The tiny cell is symmetric: equivalent grid points tie up to rounding."""
    s = system("tiny")
    _check(gpu_ctx_fp64.qrcp(s.phi, 48), "tiny", exact=False)
    po = np.ascontiguousarray(s.phi[:, : s.nocc])
    _check(gpu_ctx_fp64.qrcp(s.phi, 20, po), "tiny_half", exact=False)


def test_qrcp_half_rank_exhausted(gpu_ctx_fp64):
    """Past the numerical rank of the half-rotated row set (~27 on tiny) the residuals are
    rounding: the pivots up to it still match and the rank is reported."""
    s = system("tiny")
    po = np.ascontiguousarray(s.phi[:, : s.nocc])
    r = gpu_ctx_fp64.qrcp(s.phi, 48, po)
    d = GOLDEN["tiny_half_diag"]
    assert np.max(np.abs(r["diag"][:20] - d)) <= 1e-10 * d[0]
    assert 20 <= r["stats"].numerical_rank <= 30
    assert len(set(r["order"].tolist())) == 48
    assert np.all(np.isfinite(r["diag"]))


def test_qrcp_all_pairs_option(gpu_ctx_fp64):
    s = system("tiny")
    po = np.ascontiguousarray(s.phi[:, : s.nocc])
    gpu_ctx_fp64.set_option("qrcp_all_pairs", 1)
    try:
        r = gpu_ctx_fp64.qrcp(s.phi, 30, po)
    finally:
        gpu_ctx_fp64.set_option("qrcp_all_pairs", 0)
    ref = oracle.qrcp_gram(s.phi, 30, po, all_pairs=True)
    assert np.max(np.abs(r["diag"] - ref["diag"])) <= 1e-10 * ref["diag"][0]


def test_qrcp_invalid_arguments(gpu_ctx_fp64):
    s = system("tiny")
    with pytest.raises(capi.ThcError) as e:
        gpu_ctx_fp64.qrcp(s.phi, s.ng + 1)
    assert e.value.status == capi.THC_ERR_ARG


@pytest.mark.parametrize("name,npts", [("tiny", 48), ("c2", 256)])
def test_qrcp_complex(gpu_ctx_fp64, name, npts):
    """thc_qrcp_complex against the oracle's Gram form for complex orbitals Phi A: the same
    pivots and |R_kk| (Phi A has no symmetry-equivalent points)."""
    from tests.test_oracle import complex_orbitals
    s = system(name)
    pc = complex_orbitals(s.phi)
    r = gpu_ctx_fp64.qrcp(pc, npts)
    ref = oracle.qrcp_gram(pc, npts)
    assert np.max(np.abs(r["diag"] - ref["diag"])) <= 1e-10 * ref["diag"][0]
    assert np.array_equal(r["order"], ref["order"])
    assert np.array_equal(r["idx"], ref["idx"])
