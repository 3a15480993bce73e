"""Accuracy of the ISDF path against FP64 oracles, per config: M, the interpolating vectors
zeta and the reconstructed orbital-pair densities.

Two oracles: the CPU restatement (oracle/isdf.py, numpy/scipy) and the blocked FP64 GPU
oracle (oracle/isdf_torch.py, torch float64), the second checked against the first here
before it is used for the cells the CPU oracle cannot reach in a test.  The k-means points
of every cell come from the reference's own k-means (tests/golden/ref_kmeans.npz), so these
tests also run the ISDF at exactly the reference's points.
"""
import os

import numpy as np
import pytest

import oracle
from oracle import isdf_torch
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kmeans.npz")


def ref_idx(name):
    return np.load(GOLDEN)[f"{name}_idx"]


def _cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


_TORCH = {}


def torch_oracle(name):
    if name not in _TORCH:
        s = system(name)
        _TORCH[name] = isdf_torch.isdf_real(s.phi, ref_idx(name), s.mesh, s.coulG)
    return _TORCH[name]


@pytest.mark.parametrize("name", ["tiny", "c2", "c3"])
def test_gpu_oracle_matches_cpu_oracle(name):
    """The blocked torch FP64 oracle against the numpy/scipy restatement."""
    s = system(name)
    idx = ref_idx(name)
    cpu = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    gpu = torch_oracle(name)
    # Two FP64 solves of the same system agree to ~cond(C) u (tiny: cond 3e10).
    assert _rel(gpu["M"], cpu["M"]) < max(1e-10, gpu["cond_C"] * 2.2e-16)
    zt = gpu["zeta_t"].cpu().numpy()
    assert _rel(zt, cpu["zeta_t"]) < max(1e-10, 100 * gpu["cond_C"] * 2.2e-16)


# (config, FP64 tolerance on M / zeta, mixed tolerance on M, on zeta)
CASES = [("c2", 1e-9, 1e-9, 1e-6, 1e-5), ("c3", 1e-9, 1e-8, 1e-6, 1e-5)]


@pytest.mark.parametrize("name,tm64,tz64,tmx,tzx", CASES)
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_isdf_accuracy_against_fp64_oracle(gpu_ctx_fp64, gpu_ctx_mixed, prec, name, tm64, tz64,
                                           tmx, tzx):
    import torch
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system(name)
    idx = ref_idx(name)
    ref = torch_oracle(name)
    dev = torch.device("cuda", 0)
    r = ctx.isdf(torch.from_numpy(s.phi).to(dev), torch.from_numpy(idx).to(dev), s.mesh,
                 torch.from_numpy(s.coulG).to(dev))
    assert r["status"] == 0
    zt = torch.empty((s.nmu, s.ng), dtype=torch.float64, device=dev)
    ctx.interpolating_vectors(s.ng, s.nmu, out=zt)
    em = _rel(_cplx(r["M"]), ref["M"])
    ez = float(torch.linalg.norm(zt - ref["zeta_t"]) / torch.linalg.norm(ref["zeta_t"]))
    pairs = isdf_torch.sample_pairs(s.norb, 512)
    ep = isdf_torch.pair_density_error(zt, s.phi, idx, pairs)
    ep_ref = isdf_torch.pair_density_error(ref["zeta_t"], s.phi, idx, pairs)
    print(f"{name} {prec}: |dM|/|M| {em:.2e}  |dzeta|/|zeta| {ez:.2e}  pair density "
          f"{ep:.3e} (oracle {ep_ref:.3e})")
    assert em < (tm64 if prec == "fp64" else tmx)
    # zeta = C^{-1} Z amplifies rounding by up to cond(C).
    assert ez < max(tz64 if prec == "fp64" else tzx, 100 * ref["cond_C"] * 2.2e-16)
    # The reconstruction error is the ISDF's own (set by N_mu), not the arithmetic's.
    assert abs(ep - ep_ref) <= 1e-3 * ep_ref


def test_interpolating_vectors_host_output_and_errors(gpu_ctx_mixed):
    s = system("tiny")
    idx = ref_idx("tiny")
    gpu_ctx_mixed.isdf(s.phi, idx, s.mesh, s.coulG)
    zt = gpu_ctx_mixed.interpolating_vectors(s.ng, s.nmu)          # FP32, widened on host
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    assert _rel(zt, ref["zeta_t"]) < 1e-5
    with pytest.raises(capi.ThcError) as e:
        gpu_ctx_mixed.interpolating_vectors(s.ng + 1, s.nmu)
    assert e.value.status == capi.THC_ERR_SHAPE
    gpu_ctx_mixed.qrcp(s.phi, 8)                                     # reuses the Z slot
    with pytest.raises(capi.ThcError) as e:
        gpu_ctx_mixed.interpolating_vectors(s.ng, s.nmu)
    assert e.value.status == capi.THC_ERR_ARG


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_refined_shifted_solve_matches_oracle(gpu_ctx_fp64, gpu_ctx_mixed, prec):
    """A forced diagonal shift of 1e-6 tr(C)/N_mu on C2 (cond 2.3e6, so the shift biases the
    smallest eigen-directions by up to ~30 %), then 0, 1 and 2 refinement steps: each M
    matches the oracle's literal refinement, and every step moves M toward the unshifted
    solution."""
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system("c2")
    idx = ref_idx("c2")
    exact = torch_oracle("c2")["M"]
    prev = None
    try:
        for k in range(3):
            ctx.set_option("refine", k)
            r = ctx.isdf(s.phi, idx, s.mesh, s.coulG, 1e-6)
            assert r["status"] == 0 and r["stats"].rank_deficient == 1
            ref = isdf_torch.isdf_real(s.phi, idx, s.mesh, s.coulG, shift_rel=1e-6, refine=k,
                                       keep_zeta=False)
            M = _cplx(r["M"])
            err = _rel(M, ref["M"])
            to_exact = _rel(M, exact)
            print(f"{prec} refine {k}: |dM|/|M| vs refined oracle {err:.2e}, vs unshifted "
                  f"{to_exact:.2e}")
            assert err < (1e-9 if prec == "fp64" else 1e-6)
            if prev is not None:
                assert to_exact < 0.5 * prev
            prev = to_exact
    finally:
        ctx.set_option("refine", 0)
