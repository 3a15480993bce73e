"""GPU ISDF through the C ABI against the oracle (FP64 and mixed precision)."""
import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu

_KM = {}


def kmeans_idx(name):
    if name not in _KM:
        _KM[name] = oracle.kmeans_system(system(name)).idx
    return _KM[name]


def _cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run(ctx, name, shift=-1.0):
    s = system(name)
    idx = kmeans_idx(name)
    r = ctx.isdf(s.phi, idx, s.mesh, s.coulG, shift)
    return s, idx, r


# (config, FP64 tolerance, mixed tolerance) on ||dM||/||M|| against the oracle
CASES = [("tiny", 1e-8, 1e-6), ("c2", 1e-9, 1e-6)]


@pytest.mark.parametrize("name,tol64,tolmx", CASES)
def test_isdf_fp64_matches_oracle(gpu_ctx_fp64, name, tol64, tolmx):
    s, idx, r = _run(gpu_ctx_fp64, name)
    assert r["status"] == 0
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    M = _cplx(r["M"])
    assert _rel(M, ref["M"]) < tol64
    L = _cplx(r["L"])
    assert np.allclose(np.triu(L, 1), 0)
    assert _rel(L @ L.conj().T, M) < 1e-12
    orb = _cplx(r["orbitals"])
    assert np.array_equal(orb.real, s.phi[idx].T) and not orb.imag.any()
    assert r["stats"].rank_deficient == 0 and r["stats"].n_anti == 0


@pytest.mark.parametrize("name,tol64,tolmx", CASES)
def test_isdf_mixed_matches_oracle(gpu_ctx_mixed, name, tol64, tolmx):
    s, idx, r = _run(gpu_ctx_mixed, name)
    assert r["status"] == 0
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    M = _cplx(r["M"])
    err = _rel(M, ref["M"])
    print(f"{name}: mixed ||dM||/||M|| = {err:.3e}")
    assert err < tolmx
    L = _cplx(r["L"])
    assert _rel(L @ L.conj().T, M) < 1e-12


def test_isdf_fp64_vs_reference_qr_c2(gpu_ctx_fp64):
    """Against the literal complex restatement (zgels QR, C2C FFT, herk, zpotrf)."""
    s, idx, r = _run(gpu_ctx_fp64, "c2")
    ref = oracle.isdf_reference(s.phi, idx, s.mesh, s.coulG)
    assert _rel(_cplx(r["M"]), ref["M"]) < 1e-9
    assert _rel(_cplx(r["L"]), ref["L"]) < 1e-8


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_isdf_rank_deficient_c1(request, prec):
    """C1: N_mu = 64 exceeds the 36 independent orbital-pair products, so C is singular.

    M is then not unique (the reference's QR returns rounding noise amplified ~1e16 in the
    null space of C).  The GPU path regularises C with the shift 1e-10 tr(C)/N_mu; with
    cond(C + shift) ~ 1e10 the explicit inverse cancels by ~1e12, so M agrees with the
    identically-regularised oracle only to ~1e-4 (FP64) / ~1e-2 (sliced BF16).  What the
    factorisation must preserve is the THC reconstruction X M X^T of the orbital-pair
    Coulomb integrals, which is independent of the null-space block.
    """
    ctx = request.getfixturevalue("gpu_ctx_fp64" if prec == "fp64" else "gpu_ctx_mixed")
    s, idx, r = _run(ctx, "c1")
    st = r["stats"]
    assert st.rank_deficient == 1 and st.chol_c_info > 0 and st.n_anti > 0
    pm = s.phi[idx]
    C = (pm @ pm.T) ** 2
    tr = np.trace(C) / s.nmu
    assert abs(st.shift_used - 1e-10 * tr) < 1e-12 * tr
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG, shift=1e-10 * tr)
    M = _cplx(r["M"])
    pairs = [(i, j) for i in range(s.norb) for j in range(i, s.norb)]
    ex = oracle.pair_coulomb_exact(s.phi, s.mesh, s.coulG, pairs)
    th = oracle.thc_pair_coulomb(s.phi, idx, M, pairs)
    th_ref = oracle.thc_pair_coulomb(s.phi, idx, ref["M"], pairs)
    inv, inv_ref = _rel(th, ex), _rel(th_ref, ex)
    print(f"c1 {prec}: ||dM||/||M|| = {_rel(M, ref['M']):.3e}; pair-Coulomb error "
          f"{inv:.3e} (oracle {inv_ref:.3e})")
    assert _rel(M, ref["M"]) < (1e-3 if prec == "fp64" else 1e-2)
    assert inv < 1e-4


def test_isdf_mixed_odd_nmu_split_k(gpu_ctx_mixed):
    """An odd N_mu (21 orbitals x 3 = 63, cond(C) ~ 1e5) with the Coulomb product split
    over K (9 ways): the partials of odd splits start at odd offsets, so paired stores must
    check the address."""
    from thcpp_gb300 import synth
    lat, atoms = synth.diamond_supercell(1)
    s = synth.make_system("odd", lat, atoms, (16, 16, 16), 21, 3, 1234, 77)
    assert s.nmu % 2 == 1
    idx = oracle.kmeans_system(s).idx
    r = gpu_ctx_mixed.isdf(s.phi, idx, s.mesh, s.coulG)
    assert r["status"] == 0
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    err = _rel(_cplx(r["M"]), ref["M"])
    print(f"odd N_mu: mixed ||dM||/||M|| = {err:.3e}")
    assert err < 1e-6


def test_isdf_mixed_fft64_option(lib):
    """zeta in FP64 through a D2Z FFT (the fft64 option) against the oracle on C2, and the
    slice-depth knob of the Coulomb product: fewer slices must not be more accurate."""
    s = system("c2")
    idx = kmeans_idx("c2")
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)["M"]
    err = {}
    for fft64, sm in ((0, 5), (1, 5), (0, 3)):
        with capi.Context(0, capi.THC_PREC_MIXED) as ctx:
            ctx.set_option("fft64", fft64)
            ctx.set_option("slices_m", sm)
            r = ctx.isdf(s.phi, idx, s.mesh, s.coulG)
            assert r["status"] == 0
            err[(fft64, sm)] = _rel(_cplx(r["M"]), ref)
    print("mixed ||dM||/||M|| (fft64, slices_m):", err)
    assert err[(1, 5)] < 1e-6 and err[(0, 5)] < 1e-6
    assert err[(0, 3)] > err[(0, 5)]


def test_sliced_gemm_tc_matches_mma_sync(lib):
    """The tcgen05 sliced GEMM against the warp-level mma.sync one (same slicing).

    Both sum the same exact slice products, but in a different order and precision (the
    tcgen05 epilogue folds in double-word FP32, the mma.sync one in FP64); zeta is then
    rounded to FP32 in both, where a one-ulp flip (2^-24 = 6e-8 relative) of single entries
    is expected.  The two must agree far inside the 1e-6 budget against the FP64 path.
    """
    s = system("c2")
    idx = kmeans_idx("c2")
    out = {}
    for key in ((0, 16), (1, 16), (1, 32)):
        with capi.Context(0, capi.THC_PREC_MIXED) as ctx:
            ctx.set_option("gemm_tc", key[0])
            ctx.set_option("tc_bk", key[1])
            out[key] = _cplx(ctx.isdf(s.phi, idx, s.mesh, s.coulG)["M"])
    for key in ((1, 16), (1, 32)):
        d = _rel(out[key], out[(0, 16)])
        print(f"tc (k-step {key[1]}) vs mma.sync ||dM||/||M|| = {d:.3e}")
        assert d < 1e-7


@pytest.mark.parametrize("name", ["tiny", "c2"])
def test_sliced_gemm_tile_widths(lib, name):
    """Every product of the mixed path through the 64-wide tiles (two CTAs per SM), the
    persistent kernel (for the products with K <= 512: P and, at these sizes, zeta) and the
    128-wide tiles, the autotuner off: the same exact slice products in another tile order
    (the persistent kernel drains its level >= 3 accumulator once per tile instead of every
    128 k), so M agrees to the path's rounding (zeta is FP32), and all match the oracle."""
    s = system(name)
    idx = kmeans_idx(name)
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)["M"]
    out = {}
    for key, opt in (("128", ("tc_bn", 128)), ("64", ("tc_bn", 64)),
                     ("persistent", ("tc_persistent", 1))):
        with capi.Context(0, capi.THC_PREC_MIXED) as ctx:
            ctx.set_option(*opt)
            r = ctx.isdf(s.phi, idx, s.mesh, s.coulG)
            assert r["status"] == 0
            out[key] = _cplx(r["M"])
        e = _rel(out[key], ref)
        print(f"{name} tiles {key}: ||dM||/||M|| vs oracle = {e:.3e}")
        assert e < 1e-6
    assert _rel(out["64"], out["128"]) < 1e-7
    assert _rel(out["persistent"], out["128"]) < 1e-7


def test_isdf_mesh_mismatch(gpu_ctx_fp64):
    s = system("tiny")
    r = gpu_ctx_fp64.isdf(s.phi, kmeans_idx("tiny"), (16, 16, 15), s.coulG, raise_on_error=False)
    assert r["status"] == capi.THC_ERR_SHAPE


def test_isdf_device_pointers(gpu_ctx_mixed):
    import torch
    s = system("tiny")
    idx = kmeans_idx("tiny")
    host = gpu_ctx_mixed.isdf(s.phi, idx, s.mesh, s.coulG)
    dev_M = torch.zeros((s.nmu, s.nmu, 2), dtype=torch.float64, device="cuda")
    gpu_ctx_mixed.isdf(torch.from_numpy(s.phi).cuda(), torch.from_numpy(idx).cuda(), s.mesh,
                       torch.from_numpy(s.coulG).cuda(), out_M=dev_M, want=("M",))
    torch.cuda.synchronize()
    assert np.array_equal(dev_M.cpu().numpy(), host["M"])


# (config, tolerance on ||dM||/||M||): C_half has cond ~3e10 on tiny, ~6e6 on c2
HALF_CASES = [("tiny", 1e-6), ("c2", 1e-9)]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name,tol", HALF_CASES)
def test_isdf_half_matches_oracle(gpu_ctx_fp64, gpu_ctx_mixed, prec, name, tol):
    """thc_isdf_half (runs in FP64 in both precisions) against the oracle's half-rotated
    real form, half the orbitals occupied."""
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system(name)
    idx = kmeans_idx(name)
    nocc = s.norb // 2
    po = np.ascontiguousarray(s.phi[:, :nocc])
    r = ctx.isdf_half(s.phi, po, idx, s.mesh, s.coulG)
    assert r["status"] == 0
    ref = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG, phi_occ=po)
    M = _cplx(r["M"])
    assert _rel(M, ref["M"]) < tol
    assert np.linalg.norm(M - M.conj().T) <= 1e-14 * np.linalg.norm(M)
    orb = _cplx(r["orbitals"])
    assert np.array_equal(orb.real, s.phi[idx].T) and not orb.imag.any()
    occ = _cplx(r["occ_orbitals"])
    assert np.array_equal(occ.real, po[idx].T) and not occ.imag.any()
    assert r["stats"].chol_m_info == 0


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name,tol", [("tiny", 1e-7), ("c2", 1e-9)])
def test_isdf_complex_matches_oracle(gpu_ctx_fp64, gpu_ctx_mixed, prec, name, tol):
    """thc_isdf_complex (FP64 in both precisions): complex orbitals Phi A against the
    oracle's real form with Z = |Phi_mu^H Phi|^2."""
    from tests.test_oracle import complex_orbitals
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system(name)
    idx = kmeans_idx(name)
    pc = complex_orbitals(s.phi)
    r = ctx.isdf_complex(pc, idx, s.mesh, s.coulG)
    assert r["status"] == 0
    ref = oracle.isdf_real(pc, idx, s.mesh, s.coulG)
    M = _cplx(r["M"])
    assert _rel(M, ref["M"]) < tol
    L = _cplx(r["L"])
    assert np.allclose(np.triu(L, 1), 0)
    assert _rel(L @ L.conj().T, M) < 1e-12
    assert np.array_equal(_cplx(r["orbitals"]), pc[idx].T)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name,npts,tol", [("tiny", None, 1e-6), ("c2", 128, 1e-9)])
def test_isdf_half_complex_matches_reference_form(gpu_ctx_fp64, gpu_ctx_mixed, prec, name, npts,
                                                  tol):
    """thc_isdf_half_complex (FP64 in both precisions) against the oracle's literal
    half-rotated form with complex orbitals (complex P and P_occ, Z = P_occ o conj(P), QR
    least squares, forward and backward C2C FFTs, IVMG^T IVG).  tiny: cond(C) 1.7e10; C2 with
    the first 128 k-means points: cond 8e5."""
    from tests.test_oracle import complex_orbitals
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system(name)
    idx = kmeans_idx(name)
    if npts:
        idx = np.ascontiguousarray(idx[:npts])
    pc = complex_orbitals(s.phi)
    po = np.ascontiguousarray(pc[:, : s.norb // 2])
    r = ctx.isdf_half_complex(pc, po, idx, s.mesh, s.coulG)
    assert r["status"] == 0
    ref = oracle.isdf_half_reference(pc, po, idx, s.mesh, s.coulG)
    err = _rel(_cplx(r["M"]), ref)
    print(f"{name} {prec}: half complex ||dM||/||M|| = {err:.3e}")
    assert err < tol
    assert np.array_equal(_cplx(r["orbitals"]), pc[idx].T)
    assert np.array_equal(_cplx(r["occ_orbitals"]), po[idx].T)
    assert 0 < r["stats"].c_min_pivot <= 1
