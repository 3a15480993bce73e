"""CPU tests of the oracle: pure-Python restatements and known-answer tests."""
import math

import numpy as np
import pytest
import scipy.fft as sfft

import oracle
from thcpp_gb300 import synth
from tests import kmeans_cases


def py_classify(pts, cen):
    """Loop restatement of classify_grid_points (src/kmeans.cpp:88-106)."""
    out = []
    for p in pts:
        best, arg = None, 0
        for j, c in enumerate(cen):
            dx, dy, dz = c[0] - p[0], c[1] - p[1], c[2] - p[2]
            d = math.sqrt((dx * dx + dy * dy) + dz * dz)
            if best is None or d < best:
                best, arg = d, j
        out.append(arg)
    return np.array(out)


def py_normed_difference(a, b):
    scale = max(abs(max(a)), abs(min(a))) + max(abs(max(b)), abs(min(b)))
    diff = 0.0
    for x, y in zip(a, b):
        q = (x - y) / scale
        diff += q * q
    return scale * math.sqrt(diff)


def py_kmeans(grid, rho, init, max_it, thr):
    """Single-rank loop restatement of KMeansSolver::kernel (src/kmeans.cpp:187-264)."""
    nmu = len(init)
    cur = [tuple(grid[i]) for i in init]
    lab = py_classify(grid, cur)
    diff = 0.0
    nxt = None
    conv = False
    for it in range(max_it):
        lab = py_classify(grid, cur)
        w = [0.0] * nmu
        s = [[0.0, 0.0, 0.0] for _ in range(nmu)]
        for i in range(len(grid)):
            k = lab[i]
            w[k] += rho[i]
            for d in range(3):
                s[k][d] += rho[i] * grid[i][d]
        if min(w) < 1e-8:
            return None
        nxt = [tuple(s[k][d] / w[k] for d in range(3)) for k in range(nmu)]
        diff = py_normed_difference([x for c in nxt for x in c], [x for c in cur for x in c])
        if diff < thr:
            conv = True
            break
        cur, nxt = nxt, cur
    fin = nxt if conv else cur
    idx = sorted(py_classify(np.array(fin), [tuple(g) for g in grid]))
    return np.array(idx), it + 1, diff


def test_sqrt_tie_keeps_first_index():
    v1, v2 = kmeans_cases.sqrt_tie_vectors()
    d1 = (v1[0] * v1[0] + v1[1] * v1[1]) + v1[2] * v1[2]
    d2 = (v2[0] * v2[0] + v2[1] * v2[1]) + v2[2] * v2[2]
    assert d2 < d1 and math.sqrt(d1) == math.sqrt(d2)
    lab = oracle.classify(np.zeros((1, 3)), np.array([v1, v2]))
    assert lab[0] == 0
    assert py_classify(np.zeros((1, 3)), [v1, v2])[0] == 0


def test_exact_ties_lowest_index():
    g, _ = kmeans_cases.exact_tie_grid()
    cen = np.array([[1.0, 1.0, 1.0], [3.0, 1.0, 1.0], [1.0, 3.0, 1.0], [3.0, 3.0, 3.0]])
    a = oracle.classify(g, cen)
    b = py_classify(g, cen)
    assert np.array_equal(a, b)
    # point (2,1,1) is exactly between centroids 0 and 1
    i = int(np.nonzero((g == [2.0, 1.0, 1.0]).all(1))[0][0])
    assert a[i] == 0


def test_initial_indices_sorted_unique():
    idx = oracle.initial_indices(13824, 64, 18)
    assert np.all(np.diff(idx) > 0) and idx.min() >= 0 and idx.max() < 13824


@pytest.mark.parametrize("seed", [0, 3, 11])
def test_kmeans_oracle_matches_python_loops(seed):
    rng = np.random.default_rng(seed)
    grid = rng.uniform(0, 4, size=(60, 3))
    rho = rng.uniform(0.1, 1.0, size=60)
    init = oracle.initial_indices(60, 5, seed)
    r = oracle.kmeans(grid, rho, 5, init, 30, 1e-9, nthreads=1)
    idx, it, diff = py_kmeans(grid, rho, init, 30, 1e-9)
    assert r.status == 0
    assert np.array_equal(r.idx, idx) and r.iters == it and r.diff == diff


def test_kmeans_oracle_threads_identical():
    s = synth.config("tiny")
    a = oracle.kmeans_system(s, nthreads=1)
    b = oracle.kmeans_system(s, nthreads=4)
    assert np.array_equal(a.idx, b.idx) and a.iters == b.iters and a.diff == b.diff


def test_kmeans_oracle_empty_cluster():
    grid = np.array([[0.0, 0, 0], [1.0, 0, 0], [5.0, 0, 0]])
    rho = np.array([1.0, 1.0, 0.0])          # cluster of point 2 gets zero weight
    r = oracle.kmeans(grid, rho, 3, np.array([0, 1, 2], np.int32), 5, 1e-9)
    assert r.status == 2


def test_normed_difference_known_answer():
    a = [1.0, 2.0, 3.0]
    b = [1.0, 2.0, 5.0]
    # scale = 3 + 5 = 8; diff = sqrt((2/8)^2) * 8 = 2
    assert py_normed_difference(a, b) == 2.0


def test_fft_delta_and_plane_wave():
    mesh = (6, 5, 8)
    f = np.zeros(mesh)
    f[0, 0, 0] = 1.0
    assert np.allclose(sfft.fftn(f), 1.0)
    k = (1, 2, 3)
    idx = np.indices(mesh)
    pw = np.exp(2j * np.pi * sum(k[d] * idx[d] / mesh[d] for d in range(3)))
    F = sfft.fftn(pw)                         # FFTW_FORWARD: exp(-i ...) kernel
    assert abs(F[k] - np.prod(mesh)) < 1e-9
    F[k] = 0
    assert np.abs(F).max() < 1e-9


def test_coulomb_plane_wave_energy():
    """sum_G v(G) |rho_hat|^2 = Omega * 4 pi / (2 |G0|^2) for rho = cos(G0 . r)."""
    s = synth.config("tiny")
    lat = s.lattice
    g0 = 2 * np.pi * np.linalg.inv(lat).T[0]       # b_0
    rho = np.cos(s.grid @ g0)
    rh = sfft.fftn(rho.reshape(s.mesh)).reshape(-1)
    e = np.sum(s.coulG * np.abs(rh) ** 2)
    expect = s.volume * 4 * np.pi / (2 * g0 @ g0)
    assert abs(e - expect) < 1e-10 * expect


def test_half_spectrum_matches_full_c2c_nonorthogonal():
    """The real-form M (R2C, v_sym / v_anti) equals the complex C2C sum for any v."""
    rng = np.random.default_rng(1)
    mesh = (6, 4, 6)
    lat = np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]]) * 2.0
    v = synth.coulomb_g(lat, mesh)
    dsym, danti = oracle.half_spectrum_weights(v, mesh)
    assert np.count_nonzero(danti) > 0
    z = rng.standard_normal((3, int(np.prod(mesh))))
    zh_full = sfft.fftn(z.reshape(3, *mesh), axes=(1, 2, 3)).reshape(3, -1)
    Mfull = (zh_full.conj() * v) @ zh_full.T
    zh = sfft.rfftn(z.reshape(3, *mesh), axes=(1, 2, 3)).reshape(3, -1)
    re, im = zh.real, zh.imag
    Mre = (re * dsym) @ re.T + (im * dsym) @ im.T
    Mim = (re * danti) @ im.T - (im * danti) @ re.T
    assert np.allclose(Mre + 1j * Mim, Mfull, rtol=1e-12, atol=1e-12 * np.abs(Mfull).max())


def test_isdf_forms_agree_full_rank():
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    a = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG)
    b = oracle.isdf_reference(s.phi, km.idx, s.mesh, s.coulG)
    rel = np.linalg.norm(a["M"] - b["M"]) / np.linalg.norm(b["M"])
    # QR and Cholesky solutions differ by ~cond(C) * 1e-16; this C has cond ~1.5e9.
    assert rel < 1e-7
    L = a["L"]
    assert np.linalg.norm(L @ L.conj().T - a["M"]) < 1e-12 * np.linalg.norm(a["M"])


def test_thc_reconstructs_pair_coulomb_rank_deficient():
    """C1 has N_mu = 64 > 36 pair products: C is singular, M is not unique, but the THC
    reconstruction of the orbital-pair Coulomb integrals is."""
    s = synth.config("c1")
    km = oracle.kmeans_system(s)
    pm = s.phi[km.idx]
    tr = np.trace((pm @ pm.T) ** 2) / s.nmu
    r = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG, shift=1e-10 * tr)
    pairs = [(i, j) for i in range(s.norb) for j in range(i, s.norb)]
    ex = oracle.pair_coulomb_exact(s.phi, s.mesh, s.coulG, pairs)
    th = oracle.thc_pair_coulomb(s.phi, km.idx, r["M"], pairs)
    assert np.linalg.norm(th - ex) / np.linalg.norm(ex) < 1e-5


def test_half_rotated_forms_agree():
    """Half-rotated M: the complex QR form (setup_CZt_half, forward and backward C2C FFTs,
    IVMG^T IVG) against the real Cholesky/R2C form, with half the orbitals occupied."""
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    po = s.phi[:, : s.norb // 2]
    a = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG, phi_occ=po)
    b = oracle.isdf_half_reference(s.phi, po, km.idx, s.mesh, s.coulG)
    # C_half has cond ~3e10 here: QR and Cholesky solutions differ by ~cond * 1e-16.
    assert np.linalg.norm(a["M"] - b) / np.linalg.norm(b) < 1e-6
    assert np.allclose(a["C"], a["C"].T, rtol=0, atol=0)
    assert np.linalg.eigvalsh(a["C"]).min() > 0


def test_half_rotated_all_occupied_is_plain():
    """With every orbital occupied the half-rotated products are P o P."""
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    a = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG, phi_occ=s.phi)
    b = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG)
    assert np.array_equal(a["C"], b["C"])
    assert np.linalg.norm(a["M"] - b["M"]) <= 1e-12 * np.linalg.norm(b["M"])


def _golden_qrcp():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "qrcp.npz"))


def test_qrcp_gram_matches_householder_golden():
    """The pivoted Cholesky of Z Z^T (the CUDA formulation) picks the pivots of the literal
    Householder QRCP of Z^T (fixtures from tests/golden/make_golden.py)."""
    g = _golden_qrcp()
    tiny = synth.config("tiny")
    c2 = synth.config("c2")
    cases = [(c2.phi, 256, None, "c2"), (tiny.phi, 48, None, "tiny"),
             (tiny.phi, 20, tiny.phi[:, : tiny.nocc], "tiny_half")]
    for phi, npts, po, key in cases:
        r = oracle.qrcp_gram(phi, npts, po)
        assert np.array_equal(r["order"], g[key + "_order"]), key
        d = g[key + "_diag"]
        assert np.max(np.abs(r["diag"] - d)) <= 1e-10 * d[0], key
        assert np.array_equal(r["idx"], np.sort(g[key + "_order"]))


def test_qrcp_literal_small_matches_gram():
    s = synth.config("tiny")
    a = oracle.qrcp_reference(s.phi, 48)
    b = oracle.qrcp_gram(s.phi, 48)
    assert np.array_equal(a["order"], b["order"])


def test_qrcp_half_row_layout():
    """setup_Z_half_matrix writes pair (i, k) to row i * N_occ + k: with N_o > N_occ later
    pairs overwrite earlier ones and the tail rows stay zero."""
    s = synth.config("tiny")
    po = s.phi[:, : s.nocc]
    ne, nb = po.shape[1], s.phi.shape[1]
    zt = oracle.z_transpose(s.phi, po)
    for i in range(ne - 1):
        for k in range(ne):
            assert np.array_equal(zt[i * ne + k], po[:, i] * s.phi[:, k])
    for k in range(nb):
        assert np.array_equal(zt[(ne - 1) * ne + k], po[:, ne - 1] * s.phi[:, k])
    assert not zt[(ne - 1) * ne + nb:].any()


def test_qrcp_all_pairs_matches_explicit():
    """The all-pairs option: Gram form against Householder QRCP of every (occ, orbital) row."""
    import scipy.linalg as sla
    s = synth.config("tiny")
    po = s.phi[:, : s.nocc]
    zt = np.einsum("gi,gk->ikg", po, s.phi).reshape(-1, s.ng)
    _, perm = sla.qr(zt, mode="r", pivoting=True)
    r = oracle.qrcp_gram(s.phi, 30, po, all_pairs=True)
    assert np.array_equal(r["order"], perm[:30])


def complex_orbitals(phi, seed=7):
    """Complex orbitals Phi A (A = I + 0.3 (R1 + i R2) / sqrt(N_o)): a genuinely complex
    P = Phi_mu^H Phi with the span of the real set."""
    rng = np.random.default_rng(seed)
    no = phi.shape[1]
    a = np.eye(no) + 0.3 * (rng.standard_normal((no, no)) + 1j * rng.standard_normal((no, no))) / np.sqrt(no)
    return phi @ a


def test_isdf_complex_forms_agree():
    """Complex orbitals: the real form (Z = |P|^2, Cholesky, R2C) against the literal complex
    QR form; and invariance of M under a unitary mixing of the orbitals."""
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    pc = complex_orbitals(s.phi)
    a = oracle.isdf_real(pc, km.idx, s.mesh, s.coulG)
    b = oracle.isdf_reference(pc, km.idx, s.mesh, s.coulG)
    assert np.linalg.norm(a["M"] - b["M"]) / np.linalg.norm(b["M"]) < 1e-7   # cond(C) 1.6e9
    rng = np.random.default_rng(3)
    u, _ = np.linalg.qr(rng.standard_normal((s.norb, s.norb))
                        + 1j * rng.standard_normal((s.norb, s.norb)))
    x = oracle.isdf_real(s.phi @ u, km.idx, s.mesh, s.coulG)
    r = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG)
    assert np.linalg.norm(x["M"] - r["M"]) / np.linalg.norm(r["M"]) < 1e-7


def test_qrcp_complex_forms_agree():
    """Complex orbitals: Householder QRCP of the rows conj(phi_i) phi_k against the pivoted
    Cholesky of |Phi^H Phi|^2."""
    s = synth.config("tiny")
    pc = complex_orbitals(s.phi)
    a = oracle.qrcp_reference(pc, 48)
    b = oracle.qrcp_gram(pc, 48)
    assert np.array_equal(a["order"], b["order"])
    assert np.max(np.abs(a["diag"] - b["diag"])) <= 1e-10 * a["diag"][0]


def test_refinement_closed_form():
    """k steps of iterative refinement of a shifted solve, zeta += (C + sI)^{-1}(Z - C zeta)
    from zeta_0 = (C + sI)^{-1} Z, equal X^T P X Z with X = L^{-1} (L L^T = C + sI) and
    P = sum_{j<=k} (s X X^T)^j -- the form the library evaluates (refine_polynomial)."""
    rng = np.random.default_rng(3)
    n = 40
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.logspace(0, -9, n)
    C = (q * lam) @ q.T
    Z = rng.standard_normal((n, 7))
    s = 1e-6
    L = np.linalg.cholesky(C + s * np.eye(n))
    X = np.linalg.inv(L)
    zeta = np.linalg.solve(C + s * np.eye(n), Z)
    for k in range(4):
        if k:
            zeta = zeta + np.linalg.solve(C + s * np.eye(n), Z - C @ zeta)
        G = s * X @ X.T
        P = sum(np.linalg.matrix_power(G, j) for j in range(k + 1))
        closed = X.T @ (P @ X) @ Z
        assert np.linalg.norm(closed - zeta) <= 1e-8 * np.linalg.norm(zeta)
        # Eigen form: filter 1 - (s / (lam + s))^(k+1) on 1 / lam.
        filt = (1 - (s / (lam + s)) ** (k + 1)) / lam
        assert np.allclose(q.T @ closed, filt[:, None] * (q.T @ Z), rtol=1e-6, atol=0)


def test_rsqrt_refinement_reaches_fp64():
    """The reciprocal square root of the diagonal Cholesky pivots (dense64.cu rsqrt_fast):
    an FP32 seed y0 refined once by the second-order binomial step
    y = y0 + y0 e (1/2 + 3/8 e), e = 1 - d y0^2 (FMAs as in the kernel), stays within 2 ulp
    of 1/sqrt(d) for seeds up to 8 FP32 ulps off, over the pivot range (d spans 1e-30..1e30,
    the kernel's FP32 seed range)."""
    import math
    from fractions import Fraction as F

    def fma(a, b, c):
        return float(F(a) * F(b) + F(c))

    rng = np.random.default_rng(9)
    worst = 0.0
    for d in np.concatenate([10.0 ** rng.uniform(-30, 30, 400), [1.0, 2.0, 0.5, 3.0]]):
        d = float(d)
        ref = 1.0 / math.sqrt(d)
        s32 = float(np.float32(ref))
        for k in (-8, -3, 0, 3, 8):
            y = float(np.float32(s32) + np.float32(k) * np.spacing(np.float32(s32)))
            e = fma(-(d * y), y, 1.0)
            out = fma(y * e, fma(0.375, e, 0.5), y)
            # exact 1/sqrt(d) to ~1e-30 through a Newton step in rationals
            r = F(ref)
            r = r * (F(3) - F(d) * r * r) / 2
            err = abs(F(out) - r) / r
            worst = max(worst, float(err))
    assert worst < 2 * 2.0 ** -52
