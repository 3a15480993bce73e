"""Blocked FP64 GPU oracle of the ISDF path -- TEST INFRASTRUCTURE ONLY.

The real-arithmetic formulation of ``isdf.py:isdf_real`` (the restatement of
``src/interpolating_vectors.cpp:59-141,163-190,247-281,406-455`` the CUDA path implements),
written independently of the library in plain torch float64 (cuBLAS DGEMM, cuSOLVER
Cholesky, cuFFT D2Z through torch.fft) so that it reaches the sizes the CPU oracle cannot
(the 216-atom cell: N_g 1.26e6, N_mu 5184):

* C = (Phi_mu Phi_mu^T)^2 + shift I, its Cholesky factor L (one N_mu x N_mu FP64 solve);
* zeta^T = C^{-1} Z^T by triangular solves with L, one block of grid points at a time,
  Z^T of the block formed on the fly as (Phi_mu Phi_blk^T)^2: Z is never held whole; with a
  shift, optional steps of literal iterative refinement zeta += (C + sI)^{-1}(Z^T - C zeta);
* zeta_hat = D2Z FFT of the interpolating vectors, ``mu_block`` vectors at a time;
* M = sum_half w [v_sym Re(a) + i v_anti Im(a)], a = conj(zeta_hat_mu) zeta_hat_nu, as one
  FP64 product over the scaled half spectra.

It is checked against the CPU oracle on the smaller cells (``tests/test_gpu_accuracy.py``).
Only tests and the accuracy report under ``tests/`` use it.
"""

from __future__ import annotations

import numpy as np


def _t(a, device):
    import torch
    if isinstance(a, torch.Tensor):
        return a.to(device)
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def half_spectrum_weights(coulG, mesh, device):
    """w v_sym and w v_anti on the R2C half spectrum (n0, n1, n2//2+1), flattened."""
    import torch
    n0, n1, n2 = mesh
    nc = n2 // 2 + 1
    v = _t(coulG, device).reshape(n0, n1, n2).to(torch.float64)
    k0 = (-torch.arange(n0, device=device)) % n0
    k1 = (-torch.arange(n1, device=device)) % n1
    k2 = (-torch.arange(nc, device=device)) % n2
    vneg = v[k0][:, k1][:, :, k2]
    vpos = v[:, :, :nc]
    w = torch.full((nc,), 2.0, dtype=torch.float64, device=device)
    w[0] = 1.0
    if n2 % 2 == 0:
        w[-1] = 1.0
    dsym = (w * 0.5 * (vpos + vneg)).reshape(-1)
    danti = (w * 0.5 * (vpos - vneg)).reshape(-1)
    return dsym, danti


def isdf_real(phi, idx, mesh, coulG, shift: float = 0.0, device="cuda:0",
              grid_block: int = 1 << 16, mu_block: int = 256, keep_zeta: bool = True,
              refine: int = 0, shift_rel: float | None = None):
    """FP64 ISDF on the GPU.  ``shift`` is added to C's diagonal (absolute; or
    ``shift_rel`` tr(C)/N_mu).  ``refine`` steps of iterative refinement follow the shifted
    solve, literally: zeta <- zeta + (C + sI)^{-1} (Z^T - C zeta), per block of grid points.

    Returns dict(M (N_mu x N_mu complex128, host), L (host), C (device), zeta_t (device
    N_mu x N_g float64, when keep_zeta), cond_C, n_anti).
    """
    import torch
    phi = _t(phi, device).to(torch.float64)
    idx_t = _t(np.asarray(idx, np.int64), device)
    ng = phi.shape[0]
    n0, n1, n2 = mesh
    assert n0 * n1 * n2 == ng
    phimu = phi[idx_t]                                   # (N_mu, N_o)
    nmu = phimu.shape[0]
    C = (phimu @ phimu.T) ** 2
    ev = torch.linalg.eigvalsh(C)
    cond = float(ev[-1] / ev[0]) if float(ev[0]) > 0 else float("inf")
    if shift_rel is not None:
        shift = shift_rel * float(torch.trace(C)) / nmu
    Cs = C + shift * torch.eye(nmu, dtype=torch.float64, device=device)
    L = torch.linalg.cholesky(Cs)
    zt = torch.empty((nmu, ng), dtype=torch.float64, device=device)
    for g0 in range(0, ng, grid_block):
        g1 = min(ng, g0 + grid_block)
        zb = (phimu @ phi[g0:g1].T) ** 2                 # Z^T of the block (N_mu x b)
        x = torch.cholesky_solve(zb, L)
        for _ in range(refine):
            x = x + torch.cholesky_solve(zb - C @ x, L)
        zt[:, g0:g1] = x
        del zb, x
    dsym, danti = half_spectrum_weights(coulG, mesh, device)
    nc = dsym.numel()
    sq = torch.sqrt(torch.clamp(dsym, min=0.0))
    nz = torch.nonzero(danti).reshape(-1)
    # Scaled half spectra, [Re, Im] side by side: A A^T = sum w v_sym (re re^T + im im^T).
    A = torch.empty((nmu, 2 * nc), dtype=torch.float64, device=device)
    re_nz = torch.empty((nmu, nz.numel()), dtype=torch.float64, device=device)
    im_nz = torch.empty_like(re_nz)
    for m0 in range(0, nmu, mu_block):
        m1 = min(nmu, m0 + mu_block)
        zh = torch.fft.rfftn(zt[m0:m1].reshape(-1, n0, n1, n2), dim=(1, 2, 3)).reshape(m1 - m0, nc)
        A[m0:m1, :nc] = zh.real * sq
        A[m0:m1, nc:] = zh.imag * sq
        if nz.numel():
            re_nz[m0:m1] = zh.real[:, nz]
            im_nz[m0:m1] = zh.imag[:, nz]
        del zh
    if not keep_zeta:
        del zt
        zt = None
    Mre = A @ A.T
    del A
    if nz.numel():
        d = danti[nz]
        Mim = (re_nz * d) @ im_nz.T - (im_nz * d) @ re_nz.T
    else:
        Mim = torch.zeros_like(Mre)
    M = torch.complex(Mre, Mim)
    Lm = torch.linalg.cholesky_ex(M)[0]
    return dict(M=M.cpu().numpy(), L=Lm.cpu().numpy(), C=C, zeta_t=zt, cond_C=cond,
                n_anti=int(nz.numel()), shift=shift)


def pair_density_error(zeta_t, phi, idx, pairs, device="cuda:0", grid_block: int = 1 << 15):
    """Relative Frobenius error of the ISDF reconstruction of orbital-pair densities,
    rho_ij(r) = phi_i(r) phi_j(r) ~ sum_mu zeta_mu(r) phi_i(r_mu) phi_j(r_mu), over the
    given (i, j) pairs and every grid point."""
    import torch
    phi = _t(phi, device).to(torch.float64)
    zt = _t(zeta_t, device).to(torch.float64)
    pairs = np.asarray(pairs)
    pi = torch.from_numpy(pairs[:, 0].astype(np.int64)).to(device)
    pj = torch.from_numpy(pairs[:, 1].astype(np.int64)).to(device)
    pm = phi[_t(np.asarray(idx, np.int64), device)]
    X = pm[:, pi] * pm[:, pj]                            # (N_mu, pairs)
    num = torch.zeros((), dtype=torch.float64, device=device)
    den = torch.zeros((), dtype=torch.float64, device=device)
    ng = phi.shape[0]
    for g0 in range(0, ng, grid_block):
        g1 = min(ng, g0 + grid_block)
        rho = phi[g0:g1, pi] * phi[g0:g1, pj]
        rec = zt[:, g0:g1].T @ X
        num += ((rec - rho) ** 2).sum()
        den += (rho ** 2).sum()
    return float(torch.sqrt(num / den))


def sample_pairs(norb: int, count: int, seed: int = 7):
    """``count`` distinct orbital pairs i <= j (all of them when there are fewer)."""
    iu = np.stack(np.triu_indices(norb), axis=1)
    if iu.shape[0] <= count:
        return iu
    rng = np.random.default_rng(seed)
    return iu[np.sort(rng.choice(iu.shape[0], count, replace=False))]
