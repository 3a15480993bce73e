"""ISDF oracle: numpy/scipy restatements of IVecs (test infrastructure only).

Two formulations of the reference's interpolating-vector + Coulomb path
(``src/interpolating_vectors.cpp``):

``isdf_reference``  the literal single-rank form, complex128 throughout:
    P = Phi_mu^H Phi (setup_pseudo_dm, :59-125; pzgemm 'C','N' at :117),
    Z = P o conj(P) (setup_CZt, :127-141), C = Z[:, idx] (setup_CCt, :163-190),
    X = C^{-1} Z by Householder QR -- LAPACK zgels 'N', the serial form of pzgels
    (IVecs::kernel :416; matrix_operations.h:184-202), zeta = X^H (fft_vectors :343),
    per-column unnormalised forward C2C 3-D FFT (:371-392), scaling by sqrt(v(G))
    (construct_muv :258-263), M = zeta_hat^H zeta_hat (pzherk 'L','C', :278),
    L = zpotrf('L', M) (dump_thc_data :289), upper triangle zeroed (:307-312).

``isdf_real``  the same quantities for real orbitals in real arithmetic:
    C = (Phi_mu Phi_mu^T)^2, Cholesky of C (+ optional diagonal shift),
    zeta^T = C^{-1} Z^T, R2C FFT with half-spectrum weights, and
    M = sum_half w [v_sym Re(a) + i v_anti Im(a)] with a = conj(zh_mu) zh_nu, which equals
    the full C2C sum for any v (v_sym/v_anti are the even/odd parts of v under G -> -G).
    This is the formulation the CUDA path implements, so it is the parity target; it
    agrees with ``isdf_reference`` to ~1e-11 whenever C has full numerical rank.

``isdf_half_reference``  the half-rotated form (IVecs with rotate = true), complex128:
    P = Phi_mu^H Phi and P_occ = Phi_occ,mu^H Phi_occ (setup_pseudo_dm on aoR and aoR_half),
    Z = P_occ o conj(P) (setup_CZt_half, :143-161), C = Z[:, idx], X = C^{-1} Z by QR,
    zeta = X^H, forward and backward unnormalised C2C FFTs of every vector (fft_vectors
    :384-391), scaling by sqrt(v(G)), M = IVMG^T IVG (construct_muv :261-273, 'T','N'),
    written without a Cholesky factor as HalfTransformedMuv (dump_thc_data :317-328).
    ``isdf_real(..., phi_occ=...)`` is its real-arithmetic restatement: for real orbitals the
    backward transform is the conjugate of the forward one, so M_half has the form of M with
    Z = P_occ o P and C = (P_occ o P)[:, idx].

The pair-Coulomb helpers give an invariant check for rank-deficient C (where M is not
unique): the THC reconstruction X M X^T of the orbital-pair Coulomb integrals.
"""

from __future__ import annotations

import numpy as np
import scipy.fft as sfft
import scipy.linalg as sla
import scipy.linalg.lapack as lapack


def isdf_reference(phi: np.ndarray, idx: np.ndarray, mesh, coulG: np.ndarray, workers=-1):
    """Literal complex restatement.  Returns dict(M, L, info, zeta, cond)."""
    phi_c = np.asarray(phi).astype(np.complex128)
    idx = np.asarray(idx)
    ng = phi_c.shape[0]
    phimu = phi_c[idx]                                  # (N_mu, N_o)
    P = phimu.conj() @ phi_c.T                          # (N_mu, N_g)
    Z = P * P.conj()
    C = np.ascontiguousarray(Z[:, idx])                 # (N_mu, N_mu)
    _, x, info_ls = lapack.zgels(C, Z)                  # solves C X = Z
    X = x[: C.shape[1]]
    zeta = X.conj().T                                   # (N_g, N_mu)
    zh = sfft.fftn(zeta.T.reshape((-1,) + tuple(mesh)), axes=(1, 2, 3), workers=workers)
    zh = zh.reshape(zeta.shape[1], ng).T                # (N_g, N_mu)
    zh = zh * np.sqrt(np.asarray(coulG).reshape(-1))[:, None]
    M = zh.conj().T @ zh                                # herk, full Hermitian
    L, info = lapack.zpotrf(np.tril(M), lower=1, clean=1)
    return dict(M=M, L=np.tril(L), info=int(info), info_ls=int(info_ls), zeta=zeta, C=C)


def half_spectrum_weights(coulG: np.ndarray, mesh):
    """w * v_sym and w * v_anti on the R2C half spectrum (n0, n1, n2//2+1), flattened."""
    n0, n1, n2 = mesh
    nc = n2 // 2 + 1
    v = np.asarray(coulG).reshape(n0, n1, n2)
    k0 = (-np.arange(n0)) % n0
    k1 = (-np.arange(n1)) % n1
    k2 = (-np.arange(nc)) % n2
    vneg = v[k0][:, k1][:, :, k2]
    vpos = v[:, :, :nc]
    w = np.full(nc, 2.0)
    w[0] = 1.0
    if n2 % 2 == 0:
        w[-1] = 1.0
    dsym = (w[None, None, :] * 0.5 * (vpos + vneg)).reshape(-1)
    danti = (w[None, None, :] * 0.5 * (vpos - vneg)).reshape(-1)
    return dsym, danti


def isdf_real(phi: np.ndarray, idx: np.ndarray, mesh, coulG: np.ndarray, shift: float = 0.0,
              workers=-1, fft_dtype=np.float64, phi_occ=None, refine: int = 0):
    """Real-arithmetic formulation (the CUDA path's).  Returns dict(M, L, info, zeta, ...).

    ``shift`` is added to the diagonal of C before the Cholesky factorisation; ``refine``
    steps of iterative refinement zeta <- zeta + (C + sI)^{-1} (Z^T - C zeta) follow.  Complex
    ``phi`` (k-point orbitals) gives Z = |Phi_mu^H Phi|^2, still real.  With
    ``phi_occ`` (N_g x N_occ) the half-rotated products Z = P_occ o P, C = Z[:, idx] replace
    P o P (C stays symmetric positive semi-definite: a Schur product of two Gram matrices).
    """
    idx = np.asarray(idx)
    if np.iscomplexobj(phi):
        # Complex orbitals: P = Phi_mu^H Phi, Z = P o conj(P) = |P|^2 is real.
        phi = np.asarray(phi, np.complex128)
        ng = phi.shape[0]
        phimu = phi[idx]
        if phi_occ is not None:
            raise ValueError("the half-rotated form takes real orbitals")
        P = phimu.conj() @ phi.T
        Pc = phimu.conj() @ phimu.T
        Zt = P.real ** 2 + P.imag ** 2
        C = Pc.real ** 2 + Pc.imag ** 2
        phi_occ = False
    else:
        phi = np.asarray(phi, np.float64)
        ng = phi.shape[0]
        phimu = phi[idx]
    if phi_occ is False:
        pass
    elif phi_occ is None:
        Zt = (phimu @ phi.T) ** 2                       # (N_mu, N_g)
        C = (phimu @ phimu.T) ** 2
    else:
        po = np.asarray(phi_occ, np.float64)
        pomu = po[idx]
        Zt = (phimu @ phi.T) * (pomu @ po.T)
        C = (phimu @ phimu.T) * (pomu @ pomu.T)
    Cs = C + shift * np.eye(C.shape[0])
    Lc = np.linalg.cholesky(Cs)
    Cinv = sla.cho_solve((Lc, True), np.eye(C.shape[0]))
    zt = Cinv @ Zt                                      # zeta^T (N_mu, N_g)
    for _ in range(refine):
        zt = zt + Cinv @ (Zt - C @ zt)
    n0, n1, n2 = mesh
    zh = sfft.rfftn(zt.reshape(-1, n0, n1, n2).astype(fft_dtype), axes=(1, 2, 3),
                    workers=workers)
    zh = zh.reshape(zt.shape[0], -1).astype(np.complex128)
    dsym, danti = half_spectrum_weights(coulG, mesh)
    re = zh.real
    im = zh.imag
    Mre = (re * dsym) @ re.T + (im * dsym) @ im.T
    nz = np.nonzero(danti)[0]
    Mim = ((re[:, nz] * danti[nz]) @ im[:, nz].T) - ((im[:, nz] * danti[nz]) @ re[:, nz].T)
    M = Mre + 1j * Mim
    L, info = lapack.zpotrf(np.tril(M), lower=1, clean=1)
    return dict(M=M, L=np.tril(L), info=int(info), zeta_t=zt, C=C, Cinv=Cinv, zhat=zh,
                n_anti=int(nz.size))


def isdf_half_reference(phi: np.ndarray, phi_occ: np.ndarray, idx: np.ndarray, mesh,
                        coulG: np.ndarray):
    """Half-rotated M as the reference forms it (complex128; see the module docstring)."""
    phi = np.asarray(phi, np.complex128)
    po = np.asarray(phi_occ, np.complex128)
    idx = np.asarray(idx)
    ng = phi.shape[0]
    P = phi[idx].conj() @ phi.T                          # (N_mu, N_g)
    Pocc = po[idx].conj() @ po.T
    Z = Pocc * P.conj()
    C = Z[:, idx]
    X = np.linalg.lstsq(C, Z, rcond=None)[0]             # pzgels: least squares by QR
    zeta = X.conj()                                      # rows are the vectors zeta_mu(r)
    f = zeta.reshape((-1,) + tuple(mesh))
    ivg = sfft.fftn(f, axes=(1, 2, 3)).reshape(zeta.shape[0], -1)
    ivmg = sfft.ifftn(f, axes=(1, 2, 3), norm="forward").reshape(zeta.shape[0], -1)
    sq = np.sqrt(np.asarray(coulG, np.float64).reshape(-1))
    return (ivmg * sq) @ (ivg * sq).T


def pair_coulomb_exact(phi: np.ndarray, mesh, coulG: np.ndarray, pairs):
    """(ij|kl) = sum_G v(G) conj(rho_ij(G)) rho_kl(G) for rho_ij = phi_i phi_j (full C2C)."""
    rho = np.stack([phi[:, i] * phi[:, j] for i, j in pairs])
    rh = sfft.fftn(rho.reshape((-1,) + tuple(mesh)), axes=(1, 2, 3)).reshape(len(pairs), -1)
    v = np.asarray(coulG).reshape(-1)
    return (rh.conj() * v) @ rh.T


def thc_pair_coulomb(phi: np.ndarray, idx: np.ndarray, M: np.ndarray, pairs):
    """THC reconstruction X M X^T with X[ij, mu] = phi_i(r_mu) phi_j(r_mu)."""
    pm = phi[np.asarray(idx)]
    X = np.stack([pm[:, i] * pm[:, j] for i, j in pairs])
    return X @ M @ X.T
