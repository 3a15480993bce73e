"""QRCP oracle: numpy/scipy restatements of QRCP::QRCPSolver (test infrastructure only).

The reference (``src/qrcp.cpp``) selects interpolating points by QR with column pivoting
of Z^T, one row per orbital pair and one column per grid point:

``qrcp_reference``  the literal form.  Z^T built as setup_Z_matrix (:34-49),
    [Z^T]_{(ik)a} = phi_i(r_a) phi_k(r_a) in row i * N_o + k, or as setup_Z_half_matrix
    (:50-67), phi_occ,i(r_a) phi_k(r_a) written to row i * N_occ + k in loop order (i outer,
    k inner), so that for N_o > N_occ a later pair overwrites an earlier one and the rows
    past (N_occ - 1) N_occ + N_o stay zero -- the matrix the reference factorises.  Then
    Householder QR with column pivoting (LAPACK dgeqp3 through scipy: the serial form of
    pzgeqpf, MatrixOperations::qrcp, src/matrix_operations.h:757-790, with the same rule:
    the column of largest partial norm).  Points: the first npts pivots, sorted (:149-160);
    |R_kk| is what the reference prints (:161-171).

``qrcp_gram``  the formulation the CUDA path implements: a pivoted Cholesky factorisation
    of the Gram matrix G = Z Z^T, evaluated column by column from the orbitals
    (G = (Phi Phi^T)^2, or the half-rotated row set's Gram matrix) without forming Z^T.
    Same pivots as QRCP in exact arithmetic (d_k(a) = squared residual norm of column a);
    ties go to the lowest grid index.

Complex orbitals: rows conj(phi_i) phi_k, Gram matrix |P|^2 with P = Phi^H Phi (real).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def z_transpose(phi: np.ndarray, phi_occ=None) -> np.ndarray:
    """Z^T exactly as the reference fills it (rows x N_g)."""
    if np.iscomplexobj(phi):
        phi = np.asarray(phi, np.complex128)
        ng, nb = phi.shape
        return np.ascontiguousarray(
            (phi.conj()[:, :, None] * phi[:, None, :]).reshape(ng, nb * nb).T)
    phi = np.asarray(phi, np.float64)
    ng, nb = phi.shape
    if phi_occ is None:
        return np.ascontiguousarray(
            (phi[:, :, None] * phi[:, None, :]).reshape(ng, nb * nb).T)
    po = np.asarray(phi_occ, np.float64)
    ne = po.shape[1]
    zt = np.zeros((nb * ne, ng))
    for i in range(ne):
        for k in range(nb):
            zt[i * ne + k] = po[:, i] * phi[:, k]
    return zt


def qrcp_reference(phi: np.ndarray, npts: int, phi_occ=None):
    """Literal form.  Returns dict(idx sorted, order, diag |R_kk| for npts steps)."""
    r, perm = sla.qr(z_transpose(phi, phi_occ), mode="r", pivoting=True)
    order = np.asarray(perm[:npts], np.int64)
    diag = np.abs(np.diag(r))[:npts]
    return dict(idx=np.sort(order).astype(np.int32), order=order, diag=diag)


def _gram_column(phi, po, p, kmin):
    if np.iscomplexobj(phi):
        g = phi.conj() @ phi[p]                  # P(a, p) = sum_k conj(phi_k(a)) phi_k(p)
        return g.real ** 2 + g.imag ** 2
    g3 = phi @ phi[p]
    if po is None:
        return g3 * g3
    if kmin == 0:
        return (po @ po[p]) * g3
    ne = po.shape[1]
    g1 = po[:, : ne - 1] @ po[p, : ne - 1]
    g2 = phi[:, :kmin] @ phi[p, :kmin]
    return g1 * g2 + po[:, ne - 1] * po[p, ne - 1] * g3


def _gram_diag(phi, po, kmin):
    if np.iscomplexobj(phi):
        return np.einsum("ij,ij->i", phi.conj(), phi).real ** 2
    g3 = np.einsum("ij,ij->i", phi, phi)
    if po is None:
        return g3 * g3
    if kmin == 0:
        return np.einsum("ij,ij->i", po, po) * g3
    ne = po.shape[1]
    g1 = np.einsum("ij,ij->i", po[:, : ne - 1], po[:, : ne - 1])
    g2 = np.einsum("ij,ij->i", phi[:, :kmin], phi[:, :kmin])
    return g1 * g2 + po[:, ne - 1] ** 2 * g3


def qrcp_gram(phi: np.ndarray, npts: int, phi_occ=None, all_pairs: bool = False):
    """Pivoted Cholesky of Z Z^T.  Returns dict(idx sorted, order, diag)."""
    phi = np.asarray(phi, np.complex128 if np.iscomplexobj(phi) else np.float64)
    po = None if phi_occ is None else np.asarray(phi_occ, np.float64)
    ng, nb = phi.shape
    kmin = nb if po is None else (0 if all_pairs else min(po.shape[1], nb))
    d = _gram_diag(phi, po, kmin)
    L = np.zeros((npts, ng))
    picked = np.zeros(ng, bool)
    order, diag = [], []
    for k in range(npts):
        p = int(np.argmax(np.where(picked, -np.inf, d)))    # first index among ties
        dp = d[p]
        order.append(p)
        diag.append(np.sqrt(max(dp, 0.0)))
        if dp > 0:
            c = _gram_column(phi, po, p, kmin) - L[:k].T @ L[:k, p]
            col = c / np.sqrt(dp)
        else:
            col = np.zeros(ng)
        col[picked] = 0.0
        col[p] = np.sqrt(max(dp, 0.0))
        L[k] = col
        d = d - col * col
        picked[p] = True
    order = np.asarray(order, np.int64)
    return dict(idx=np.sort(order).astype(np.int32), order=order, diag=np.asarray(diag))
