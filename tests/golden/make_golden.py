"""Regenerate the golden fixtures from the oracle (run from the repository root).

tiny.npz  k-means indices / iterations / final difference and the ISDF M, L of the
          'tiny' system (oracle: C++ k-means restatement + isdf_real).
c1_idx.npz the k-means indices of the 2-atom primitive cell (24^3, N_mu = 64).
qrcp.npz  QRCP pivots and |R_kk| from the literal oracle form (explicit Z^T, pivoted
          Householder QR): c2 (256 points of 1024 x 110,592), tiny (48 points) and the
          tiny half-rotated row set (20 points, below its numerical rank of ~27).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from thcpp_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    r = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG)
    np.savez_compressed(os.path.join(HERE, "tiny.npz"), idx=km.idx, iters=km.iters,
                        diff=km.diff, M=r["M"], L=r["L"])
    c1 = synth.config("c1")
    k1 = oracle.kmeans_system(c1)
    np.savez_compressed(os.path.join(HERE, "c1_idx.npz"), idx=k1.idx, iters=k1.iters,
                        diff=k1.diff)
    c2 = synth.config("c2")
    q2 = oracle.qrcp_reference(c2.phi, c2.nmu)
    qt = oracle.qrcp_reference(s.phi, s.nmu)
    qh = oracle.qrcp_reference(s.phi, 20, s.phi[:, : s.nocc])
    np.savez_compressed(os.path.join(HERE, "qrcp.npz"), c2_order=q2["order"],
                        c2_diag=q2["diag"], tiny_order=qt["order"], tiny_diag=qt["diag"],
                        tiny_half_order=qh["order"], tiny_half_diag=qh["diag"])


if __name__ == "__main__":
    main()
