"""Regenerate the golden fixtures from the oracle (run from the repository root).

tiny.npz  k-means indices / iterations / final difference and the ISDF M, L of the
          'tiny' system (oracle: C++ k-means restatement + isdf_real).
c1_idx.npz the k-means indices of the 2-atom primitive cell (24^3, N_mu = 64).
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


if __name__ == "__main__":
    main()
