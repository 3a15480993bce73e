"""Fixtures made by the reference's OWN k-means (run from the repository root).

Runs ``src/kmeans.cpp`` of the reference, compiled unmodified by ``oracle/ref/Makefile``
(``oracle/reference.py``), on the workloads below and stores what its
``KMeansSolver::kernel`` produced, so that machines without the reference tree (the GPU
tests) compare against the reference itself:

  <case>_idx     the interpolating-point indices (int32, sorted)
  <case>_steps   its printed step table: (iteration, normed difference, % changed) every
                 10 iterations, as printed with 6 significant digits (src/kmeans.cpp:238)
  <case>_conv    1 if the threshold was breached (converged), 0 otherwise

Cases: tiny, c1, c2, c3 (the seeded synthetic systems), c4_0 .. c4_3 (the first batched
systems), limit (N_g 65,536, N_mu 1,024, threshold 1e-6: the size limits of
thc_kmeans_noalloc) and limit_full (the same with a negative threshold, so that all 1,000
iterations run).  Takes ~15 minutes on 8 cores (c3 alone ~8).
"""
import concurrent.futures as cf
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import reference  # noqa: E402
from thcpp_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ref_kmeans.npz")


def run(name):
    from tests.kmeans_cases import ref_case_inputs
    g, r, no, cfac, mi, th, seed = ref_case_inputs(name)
    res = reference.kmeans(g, r, no, cfac, mi, th, seed)
    steps = np.array(res.steps, dtype=np.float64).reshape(-1, 3)
    return name, res.idx, steps, int(res.threshold_breached)


def main(names=None):
    names = names or ["tiny", "c1", "c2", "c3", "c4_0", "c4_1", "c4_2", "c4_3", "limit",
                      "limit_full"]
    reference.build()
    out = {}
    if os.path.exists(OUT):
        out.update(dict(np.load(OUT)))
    with cf.ProcessPoolExecutor(max_workers=os.cpu_count(),
                                mp_context=__import__("multiprocessing").get_context("spawn")) as ex:
        for name, idx, steps, conv in ex.map(run, names):
            out[f"{name}_idx"] = idx
            out[f"{name}_steps"] = steps
            out[f"{name}_conv"] = np.int32(conv)
            print(name, len(idx), "points,", len(steps), "printed steps, converged", conv,
                  flush=True)
    np.savez_compressed(OUT, **out)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
