"""The k-means oracle against the reference's OWN k-means (src/kmeans.cpp).

Live, where the reference tree is present: oracle/ref/Makefile compiles src/kmeans.cpp
unmodified (one-rank MPI stand-in, in-memory datasets) and the tests run its
KMeansSolver::kernel.  Everywhere: the restatement reproduces the fixtures that binary made
(tests/golden/ref_kmeans.npz, tests/golden/make_ref_golden.py) -- indices, the printed step
table (normed difference and percentage_change every 10 iterations, src/kmeans.cpp:238)
and whether the threshold was breached.
"""
import os

import numpy as np
import pytest

import oracle
from oracle import reference
from thcpp_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kmeans.npz")


def printed_steps_match(steps, diffs, pct):
    """Every (iteration, diff, pct) the reference printed with 6 significant digits equals
    the per-iteration value rounded the same way."""
    for it, d, p in np.asarray(steps).reshape(-1, 3):
        it = int(it)
        for ours, printed in ((diffs[it], d), (pct[it], p)):
            if "%.5e" % ours != "%.5e" % printed:
                return False
    return True


def _fixture():
    if not os.path.exists(GOLDEN):
        pytest.skip("tests/golden/ref_kmeans.npz not generated")
    return np.load(GOLDEN)


def _inputs(name):
    from tests.kmeans_cases import ref_case_inputs
    return ref_case_inputs(name)


def _oracle(name):
    g, r, no, cfac, mi, th, seed = _inputs(name)
    init = oracle.initial_indices(g.shape[0], no * cfac, seed)
    return oracle.kmeans(g, r, no * cfac, init, mi, th)


@pytest.mark.parametrize("name", ["tiny", "c1", "c2", "c4_0", "c4_1", "limit"])
def test_oracle_reproduces_reference_fixture(name):
    f = _fixture()
    o = _oracle(name)
    assert o.status == 0
    assert np.array_equal(o.idx, f[f"{name}_idx"])
    assert printed_steps_match(f[f"{name}_steps"], o.diffs, o.pct)
    assert (o.diff < _inputs(name)[5]) == bool(f[f"{name}_conv"])


@pytest.mark.skipif(not reference.available(), reason="reference tree not present")
@pytest.mark.parametrize("name", ["tiny", "c1"])
def test_oracle_matches_reference_live(name):
    """Run the reference's KMeansSolver now and compare with the restatement."""
    s = synth.config(name)
    ref = reference.kmeans_system(s)
    o = oracle.kmeans_system(s)
    assert np.array_equal(o.idx, ref.idx)
    assert len(ref.steps) == (o.iters + 9) // 10
    assert printed_steps_match(ref.steps, o.diffs, o.pct)
    assert ref.threshold_breached == (o.diff < s.threshold)


@pytest.mark.skipif(not reference.available(), reason="reference tree not present")
def test_reference_not_converged_maps_newest_centroids():
    """max_it reached without breaching the threshold: the reference maps its newest
    centroids (src/kmeans.cpp:250-257), as the restatement does."""
    s = synth.config("c1")
    ref = reference.kmeans(s.grid, s.density, s.norb, s.thc_cfac, 7, s.threshold,
                           s.rng_seed)
    init = oracle.initial_indices(s.ng, s.nmu, s.rng_seed)
    o = oracle.kmeans(s.grid, s.density, s.nmu, init, 7, s.threshold)
    assert not ref.threshold_breached and o.iters == 7
    assert np.array_equal(o.idx, ref.idx)
