"""GPU k-means against the reference's OWN k-means (src/kmeans.cpp, built unmodified from
the reference tree), through the fixtures that binary generated
(tests/golden/ref_kmeans.npz, tests/golden/make_ref_golden.py).

Bit-exact: the interpolating-point indices, and every normed difference and
percentage_change (src/kmeans.cpp:177-185) the reference printed (every 10 iterations, 6
significant digits), in both precisions.
"""
import os

import numpy as np
import pytest

from thcpp_gb300 import capi
from tests.kmeans_cases import ref_case_inputs
from tests.test_reference_pinned import printed_steps_match

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kmeans.npz")
CASES = ["tiny", "c1", "c2", "c3", "c4_0", "c4_1", "c4_2", "c4_3", "limit", "limit_full"]


@pytest.fixture(scope="module")
def fixture():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_matches_reference(gpu_ctx_fp64, gpu_ctx_mixed, fixture, prec, name):
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    g, r, no, cfac, mi, th, seed = ref_case_inputs(name)
    nmu = no * cfac
    init = capi.initial_indices(g.shape[0], nmu, seed)
    idx, st, status = ctx.kmeans(g, r, nmu, init, mi, th)
    assert status == capi.THC_OK
    assert np.array_equal(idx, fixture[f"{name}_idx"])
    assert bool(st.converged) == bool(fixture[f"{name}_conv"])
    diffs, pct = ctx.kmeans_history(st.iterations)
    steps = fixture[f"{name}_steps"]
    assert len(steps) == (st.iterations + 9) // 10
    assert printed_steps_match(steps, diffs, pct)
