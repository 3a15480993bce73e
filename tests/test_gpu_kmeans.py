"""GPU k-means through the C ABI: bit-identical to the oracle (one rank of the reference)."""
import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests import kmeans_cases
from tests.conftest import system

pytestmark = pytest.mark.gpu


def _ctx(request, prec):
    return request.getfixturevalue("gpu_ctx_fp64" if prec == "fp64" else "gpu_ctx_mixed")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["tiny", "c1", "c2"])
def test_kmeans_bit_exact(request, name, prec):
    s = system(name)
    ref = oracle.kmeans_system(s)
    ctx = _ctx(request, prec)
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    idx, st, status = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
    assert status == 0
    assert np.array_equal(idx, ref.idx)
    assert st.iterations == ref.iters
    assert st.final_diff == ref.diff          # bit-identical normed difference
    assert st.converged == (ref.diff < s.threshold)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_sqrt_tie(request, prec):
    grid, rho = kmeans_cases.sqrt_tie_grid()
    init = np.array([0, 1], np.int32)
    ref = oracle.kmeans(grid, rho, 2, init, 1, 0.0)
    idx, st, status = _ctx(request, prec).kmeans(grid, rho, 2, init, 1, 0.0)
    assert status == 0 and ref.status == 0
    assert np.array_equal(idx, ref.idx)
    assert list(idx) == [1, 2]                # P0 joined centroid 0 (first index)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_exact_ties(request, prec):
    g, rho = kmeans_cases.exact_tie_grid(8)
    init = oracle.initial_indices(g.shape[0], 12, 5)
    ref = oracle.kmeans(g, rho, 12, init, 50, 1e-12)
    idx, st, status = _ctx(request, prec).kmeans(g, rho, 12, init, 50, 1e-12)
    assert status == 0 and np.array_equal(idx, ref.idx) and st.iterations == ref.iters


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_rounding_stress(request, prec):
    g, rho = kmeans_cases.rounding_stress_grid()
    init = oracle.initial_indices(g.shape[0], 32, 3)
    ref = oracle.kmeans(g, rho, 32, init, 30, 1e-14)
    idx, st, status = _ctx(request, prec).kmeans(g, rho, 32, init, 30, 1e-14)
    assert status == 0 and ref.status == 0
    assert np.array_equal(idx, ref.idx) and st.iterations == ref.iters
    assert st.final_diff == ref.diff


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_context_reuse_across_sizes(request, prec):
    """One context, systems of different sizes in turn: workspace slots grow and move, and
    the cached iteration graph must follow them."""
    ctx = _ctx(request, prec)
    for name in ["tiny", "c1", "tiny", "c2", "c1", "tiny"]:
        s = system(name)
        ref = oracle.kmeans_system(s)
        init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
        idx, st, status = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
        assert status == 0 and np.array_equal(idx, ref.idx), name
        assert st.final_diff == ref.diff, name


_C4_4 = {}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_pruned_repeatable(request, prec):
    """A large cell with few, big clusters (C4 system 4: 157,464 points, 216 centroids),
    three runs in a row: identical to the oracle every time (the pruned assign's shared
    candidate list must be complete before any thread scans it)."""
    from thcpp_gb300 import synth
    if "s" not in _C4_4:
        _C4_4["s"] = synth.c4_system(4)
        _C4_4["ref"] = oracle.kmeans_system(_C4_4["s"])
    s, ref = _C4_4["s"], _C4_4["ref"]
    ctx = _ctx(request, prec)
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    for _ in range(3):
        idx, st, status = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
        assert status == 0 and np.array_equal(idx, ref.idx)
        assert st.iterations == ref.iters and st.final_diff == ref.diff


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_empty_cluster(request, prec):
    grid = np.array([[0.0, 0, 0], [1.0, 0, 0], [5.0, 0, 0]])
    rho = np.array([1.0, 1.0, 0.0])
    _, _, status = _ctx(request, prec).kmeans(grid, rho, 3, np.array([0, 1, 2], np.int32), 5,
                                               1e-9, raise_on_error=False)
    assert status == capi.THC_ERR_EMPTY_CLUSTER


def test_kmeans_zero_filled_when_diff_equals_threshold(gpu_ctx_fp64):
    s = system("tiny")
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    _, st, _ = gpu_ctx_fp64.kmeans(s.grid, s.density, s.nmu, init, 5, 0.0)
    d = st.final_diff
    ref = oracle.kmeans(s.grid, s.density, s.nmu, init, 5, d)
    idx, st2, status = gpu_ctx_fp64.kmeans(s.grid, s.density, s.nmu, init, 5, d)
    assert status == 0 and st2.zero_filled == 1
    assert np.array_equal(idx, ref.idx) and not idx.any()


def test_kmeans_device_pointers(gpu_ctx_mixed):
    import torch
    s = system("tiny")
    ref = oracle.kmeans_system(s)
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    g = torch.from_numpy(s.grid).cuda()
    r = torch.from_numpy(s.density).cuda()
    i0 = torch.from_numpy(init).cuda()
    out = torch.zeros(s.nmu, dtype=torch.int32, device="cuda")
    gpu_ctx_mixed.kmeans(g, r, s.nmu, i0, s.max_it, s.threshold, out_idx=out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref.idx)


def test_kmeans_argument_errors(gpu_ctx_fp64):
    s = system("tiny")
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    _, _, st = gpu_ctx_fp64.kmeans(s.grid, s.density, s.nmu, init, 0, 1e-6, raise_on_error=False)
    assert st == capi.THC_ERR_ARG


@pytest.mark.parametrize("prec", [capi.THC_PREC_FP64, capi.THC_PREC_MIXED])
@pytest.mark.parametrize("opts", [{"km_prune": 0}, {"graphs": 0}, {"km_prune": 0, "graphs": 0}])
def test_kmeans_options_identical(lib, prec, opts):
    """Pruned / exhaustive assignment and graph / eager launches give identical results."""
    s = system("c2")
    ref = oracle.kmeans_system(s)
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    with capi.Context(0, prec) as ctx:
        for k, v in opts.items():
            ctx.set_option(k, v)
        idx, st, status = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
    assert status == 0 and np.array_equal(idx, ref.idx) and st.final_diff == ref.diff


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kmeans_exact_ties_pruned(request, prec):
    """Integer lattice with 64 centroids (pruned path) and many exact ties."""
    g, rho = kmeans_cases.exact_tie_grid(12)
    init = oracle.initial_indices(g.shape[0], 64, 7)
    ref = oracle.kmeans(g, rho, 64, init, 40, 1e-12)
    idx, st, status = _ctx(request, prec).kmeans(g, rho, 64, init, 40, 1e-12)
    assert status == 0 and np.array_equal(idx, ref.idx) and st.iterations == ref.iters
