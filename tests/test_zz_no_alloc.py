"""thc_kmeans_noalloc (no device allocation) against thc_kmeans, through the C ABI.

Collected last on purpose: it must pass both alone in a fresh process and after every other
test has used the library.
"""
import numpy as np
import pytest

from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [capi.THC_PREC_FP64, capi.THC_PREC_MIXED])
@pytest.mark.parametrize("name", ["tiny", "c1"])
def test_noalloc_matches_kmeans_twice(name, prec):
    s = system(name)
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    with capi.Context(0, prec) as ctx:
        ref_idx, ref_st, _ = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
        for _ in range(2):   # the second call starts from the first call's leftover scratch
            idx, st, status = ctx.kmeans_noalloc(s.grid, s.density, s.nmu, init, s.max_it,
                                                 s.threshold)
            assert status == capi.THC_OK
            assert np.array_equal(idx, ref_idx)           # integer output: exact
            assert st.iterations == ref_st.iterations
            assert st.final_diff == ref_st.final_diff
            assert st.converged == ref_st.converged


def test_noalloc_device_pointers_twice():
    import torch
    s = system("c1")
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    with capi.Context(0, capi.THC_PREC_MIXED) as ctx:
        ref_idx, _, _ = ctx.kmeans(s.grid, s.density, s.nmu, init, s.max_it, s.threshold)
        g = torch.from_numpy(s.grid).cuda()
        r = torch.from_numpy(s.density).cuda()
        i0 = torch.from_numpy(init).cuda()
        for _ in range(2):
            out = torch.full((s.nmu,), -1, dtype=torch.int32, device="cuda")
            _, _, status = ctx.kmeans_noalloc(g, r, s.nmu, i0, s.max_it, s.threshold, out_idx=out)
            torch.cuda.synchronize()
            assert status == capi.THC_OK
            assert np.array_equal(out.cpu().numpy(), ref_idx)


@pytest.mark.parametrize("name", ["limit", "limit_full"])
def test_noalloc_at_its_limits_matches_the_reference(name):
    """N_g 65,536, N_mu 1,024, max_it 1,000 -- the largest sizes the fixed scratch takes --
    against the reference's own k-means (tests/golden/ref_kmeans.npz), and against
    thc_kmeans, twice in a row.  ``limit_full`` runs all 1,000 iterations."""
    import os
    from tests.kmeans_cases import ref_case_inputs
    g, r, no, cfac, mi, th, seed = ref_case_inputs(name)
    nmu = no * cfac
    assert (g.shape[0], nmu, mi) == (65536, 1024, 1000)
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                               "ref_kmeans.npz"))[f"{name}_idx"]
    init = capi.initial_indices(g.shape[0], nmu, seed)
    with capi.Context(0, capi.THC_PREC_MIXED) as ctx:
        base, base_st, _ = ctx.kmeans(g, r, nmu, init, mi, th)
        assert np.array_equal(base, ref)
        for _ in range(2):
            idx, st, status = ctx.kmeans_noalloc(g, r, nmu, init, mi, th)
            assert status == capi.THC_OK
            assert np.array_equal(idx, ref)
            assert st.iterations == base_st.iterations
            assert st.final_diff == base_st.final_diff


@pytest.mark.parametrize("prec", [capi.THC_PREC_FP64, capi.THC_PREC_MIXED])
def test_noalloc_allocates_no_device_memory(prec):
    """A call on a context that never ran thc_kmeans leaves the device's free memory as it
    was (device pointers in and out, so no staging either).  One earlier call on another
    context has already loaded the kernels and resolved the scratch array's address."""
    import torch
    s = system("c1")
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    g = torch.from_numpy(s.grid).cuda()
    r = torch.from_numpy(s.density).cuda()
    i0 = torch.from_numpy(init).cuda()
    out = torch.zeros(s.nmu, dtype=torch.int32, device="cuda")
    with capi.Context(0, prec) as warm:
        warm.kmeans_noalloc(g, r, s.nmu, i0, s.max_it, s.threshold, out_idx=out)
    torch.cuda.synchronize()
    with capi.Context(0, prec) as ctx:
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        _, _, status = ctx.kmeans_noalloc(g, r, s.nmu, i0, s.max_it, s.threshold, out_idx=out)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
    assert status == capi.THC_OK
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_the_scratch():
    ng = 65537
    grid = np.zeros((ng, 3))
    rho = np.ones(ng)
    init = np.arange(8, dtype=np.int32)
    with capi.Context(0, capi.THC_PREC_FP64) as ctx:
        _, _, status = ctx.kmeans_noalloc(grid, rho, 8, init, 10, 1e-6, raise_on_error=False)
        assert status == capi.THC_ERR_SHAPE
        _, _, status = ctx.kmeans_noalloc(grid[:1024], rho[:1024], 8, init, 1001, 1e-6,
                                          raise_on_error=False)
        assert status == capi.THC_ERR_SHAPE
        _, _, status = ctx.kmeans_noalloc(grid[:1024], rho[:1024], 1025,
                                          np.arange(1025, dtype=np.int32) % 1024, 10, 1e-6,
                                          raise_on_error=False)
        assert status == capi.THC_ERR_SHAPE
