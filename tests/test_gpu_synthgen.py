"""GPU generator of the synthetic Gaussian basis (thc_synth_gaussian_basis) against the host
restatement synth.gaussian_sp_basis (FP64, numpy)."""
import numpy as np
import pytest

from thcpp_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_ctx_fp64):
    return gpu_ctx_fp64


@pytest.mark.parametrize("name", ["tiny", "c1", "c4_5"])
def test_basis_matches_host(ctx, name):
    import torch
    _, lat, atoms, mesh, norb, _, seed, _ = synth.config_args(name)
    alphas, _ = synth.draw_parameters(atoms, norb, seed)
    grid = synth.uniform_grid(lat, mesh)
    ref = synth.gaussian_sp_basis(grid, lat, atoms, alphas, norb)
    cen, cat, rcut = synth.image_centres(lat, atoms, alphas, norb)
    d_grid = torch.from_numpy(grid).cuda()
    out = torch.full((grid.shape[0], norb), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.gaussian_basis(d_grid, mesh, cen, cat, alphas, norb, rcut, out)
    got = out.cpu().numpy()
    # FP32 distances and expf: |error| <= ~4e-6 of the largest value (alpha r^2 <= 40).
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err


def test_device_system_matches_host(ctx):
    import torch
    host = synth.config("c1")
    dev = synth.config_gpu("c1", ctx, torch.device("cuda", 0))
    assert dev.mesh == host.mesh and dev.nmu == host.nmu and dev.norb == host.norb
    np.testing.assert_array_equal(dev.grid.cpu().numpy(), host.grid)
    np.testing.assert_array_equal(dev.coulG.cpu().numpy(), host.coulG)
    phi = dev.phi.cpu().numpy()
    assert np.abs(phi - host.phi).max() / np.abs(host.phi).max() < 1e-4
    rho = dev.density.cpu().numpy()
    assert np.abs(rho - host.density).max() / np.abs(host.density).max() < 1e-4
