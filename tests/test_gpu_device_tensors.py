"""The Python binding and the C ABI with device-resident (torch CUDA) inputs and outputs.

Every entry point takes host or device pointers; these tests feed CUDA tensors to the
wrappers that used to inspect their inputs with numpy (qrcp, isdf_complex), to isdf_half,
and device output buffers to thc_qrcp, and compare with the host-array calls.
"""
import ctypes

import numpy as np
import pytest

import oracle
from thcpp_gb300 import capi
from tests.conftest import system

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_qrcp_device_tensor_input(gpu_ctx_fp64, gpu_ctx_mixed, prec):
    ctx = gpu_ctx_fp64 if prec == "fp64" else gpu_ctx_mixed
    s = system("c2")
    host = ctx.qrcp(s.phi, 256)
    dev = ctx.qrcp(_dev(s.phi), 256)
    assert np.array_equal(dev["order"], host["order"])
    assert np.array_equal(dev["idx"], host["idx"])
    assert np.array_equal(dev["diag"], host["diag"])


def test_qrcp_complex_device_tensor_input(gpu_ctx_fp64):
    from tests.test_oracle import complex_orbitals
    s = system("tiny")
    pc = complex_orbitals(s.phi)
    host = gpu_ctx_fp64.qrcp(pc, 48)
    dev = gpu_ctx_fp64.qrcp(_dev(pc), 48)
    assert np.array_equal(dev["order"], host["order"])
    assert np.array_equal(dev["diag"], host["diag"])


def test_qrcp_device_outputs(gpu_ctx_fp64):
    """Device output pointers are written on the context's stream before the call returns."""
    import torch
    s = system("c2")
    host = gpu_ctx_fp64.qrcp(s.phi, 256)
    lib = capi.load()
    d_idx = torch.full((256,), -7, dtype=torch.int32, device="cuda:0")
    d_order = torch.full((256,), -7, dtype=torch.int32, device="cuda:0")
    d_diag = torch.full((256,), -7.0, dtype=torch.float64, device="cuda:0")
    st = lib.thc_qrcp(gpu_ctx_fp64.h, capi._ptr(_dev(s.phi)), s.ng, s.norb, None, 0, 256,
                      capi._ptr(d_idx), capi._ptr(d_order), capi._ptr(d_diag),
                      ctypes.byref(capi.QrcpStats()))
    assert st == capi.THC_OK
    # Read back on a different (torch's) stream: the call has already completed the copies.
    assert np.array_equal(d_order.cpu().numpy(), host["order"])
    assert np.array_equal(d_idx.cpu().numpy(), host["idx"])
    assert np.array_equal(d_diag.cpu().numpy(), host["diag"])


def test_qrcp_nan_orbitals_reported_and_context_reusable(gpu_ctx_fp64):
    """Orbitals with a NaN column leave no finite residual to pivot on after the first
    steps: the call reports THC_ERR_ARG, and the next call on the context is unaffected."""
    s = system("tiny")
    bad = s.phi.copy()
    bad[:, 3] = np.nan
    with pytest.raises(capi.ThcError) as e:
        gpu_ctx_fp64.qrcp(bad, 20)
    assert e.value.status == capi.THC_ERR_ARG
    r = gpu_ctx_fp64.qrcp(s.phi, 48)
    ref = oracle.qrcp_gram(s.phi, 48)
    assert np.max(np.abs(r["diag"] - ref["diag"])) <= 1e-10 * ref["diag"][0]


def test_isdf_complex_device_tensor_input(gpu_ctx_fp64):
    import torch
    from tests.test_oracle import complex_orbitals
    s = system("tiny")
    idx = oracle.kmeans_system(s).idx
    pc = complex_orbitals(s.phi)
    host = gpu_ctx_fp64.isdf_complex(pc, idx, s.mesh, s.coulG)
    dev = gpu_ctx_fp64.isdf_complex(_dev(pc), _dev(idx), s.mesh, _dev(s.coulG))
    assert dev["status"] == host["status"] == 0
    assert dev["M"].dtype == np.float64 and torch.is_tensor(pc) is False
    assert np.array_equal(dev["M"], host["M"])
    assert np.array_equal(dev["orbitals"], host["orbitals"])


def test_isdf_half_device_tensor_input(gpu_ctx_fp64):
    s = system("tiny")
    idx = oracle.kmeans_system(s).idx
    po = np.ascontiguousarray(s.phi[:, : s.nocc])
    host = gpu_ctx_fp64.isdf_half(s.phi, po, idx, s.mesh, s.coulG)
    dev = gpu_ctx_fp64.isdf_half(_dev(s.phi), _dev(po), _dev(idx), s.mesh, _dev(s.coulG))
    assert np.array_equal(dev["M"], host["M"])
    assert np.array_equal(dev["occ_orbitals"], host["occ_orbitals"])
