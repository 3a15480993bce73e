"""thc_factorize_batched against one-at-a-time thc_kmeans + thc_isdf (the C4 workload)."""
import numpy as np
import pytest

from thcpp_gb300 import batch, capi, synth
from tests.conftest import system

pytestmark = pytest.mark.gpu

_C4 = {}


def c4(s):
    if s not in _C4:
        _C4[s] = synth.c4_system(s)
    return _C4[s]


@pytest.mark.parametrize("prec", [capi.THC_PREC_FP64, capi.THC_PREC_MIXED])
def test_batched_matches_sequential(prec):
    import torch
    systems = [system("tiny"), c4(0), c4(1)]
    dev = torch.device("cuda", 0)
    seq = [batch.system_arrays(s, dev) for s in systems]
    bat = [batch.system_arrays(s, dev) for s in systems]
    with capi.Context(0, prec) as ctx:
        st_seq = batch.run_sequential(ctx, systems, seq)
    st, st_bat = batch.run_batched(systems, bat, prec, nstreams=2)
    torch.cuda.synchronize()
    # THC_ERR_NOT_PD (the reference's Cholesky warning on M; L is still written) is a result,
    # not a failure: an M with eigenvalues below its mixed-precision error can report it.
    assert all(x in (capi.THC_OK, capi.THC_ERR_NOT_PD) for x in st_seq)
    assert st == capi.THC_OK and st_bat == st_seq
    for s, a, b in zip(systems, seq, bat):
        assert torch.equal(a["out_idx"], b["out_idx"]), s.name
        m_a, m_b = a["out_M"].cpu().numpy(), b["out_M"].cpu().numpy()
        d = np.linalg.norm(m_a - m_b) / np.linalg.norm(m_a)
        assert d <= 1e-12, (s.name, d)
        assert torch.equal(a["out_orbitals"], b["out_orbitals"]), s.name


def test_batched_reports_per_system_errors():
    """An empty cluster in one system fails that system only."""
    import torch
    good = system("tiny")
    dev = torch.device("cuda", 0)
    a_good = batch.system_arrays(good, dev)
    bad_s = synth.config("tiny")
    bad_s.density = np.zeros_like(bad_s.density)   # every centroid weight 0
    a_bad = batch.system_arrays(bad_s, dev)
    st, per = batch.run_batched([good, bad_s], [a_good, a_bad], capi.THC_PREC_MIXED, nstreams=2)
    assert per[0] == capi.THC_OK
    assert per[1] == capi.THC_ERR_EMPTY_CLUSTER
    assert st == capi.THC_ERR_EMPTY_CLUSTER
