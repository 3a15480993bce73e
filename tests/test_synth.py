"""Synthetic input contract (the orbital-file datasets of transform_basis.py)."""
import numpy as np

from thcpp_gb300 import synth
import oracle


def test_grid_order_c_order_n2_fastest():
    s = synth.config("tiny")
    n0, n1, n2 = s.mesh
    g = s.grid.reshape(n0, n1, n2, 3)
    a = s.lattice
    assert np.allclose(g[0, 0, 1], a[2] / n2)
    assert np.allclose(g[1, 0, 0], a[0] / n0)


def test_orbitals_orthonormal_and_density():
    s = synth.config("tiny")
    S = (s.volume / s.ng) * (s.phi.T @ s.phi)
    assert np.allclose(S, np.eye(s.norb), atol=1e-10)
    occ = s.phi[:, : s.nocc]
    assert np.allclose(s.density, np.einsum("ij,ij->i", occ, occ))
    assert (s.density >= 0).all()


def test_coulomb_cubic_is_even_and_fcc_is_not():
    s = synth.config("tiny")
    _, anti = oracle.half_spectrum_weights(s.coulG, s.mesh)
    assert not anti.any()
    assert s.coulG[0] == 0.0 and (s.coulG[1:] > 0).all()
    c1 = synth.config("c1")
    _, anti1 = oracle.half_spectrum_weights(c1.coulG, c1.mesh)
    assert anti1.any()


def test_config_sizes():
    s = synth.config("c1")
    assert (s.ng, s.norb, s.nmu) == (13824, 8, 64)


def test_seeded_reproducible():
    a = synth.config("tiny")
    b = synth.make_system("tiny", a.lattice, a.atoms, a.mesh, 12, 4, 1099, 99)
    assert np.array_equal(a.phi, b.phi)
