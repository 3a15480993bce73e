"""The drop-in C++ driver (thcpp_gb300.x: IPoints -> IVecs -> dump_qmcpack_data) end to end."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
from thcpp_gb300 import build, capi, h5, synth
from tests.conftest import system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_driver_tiny(tmp_path, lib, precision):
    build.build_host()
    s = system("tiny")
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(s, orb)
    inp = tmp_path / "input.json"
    inp.write_text(json.dumps(synth.input_json(s, orb, out, precision=precision)))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Finding interpolation points using K-Means" in r.stdout
    ref = oracle.kmeans_system(s)
    f = h5.Reader(out)
    idx = f.read("/Hamiltonian/THC/InterpIndx")
    assert np.array_equal(idx, ref.idx)
    orbs = f.read("/Hamiltonian/THC/Orbitals")
    assert orbs.shape == (s.norb, s.nmu, 2)
    assert np.array_equal(orbs[..., 0], s.phi[ref.idx].T) and not orbs[..., 1].any()
    L = f.read("/Hamiltonian/THC/Luv")
    assert L.shape == (s.nmu, s.nmu, 2)
    Lc = L[..., 0] + 1j * L[..., 1]
    assert np.allclose(np.triu(Lc, 1), 0)
    isd = oracle.isdf_real(s.phi, ref.idx, s.mesh, s.coulG)
    M = Lc @ Lc.conj().T
    assert np.linalg.norm(M - isd["M"]) / np.linalg.norm(isd["M"]) < 1e-6
    assert f.read("/Hamiltonian/THC/dims").tolist() == [s.norb, s.nmu, s.nmu]
    assert f.read("/Hamiltonian/dims").tolist() == [-1, 0, 0, s.norb, s.nocc, s.nocc, 0, 0]
    assert f.read("/Hamiltonian/occups").tolist() == [0] * (2 * s.nocc)
    assert f.read("/Hamiltonian/hcore").shape == (s.norb, s.norb, 2)
    assert f.read("/Hamiltonian/Energies").shape == (1,)


def test_driver_half_rotated(tmp_path, lib):
    """half_rotated with thc_half_cfac != thc_cfac (src/main.cpp:53-72): the plain pass
    (Orbitals, InterpIndx, Luv), new k-means points for the half pass, then
    HalfTransformed{Full,Occ}{Orbitals,InterpIndx} and HalfTransformedMuv."""
    build.build_host()
    s = system("tiny")
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(s, orb, half_rotate=True)
    inp = tmp_path / "input.json"
    d = synth.input_json(s, orb, out)
    d["half_rotated"] = True
    d["thc_half_cfac"] = 2
    inp.write_text(json.dumps(d))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    f = h5.Reader(out)
    ref = oracle.kmeans_system(s)
    assert np.array_equal(f.read("/Hamiltonian/THC/InterpIndx"), ref.idx)
    assert f.read("/Hamiltonian/THC/Luv").shape == (s.nmu, s.nmu, 2)
    hs = synth.System(**{**s.__dict__, "thc_cfac": 2})
    href = oracle.kmeans_system(hs)
    po = s.phi[:, : s.nocc]
    for part, src in (("Full", s.phi), ("Occ", po)):
        idx = f.read(f"/Hamiltonian/THC/HalfTransformed{part}InterpIndx")
        assert np.array_equal(idx, href.idx)
        o = f.read(f"/Hamiltonian/THC/HalfTransformed{part}Orbitals")
        assert o.shape == (src.shape[1], hs.nmu, 2)
        assert np.array_equal(o[..., 0], src[href.idx].T) and not o[..., 1].any()
    M = f.read("/Hamiltonian/THC/HalfTransformedMuv")
    M = M[..., 0] + 1j * M[..., 1]
    isd = oracle.isdf_real(s.phi, href.idx, s.mesh, s.coulG, phi_occ=po)
    assert np.linalg.norm(M - isd["M"]) / np.linalg.norm(isd["M"]) < 1e-8
    assert f.read("/Hamiltonian/THC/dims").tolist() == [s.norb, s.nmu, hs.nmu]


def test_driver_qrcp(tmp_path, lib, gpu_ctx_fp64):
    """"interpolating_points": {"qrcp": {}} selects QRCPSolver (src/interpolating_points.cpp:
    43-50): the QRCP points, then the ISDF pass on them."""
    build.build_host()
    s = system("tiny")
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(s, orb)
    inp = tmp_path / "input.json"
    d = synth.input_json(s, orb, out)
    d["interpolating_points"] = {"qrcp": {}}
    inp.write_text(json.dumps(d))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Using QRCP solver" in r.stdout and "full_ix_diag 47 " in r.stdout
    f = h5.Reader(out)
    idx = f.read("/Hamiltonian/THC/InterpIndx")
    assert np.array_equal(idx, gpu_ctx_fp64.qrcp(s.phi, s.nmu)["idx"])
    L = f.read("/Hamiltonian/THC/Luv")
    Lc = L[..., 0] + 1j * L[..., 1]
    isd = oracle.isdf_real(s.phi, idx, s.mesh, s.coulG)
    assert np.linalg.norm(Lc @ Lc.conj().T - isd["M"]) / np.linalg.norm(isd["M"]) < 1e-6


def test_driver_complex_orbitals(tmp_path, lib):
    """A complex aoR (k-point orbitals) runs thc_isdf_complex; Orbitals keep the imaginary
    parts."""
    from tests.test_oracle import complex_orbitals
    build.build_host()
    s = system("tiny")
    pc = complex_orbitals(s.phi)
    z = synth.System(**{**s.__dict__, "phi": pc})
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(z, orb)
    inp = tmp_path / "input.json"
    inp.write_text(json.dumps(synth.input_json(z, orb, out)))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = oracle.kmeans_system(s)
    f = h5.Reader(out)
    assert np.array_equal(f.read("/Hamiltonian/THC/InterpIndx"), ref.idx)
    o = f.read("/Hamiltonian/THC/Orbitals")
    assert np.array_equal(o[..., 0] + 1j * o[..., 1], pc[ref.idx].T)
    L = f.read("/Hamiltonian/THC/Luv")
    Lc = L[..., 0] + 1j * L[..., 1]
    isd = oracle.isdf_real(pc, ref.idx, s.mesh, s.coulG)
    assert np.linalg.norm(Lc @ Lc.conj().T - isd["M"]) / np.linalg.norm(isd["M"]) < 1e-6


def test_driver_qrcp_complex(tmp_path, lib, gpu_ctx_fp64):
    """QRCP points and the ISDF pass on a complex orbital file."""
    from tests.test_oracle import complex_orbitals
    build.build_host()
    s = system("tiny")
    pc = complex_orbitals(s.phi)
    z = synth.System(**{**s.__dict__, "phi": pc})
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(z, orb)
    inp = tmp_path / "input.json"
    d = synth.input_json(z, orb, out)
    d["interpolating_points"] = {"qrcp": {}}
    inp.write_text(json.dumps(d))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    f = h5.Reader(out)
    idx = f.read("/Hamiltonian/THC/InterpIndx")
    assert np.array_equal(idx, oracle.qrcp_gram(pc, s.nmu)["idx"])
    L = f.read("/Hamiltonian/THC/Luv")
    Lc = L[..., 0] + 1j * L[..., 1]
    isd = oracle.isdf_real(pc, idx, s.mesh, s.coulG)
    assert np.linalg.norm(Lc @ Lc.conj().T - isd["M"]) / np.linalg.norm(isd["M"]) < 1e-6


def test_driver_empty_cluster_exits(tmp_path, lib):
    """Reference behaviour: CRITICAL ERROR message and exit(1) (src/kmeans.cpp:137-143)."""
    s = system("tiny")
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    # zero density everywhere -> every cluster weight falls below 1e-8
    z = synth.System(**{**s.__dict__, "density": np.zeros_like(s.density)})
    synth.write_orbital_file(z, orb)
    inp = tmp_path / "input.json"
    inp.write_text(json.dumps(synth.input_json(z, orb, out)))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 1
    assert "CRITICAL ERROR: Found centroid with weight ~ 0" in r.stdout


def test_driver_half_rotated_complex(tmp_path, lib):
    """half_rotated on a complex orbital file: the half pass runs thc_isdf_half_complex and
    HalfTransformedMuv matches the oracle's literal complex half-rotated form."""
    from tests.test_oracle import complex_orbitals
    build.build_host()
    s = system("tiny")
    pc = complex_orbitals(s.phi)
    z = synth.System(**{**s.__dict__, "phi": pc})
    orb = str(tmp_path / "orbitals.h5")
    out = str(tmp_path / "thc.h5")
    synth.write_orbital_file(z, orb, half_rotate=True)
    inp = tmp_path / "input.json"
    d = synth.input_json(z, orb, out)
    d["half_rotated"] = True
    d["thc_half_cfac"] = 2
    inp.write_text(json.dumps(d))
    r = subprocess.run([build.DRIVER, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    f = h5.Reader(out)
    hs = synth.System(**{**s.__dict__, "thc_cfac": 2})
    href = oracle.kmeans_system(hs)
    po = pc[:, : s.nocc]
    for part, src in (("Full", pc), ("Occ", po)):
        assert np.array_equal(f.read(f"/Hamiltonian/THC/HalfTransformed{part}InterpIndx"), href.idx)
        o = f.read(f"/Hamiltonian/THC/HalfTransformed{part}Orbitals")
        assert np.array_equal(o[..., 0] + 1j * o[..., 1], src[href.idx].T)
    M = f.read("/Hamiltonian/THC/HalfTransformedMuv")
    M = M[..., 0] + 1j * M[..., 1]
    ref = oracle.isdf_half_reference(pc, po, href.idx, s.mesh, s.coulG)
    assert np.linalg.norm(M - ref) / np.linalg.norm(ref) < 1e-6
