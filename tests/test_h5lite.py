"""h5lite (the self-written HDF5 subset) round trips and reads libhdf5-written files."""
import os

import numpy as np
import pytest

from thcpp_gb300 import h5, synth


@pytest.fixture(scope="module", autouse=True)
def built(lib):
    from thcpp_gb300 import build
    build.build_host()


def test_round_trip_types(tmp_path):
    p = str(tmp_path / "t.h5")
    rng = np.random.default_rng(0)
    a = rng.standard_normal((5, 4, 2))
    b = np.arange(7, dtype=np.int32) - 3
    c = rng.standard_normal((6, 3)) + 1j * rng.standard_normal((6, 3))
    with h5.Writer(p) as w:
        w.write("/Hamiltonian/THC/Luv", a)
        w.write("/Hamiltonian/THC/InterpIndx", b)
        w.write("aoR", c)
    r = h5.Reader(p)
    assert np.array_equal(r.read("/Hamiltonian/THC/Luv"), a)
    assert np.array_equal(r.read("/Hamiltonian/THC/InterpIndx"), b)
    assert np.array_equal(r.read("aoR"), c)
    assert r.info("aoR") == (h5.KIND_COMPLEX, (6, 3))
    assert not r.exists("/nope")


def test_append_mode_keeps_datasets(tmp_path):
    p = str(tmp_path / "t.h5")
    with h5.Writer(p) as w:
        w.write("/Hamiltonian/hcore", np.ones((2, 2, 2)))
    with h5.Writer(p, truncate=False) as w:
        w.write("/Hamiltonian/dims", np.array([-1, 0, 0, 8, 4, 4, 0, 0], dtype=np.int32))
    r = h5.Reader(p)
    assert np.array_equal(r.read("/Hamiltonian/hcore"), np.ones((2, 2, 2)))
    assert list(r.read("/Hamiltonian/dims")) == [-1, 0, 0, 8, 4, 4, 0, 0]


def test_many_members_in_one_group(tmp_path):
    p = str(tmp_path / "t.h5")
    with h5.Writer(p) as w:
        for i in range(40):
            w.write(f"/g/d{i:02d}", np.full(3, float(i)))
    r = h5.Reader(p)
    assert r.read("/g/d37")[2] == 37.0


def test_orbital_file_contract(tmp_path):
    s = synth.config("tiny")
    p = str(tmp_path / "orb.h5")
    synth.write_orbital_file(s, p, half_rotate=True)
    r = h5.Reader(p)
    assert r.info("aoR") == (h5.KIND_COMPLEX, (s.ng, s.norb))
    assert np.array_equal(r.read("aoR").real, s.phi)
    assert np.array_equal(r.read("real_space_grid"), s.grid)
    assert np.array_equal(r.read("fft_coulomb").ravel(), s.coulG)
    assert r.read("fft_grid").ravel().tolist() == list(s.mesh)
    assert r.info("aoR_half")[1] == (s.ng, s.nocc)


def _reference_fixture():
    """The reference tree's HDF5 fixture (tests/data/eri_thc.h5), where the tree is present;
    its location is the one the reference build recipe (oracle/ref/Makefile) compiles from."""
    from oracle import reference
    try:
        return os.path.join(reference.reference_dir(), "tests", "data", "eri_thc.h5")
    except Exception:
        return ""


REF_FIXTURE = _reference_fixture()


@pytest.mark.skipif(not os.path.exists(REF_FIXTURE), reason="reference fixture not present")
def test_reads_libhdf5_fixture():
    """The reference's molecular fixture, written by libhdf5 (superblock v0)."""
    r = h5.Reader(REF_FIXTURE)
    hcore = r.read("hcore")
    assert hcore.shape == (10, 10)
    assert np.allclose(hcore, hcore.T)
    assert r.read("nelec").ravel().tolist()[0] == 5
    for name, shape in [("etaPm", (140, 10)), ("eri_df", (140, 100)), ("T", (140, 140))]:
        assert r.info(name)[1] == shape


_READ_ALL = r"""
import sys
sys.path.insert(0, {root!r})
from thcpp_gb300 import h5
try:
    r = h5.Reader({path!r})
    for name in ("real_space_grid", "aoR", "fft_coulomb", "fft_grid", "density_occ"):
        r.read(name)
    print("READ_OK")
except (OSError, KeyError) as e:
    print("READ_ERROR", e)
"""


def _read_in_child(path):
    """Read every dataset in a child process: a corrupt file must give an error, not a
    crash (a crash would end the child with a signal)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", _READ_ALL.format(root=root, path=path)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, (p.returncode, p.stderr[-500:])
    return p.stdout


def test_truncated_and_corrupt_orbital_files_raise(tmp_path):
    """Orbital files cut short at several offsets, or with bytes of the metadata overwritten,
    raise OSError/KeyError from the reader (the drop-in's THC_ERR_IO) instead of crashing."""
    s = synth.config("tiny")
    good = str(tmp_path / "orb.h5")
    synth.write_orbital_file(s, good)
    assert "READ_OK" in _read_in_child(good)
    data = open(good, "rb").read()
    rng = np.random.default_rng(5)
    cases = [data[:n] for n in (0, 7, 100, 600, len(data) // 3, len(data) - 9)]
    for _ in range(12):
        b = bytearray(data)
        off = int(rng.integers(0, 2048))               # superblock, object headers, B-trees
        b[off:off + 8] = bytes(rng.integers(0, 256, 8, dtype=np.uint8))
        cases.append(bytes(b))
    n_err = 0
    for k, blob in enumerate(cases):
        p = str(tmp_path / f"bad{k}.h5")
        open(p, "wb").write(blob)
        out = _read_in_child(p)
        assert "READ_OK" in out or "READ_ERROR" in out
        n_err += "READ_ERROR" in out
    assert n_err >= 6            # every truncation is an error; some flips hit only data
