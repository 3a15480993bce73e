"""Seeded synthetic ISDF systems: periodic Gaussian s/p orbitals on a real-space grid.

This restates, for a Gaussian basis instead of a pyscf SCF, the orbital-file contract
that ``tools/thcpy/thcpy/transform_basis.py:51-148`` (``write_orbitals``) defines for
thcpp's input:

* ``real_space_grid`` (N_g, 3): r = sum_i (n_i / N_i) a_i, C order over (n0, n1, n2) with
  n2 fastest, as pyscf's ``gen_uniform_grids`` orders it (``transform_basis.py:60``).
* ``aoR`` (N_g, N_o): orbitals on the grid (stored complex128 by the reference; the
  synthetic orbitals are real, so the imaginary part is exactly zero).
* ``density`` / ``density_occ`` (N_g, 1): sum_i |phi_i|^2, unnormalised
  (``transform_basis.py:125,131``).  Here the k-means weight is the occupied density
  sum_{i < N_o/2} |phi_i|^2.
* ``fft_grid`` (3, 1): the mesh.
* ``fft_coulomb`` (N_g, 1): ``get_coulG(cell, k=0) * Omega / N_g**2``
  (``transform_basis.py:64-67``) = 4 pi / |G|^2 * Omega / N_g^2 with G = 0 set to 0 and G
  taken on the ``fftfreq`` ordering of the mesh.
* ``hcore`` = 0 (N_o, N_o), ``num_electrons`` = (N_o/2, N_o/2),
  ``constant_energy_factors`` = 0.

Cells, basis and seeds (the workload definitions used by the tests and the benchmark):

* ``c1``: fcc primitive diamond cell, a = 6.74 bohr, vectors a/2 (0,1,1), (1,0,1), (1,1,0),
  atoms at 0 and a/4 (1,1,1); mesh 24^3; N_o = 8; N_mu = 8 N_o = 64.
* ``c2``: 8-atom cubic conventional diamond cell, a = 6.74; mesh 48^3; N_o = 32; N_mu = 256.
* ``c3``: 2x2x2 repeat of c2 (64 atoms); mesh 72^3; N_o = 256; N_mu = 2048.
* ``c5``: 3x3x3 repeat of c2 (216 atoms); mesh 108^3; N_o = 864; N_mu = 5184; half of
  the exponents redrawn from U[3, 6] so that C is near rank-deficient (cond 2.8e11).
* ``c4``: 48 random cubic cells (see :func:`c4_system`).

Per atom four functions s = exp(-a|r-R|^2) and p_x,y,z = (x-X) exp(-a|r-R|^2), each with
its own exponent a ~ U[0.3, 1.5] bohr^-2, periodised by summing lattice images within
|r - R - T| < sqrt(40 / a_min); mixed by a seeded standard-normal N_o x N_o matrix and
Loewdin-orthonormalised with S = (Omega/N_g) Phi^T Phi so that int |phi|^2 = 1.
Random draws come from ``numpy.random.default_rng(1000 + config number)`` in this order:
exponents (N_o), mixing matrix (N_o x N_o).  The k-means seed is 17 + config number.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

A_DIAMOND = 6.74

_DIAMOND_FRAC = np.array(
    [[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0],
     [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25]])


@dataclasses.dataclass
class System:
    """One ISDF input system: everything the reference reads from ``orbital_file``.

    Arrays are the in-memory form of the orbital-file datasets (C order).
    ``phi`` holds the real orbitals (the reference's complex ``aoR`` with zero imaginary
    part); ``density`` is the k-means weight named by ``density_label``.
    """
    name: str
    lattice: np.ndarray          # (3, 3) rows are a_0, a_1, a_2 (bohr)
    atoms: np.ndarray            # (n_atom, 3) Cartesian (bohr)
    mesh: tuple                  # (n0, n1, n2)
    grid: np.ndarray             # (N_g, 3) float64
    phi: np.ndarray              # (N_g, N_o) float64
    density: np.ndarray          # (N_g,) float64
    coulG: np.ndarray            # (N_g,) float64
    thc_cfac: int
    max_it: int = 100
    threshold: float = 1e-6
    rng_seed: int = 17
    density_label: str = "density_occ"

    @property
    def ng(self) -> int:
        return self.grid.shape[0]

    @property
    def norb(self) -> int:
        return self.phi.shape[1]

    @property
    def nmu(self) -> int:
        return self.thc_cfac * self.norb

    @property
    def volume(self) -> float:
        return float(abs(np.linalg.det(self.lattice)))

    @property
    def nocc(self) -> int:
        return self.norb // 2


def uniform_grid(lattice: np.ndarray, mesh) -> np.ndarray:
    """r = sum_i (n_i/N_i) a_i over the mesh in C order (n2 fastest)."""
    n0, n1, n2 = mesh
    f0 = np.arange(n0) / n0
    f1 = np.arange(n1) / n1
    f2 = np.arange(n2) / n2
    frac = np.stack(np.meshgrid(f0, f1, f2, indexing="ij"), axis=-1).reshape(-1, 3)
    return frac @ lattice


def coulomb_g(lattice: np.ndarray, mesh) -> np.ndarray:
    """4 pi / |G|^2 * Omega / N_g^2 on the fftfreq-ordered mesh, G = 0 -> 0."""
    recip = 2.0 * np.pi * np.linalg.inv(lattice).T      # rows b_i, a_i . b_j = 2 pi d_ij
    ks = [np.fft.fftfreq(n, 1.0 / n) for n in mesh]     # integer frequencies
    kk = np.stack(np.meshgrid(*ks, indexing="ij"), axis=-1).reshape(-1, 3)
    gv = kk @ recip
    g2 = np.einsum("ij,ij->i", gv, gv)
    ng = int(np.prod(mesh))
    vol = abs(np.linalg.det(lattice))
    v = np.zeros(ng)
    nz = g2 > 1e-12
    v[nz] = 4.0 * np.pi / g2[nz]
    return v * vol / ng**2


def _images(lattice: np.ndarray, rcut: float):
    """Lattice translations whose image can come within rcut of the home cell."""
    vol = abs(np.linalg.det(lattice))
    heights = [vol / np.linalg.norm(np.cross(lattice[(i + 1) % 3], lattice[(i + 2) % 3]))
               for i in range(3)]
    nmax = [int(math.ceil(rcut / h)) + 1 for h in heights]
    rng = [range(-n, n + 1) for n in nmax]
    out = []
    for i in rng[0]:
        for j in rng[1]:
            for k in rng[2]:
                out.append(i * lattice[0] + j * lattice[1] + k * lattice[2])
    return np.array(out)


def gaussian_sp_basis(grid, lattice, atoms, alphas, nfunc):
    """Periodised s/p Gaussians, atom-major (s, px, py, pz), first ``nfunc`` kept."""
    ng = grid.shape[0]
    phi = np.zeros((ng, nfunc))
    amin = float(np.min(alphas[:nfunc]))
    rcut = math.sqrt(40.0 / amin)
    trans = _images(lattice, rcut)
    # Bounding sphere of the home cell, used to drop images that never come within rcut.
    centre = 0.5 * lattice.sum(axis=0)
    corners = np.array([[i, j, k] for i in (0, 1) for j in (0, 1) for k in (0, 1)]) @ lattice
    cell_r = float(np.max(np.linalg.norm(corners - centre, axis=1)))
    chunk = 1 << 16
    natom = (nfunc + 3) // 4
    for a in range(natom):
        funcs = [f for f in range(4 * a, 4 * a + 4) if f < nfunc]
        for t in trans:
            pos = atoms[a] + t
            if np.linalg.norm(pos - centre) > cell_r + rcut:
                continue
            for s in range(0, ng, chunk):
                d = grid[s:s + chunk] - pos
                r2 = np.einsum("ij,ij->i", d, d)
                m = np.nonzero(r2 < rcut * rcut)[0]
                if m.size == 0:
                    continue
                r2m = r2[m]
                dm = d[m]
                for f in funcs:
                    g = np.exp(-alphas[f] * r2m)
                    kind = f % 4
                    if kind:
                        g *= dm[:, kind - 1]
                    phi[s + m, f] += g
    return phi


def loewdin(phi: np.ndarray, volume: float) -> np.ndarray:
    ng = phi.shape[0]
    s = (volume / ng) * (phi.T @ phi)
    w, u = np.linalg.eigh(s)
    return phi @ (u * (1.0 / np.sqrt(w))) @ u.T


# Cells whose interpolation matrix C is made near rank-deficient on purpose: a fraction of
# the basis functions gets tight exponents.  The 216-atom cell with every exponent in
# [0.3, 1.5] gives cond(C) 2.6e6; with half of them redrawn from [3, 6] cond(C) = 2.8e11
# (129 eigenvalues below 1e-8 tr(C)/N_mu), measured on the k-means points of the GPU path.
# (Broader functions do the opposite: [0.3, 0.5] for every function gives 3.9e3.)
_TIGHT = {"c5": (0.5, 3.0, 6.0)}


def draw_parameters(atoms, norb, seed, tight=None):
    """The seeded exponents (one per function, atom-major s, px, py, pz) and mixing matrix.

    ``tight`` = (fraction, lo, hi): that fraction of the exponents, chosen by
    ``default_rng(seed + 777)``, is redrawn from U[lo, hi] by the same generator."""
    rng = np.random.default_rng(seed)
    alphas = rng.uniform(0.3, 1.5, size=4 * atoms.shape[0])
    mix = rng.standard_normal((norb, norb))
    if tight is not None:
        frac, lo, hi = tight
        r2 = np.random.default_rng(seed + 777)
        n = alphas.size
        k = int(round(frac * n))
        sel = np.sort(r2.choice(n, k, replace=False))
        alphas = alphas.copy()
        alphas[sel] = r2.uniform(lo, hi, size=k)
    return alphas, mix


def image_centres(lattice, atoms, alphas, nfunc):
    """The atom + lattice-translation centres that gaussian_sp_basis sums over, grouped by
    atom (same filter), with their atom indices and the cutoff radius."""
    amin = float(np.min(alphas[:nfunc]))
    rcut = math.sqrt(40.0 / amin)
    trans = _images(lattice, rcut)
    centre = 0.5 * lattice.sum(axis=0)
    corners = np.array([[i, j, k] for i in (0, 1) for j in (0, 1) for k in (0, 1)]) @ lattice
    cell_r = float(np.max(np.linalg.norm(corners - centre, axis=1)))
    cen, cat = [], []
    for a in range((nfunc + 3) // 4):
        for t in trans:
            pos = atoms[a] + t
            if np.linalg.norm(pos - centre) > cell_r + rcut:
                continue
            cen.append(pos)
            cat.append(a)
    return (np.ascontiguousarray(np.array(cen, np.float64).reshape(-1, 3)),
            np.array(cat, np.int32), rcut)


def make_system(name, lattice, atoms, mesh, norb, cfac, seed, kmeans_seed,
                max_it=100, threshold=1e-6) -> System:
    alphas, mix = draw_parameters(atoms, norb, seed, _TIGHT.get(name))
    grid = uniform_grid(lattice, mesh)
    raw = gaussian_sp_basis(grid, lattice, atoms, alphas, norb)
    vol = abs(np.linalg.det(lattice))
    phi = loewdin(raw @ mix, vol)
    nocc = norb // 2
    dens = np.einsum("ij,ij->i", phi[:, :nocc], phi[:, :nocc])
    return System(name=name, lattice=lattice, atoms=atoms, mesh=tuple(int(m) for m in mesh),
                  grid=grid, phi=np.ascontiguousarray(phi), density=dens,
                  coulG=coulomb_g(lattice, mesh), thc_cfac=cfac, max_it=max_it,
                  threshold=threshold, rng_seed=kmeans_seed)


def diamond_supercell(rep: int):
    lat = A_DIAMOND * rep * np.eye(3)
    cells = [np.array([i, j, k]) for i in range(rep) for j in range(rep) for k in range(rep)]
    atoms = np.concatenate([(_DIAMOND_FRAC + c) * A_DIAMOND for c in cells])
    return lat, atoms


def config_args(name: str):
    """make_system arguments of the named workload ('c1', 'c2', 'c3', 'c5', 'tiny', 'c4_<s>')."""
    if name == "c1":
        a = A_DIAMOND
        lat = 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
        atoms = np.array([[0.0, 0.0, 0.0], [0.25 * a, 0.25 * a, 0.25 * a]])
        return ("c1", lat, atoms, (24, 24, 24), 8, 8, 1001, 18)
    if name == "c2":
        lat, atoms = diamond_supercell(1)
        return ("c2", lat, atoms, (48, 48, 48), 32, 8, 1002, 19)
    if name == "c3":
        lat, atoms = diamond_supercell(2)
        return ("c3", lat, atoms, (72, 72, 72), 256, 8, 1003, 20)
    if name == "c5":
        lat, atoms = diamond_supercell(3)
        return ("c5", lat, atoms, (108, 108, 108), 864, 6, 1005, 22)
    if name == "tiny":
        # A small cubic cell used by unit tests: 8 atoms, 16^3 mesh, N_o = 12, N_mu = 48.
        lat, atoms = diamond_supercell(1)
        return ("tiny", lat, atoms, (16, 16, 16), 12, 4, 1099, 99)
    if name.startswith("c4_"):
        return c4_args(int(name[3:]))
    raise KeyError(name)


def config(name: str) -> System:
    """The named workload: 'c1', 'c2', 'c3', 'c5' (and 'tiny' for unit tests)."""
    return make_system(*config_args(name))


_SMOOTH = sorted({2**a * 3**b * 5**c * 7**d for a in range(7) for b in range(4)
                  for c in range(3) for d in range(3)
                  if 32 <= 2**a * 3**b * 5**c * 7**d <= 64})


# The reference exits on an empty k-means cluster (centroid weight < 1e-8).  The batched
# workload keeps only systems whose k-means completes: the CPU restatement of the reference
# k-means was run on each system; systems 1 and 23 complete with k-means seed 23 instead of
# 21, and system 47 (a cell one third vacuum with N_mu = 132) empties a cluster for every
# seed tried (21..79), so it is redrawn with its second draw.
_C4_KMEANS_SEED = {1: 23, 23: 23}
_C4_REDRAW = {47: 1}


def c4_args(s: int):
    """make_system arguments of system ``s`` (0..47) of the batched workload.

    Cubic cell with edge L ~ U[6, 14] bohr; N_o ~ U{16..200}; ceil(N_o/4) atoms placed
    uniformly at random with minimum-image separation >= 2.5 bohr (L is redrawn when the
    atoms cannot be packed in 2000 attempts); mesh edge drawn from the 2,3,5,7-smooth
    values in [32, 64]; N_mu = N_o * U{6..10}.  Draws come from
    ``default_rng(4000 + s)`` in the order L, N_o, mesh, factor, positions, then the
    exponents and mixing matrix of :func:`make_system` from ``default_rng(5000 + s)``.
    """
    rng = np.random.default_rng(4000 + s + 100000 * _C4_REDRAW.get(s, 0))
    while True:
        edge = float(rng.uniform(6.0, 14.0))
        norb = int(rng.integers(16, 201))
        n = int(rng.choice(_SMOOTH))
        cfac = int(rng.integers(6, 11))
        natom = (norb + 3) // 4
        pos = []
        tries = 0
        while len(pos) < natom and tries < 2000:
            tries += 1
            p = rng.uniform(0.0, edge, size=3)
            ok = True
            for q in pos:
                d = p - q
                d -= edge * np.round(d / edge)
                if np.linalg.norm(d) < 2.5:
                    ok = False
                    break
            if ok:
                pos.append(p)
        if len(pos) == natom:
            break
    lat = edge * np.eye(3)
    return (f"c4_{s}", lat, np.array(pos), (n, n, n), norb, cfac,
            5000 + s + 100000 * _C4_REDRAW.get(s, 0), _C4_KMEANS_SEED.get(s, 17 + 4))


def c4_system(s: int) -> System:
    """System ``s`` (0..47) of the batched workload (see :func:`c4_args`)."""
    return make_system(*c4_args(s))


def write_orbital_file(system: System, path: str, half_rotate: bool = False) -> None:
    """Write ``system`` in the orbital-file layout of ``transform_basis.write_orbitals``.

    Datasets (``tools/thcpy/thcpy/transform_basis.py:74-95``): real_space_grid, kmesh,
    fft_grid (3, 1), hcore, constant_energy_factors (1, 1), num_electrons (1, 2),
    fft_coulomb (N_g, 1), density and density_occ (N_g, 1), aoR (N_g, N_o) complex128,
    aoR_half (N_g, nup) complex128.
    """
    from . import h5
    nup = system.nocc
    full = np.einsum("ij,ij->i", np.conj(system.phi), system.phi).real
    with h5.Writer(path, truncate=True) as w:
        w.write("real_space_grid", system.grid)
        w.write("kmesh", np.ones(3, dtype=np.int32))
        w.write("fft_grid", np.asarray(system.mesh, dtype=np.int32).reshape(3, 1))
        w.write("hcore", np.zeros((system.norb, system.norb), dtype=np.complex128))
        w.write("constant_energy_factors", np.zeros((1, 1)))
        w.write("num_electrons", np.array([[nup, nup]], dtype=np.int32))
        w.write("fft_coulomb", system.coulG.reshape(-1, 1))
        w.write("density", full.reshape(-1, 1))
        w.write("density_occ", system.density.reshape(-1, 1))
        w.write("aoR", system.phi.astype(np.complex128))
        if half_rotate:
            w.write("aoR_half", system.phi[:, :nup].astype(np.complex128))


def input_json(system: System, orbital_file: str, output_file: str, **gpu) -> dict:
    """The thcpp input JSON for ``system`` (keys of src/utils.h:73-113, src/kmeans.cpp:16-44)."""
    d = {"orbital_file": orbital_file, "output_file": output_file,
         "thc_cfac": system.thc_cfac,
         "interpolating_points": {"kmeans": {"max_it": system.max_it,
                                             "threshold": system.threshold,
                                             "rng_seed": system.rng_seed,
                                             "density": system.density_label}}}
    if gpu:
        d["gpu"] = gpu
    return d


@dataclasses.dataclass
class DeviceSystem:
    """A synthetic system generated on the GPU: grid, phi, density and coulG are device
    tensors (FP64); the other fields match :class:`System`."""
    name: str
    lattice: np.ndarray
    atoms: np.ndarray
    mesh: tuple
    grid: object
    phi: object
    density: object
    coulG: object
    thc_cfac: int
    max_it: int = 100
    threshold: float = 1e-6
    rng_seed: int = 17

    @property
    def ng(self) -> int:
        return int(self.grid.shape[0])

    @property
    def norb(self) -> int:
        return int(self.phi.shape[1])

    @property
    def nmu(self) -> int:
        return self.thc_cfac * self.norb


def make_system_gpu(name, lattice, atoms, mesh, norb, cfac, seed, kmeans_seed, ctx, device,
                    max_it=100, threshold=1e-6) -> DeviceSystem:
    """make_system with the basis evaluated on the GPU (thc_synth_gaussian_basis) and the
    mixing, Loewdin orthonormalisation and density formed there (FP64).  Same draws as
    make_system; orbitals agree with it to ~1e-6 relative (FP32 Gaussians)."""
    import torch
    alphas, mix = draw_parameters(atoms, norb, seed, _TIGHT.get(name))
    grid = uniform_grid(lattice, mesh)
    ng = grid.shape[0]
    cen, cat, rcut = image_centres(lattice, atoms, alphas, norb)
    d_grid = torch.from_numpy(grid).to(device)
    torch.cuda.synchronize(device)
    raw = torch.empty((ng, norb), dtype=torch.float64, device=device)
    ctx.gaussian_basis(d_grid, mesh, cen, cat, np.ascontiguousarray(alphas), norb, rcut, raw)
    phi0 = raw @ torch.from_numpy(mix).to(device)
    del raw
    vol = abs(np.linalg.det(lattice))
    s_mat = ((vol / ng) * (phi0.T @ phi0)).cpu().numpy()
    w, u = np.linalg.eigh(s_mat)
    phi = phi0 @ torch.from_numpy((u * (1.0 / np.sqrt(w))) @ u.T).to(device)
    del phi0
    nocc = norb // 2
    dens = (phi[:, :nocc] * phi[:, :nocc]).sum(dim=1)
    coul = torch.from_numpy(coulomb_g(lattice, mesh)).to(device)
    torch.cuda.synchronize(device)
    return DeviceSystem(name=name, lattice=lattice, atoms=atoms,
                        mesh=tuple(int(m) for m in mesh), grid=d_grid, phi=phi.contiguous(),
                        density=dens.contiguous(), coulG=coul, thc_cfac=cfac, max_it=max_it,
                        threshold=threshold, rng_seed=kmeans_seed)


def config_gpu(name: str, ctx, device) -> DeviceSystem:
    """The named workload generated on the GPU (see :func:`make_system_gpu`)."""
    return make_system_gpu(*config_args(name), ctx=ctx, device=device)
