"""Hand-made k-means inputs with constructed ties (shared by CPU and GPU tests)."""
import math

import numpy as np


def sqrt_tie_vectors(s=1.3):
    """Two offsets v1, v2 with d2(v2) < d2(v1) but sqrt(d2(v1)) == sqrt(d2(v2)).

    d2 is evaluated as the reference does: ((dx*dx + dy*dy) + dz*dz) in IEEE double.
    A first-index argmin over sqrt values must keep v1 (index 0); an argmin over the
    squared distances would wrongly pick v2.
    """
    def d2(v):
        return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]

    v1 = (s, 0.0, 0.0)
    a1 = d2(v1)
    r1 = math.sqrt(a1)
    want = math.nextafter(a1, 0.0)           # the double just below d2(v1)
    for k in range(1, 4000):
        a = s * (1.0 - k * 2.0 ** -30)
        target = want - a * a
        if target <= 0:
            continue
        b = math.sqrt(target)
        v2 = (a, b, 0.0)
        a2 = d2(v2)
        if a2 < a1 and math.sqrt(a2) == r1:
            return v1, v2
    raise RuntimeError("no sqrt tie found")


def sqrt_tie_grid():
    """Grid [C0, C1, P0] with P0 at the origin tied (after sqrt) between C0 and C1.

    With initial centroids at grid points 0 and 1, one iteration moves the centroid that
    captures P0 (weight 10) onto P0; map_to_grid then returns {0 or 1, 2}.
    """
    v1, v2 = sqrt_tie_vectors()
    grid = np.array([v1, v2, (0.0, 0.0, 0.0)], dtype=np.float64)
    rho = np.array([1.0, 1.0, 10.0])
    return grid, rho


def exact_tie_grid(n=6):
    """Integer lattice with centroids placed so that many points are exactly equidistant."""
    ax = np.arange(n, dtype=np.float64)
    g = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    rho = 1.0 + 0.01 * np.arange(g.shape[0]) % 7
    return g, rho


def rounding_stress_grid(seed: int = 11):
    """A lattice whose centroid sums round on nearly every step, with exact halves.

    Coordinates are multiples of 2^-4 on both sides of zero and the weights are
    1 + m 2^-40: products carry bits down to 2^-44 while sums of ~10^3 terms round at
    2^-42, so a quarter of the additions are exact ties, and the coordinate sums change sign
    and binade.  Pins the warp-parallel sequential summation against the plain loop.
    """
    rng = np.random.default_rng(seed)
    n = 16
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    grid = np.stack([(i - 7.5) * 0.5, (j - 8) * 0.5625, (k - 6) * 0.4375], -1).reshape(-1, 3)
    grid = grid + rng.integers(-3, 4, size=grid.shape) * 2.0 ** -4
    rho = 1.0 + rng.integers(0, 2 ** 40, size=grid.shape[0]).astype(np.float64) * 2.0 ** -40
    return np.ascontiguousarray(grid), rho


def limit_case():
    """k-means at the size limits of thc_kmeans_noalloc: N_g = 65,536 (a 64 x 32 x 32 mesh
    of the 8-atom diamond cell), N_mu = 1,024, max_it = 1,000, threshold 1e-6.

    The weight is a sum of Gaussians exp(-0.6 |r - R|^2) over the atoms and their nearest
    periodic images, so every region of the cell carries weight and no cluster empties.
    Returns (grid, rho, nmu, max_it, threshold, rng_seed).
    """
    from thcpp_gb300 import synth
    a = synth.A_DIAMOND
    lattice = np.eye(3) * a
    grid = synth.uniform_grid(lattice, (64, 32, 32))
    atoms = synth._DIAMOND_FRAC @ lattice
    shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)],
                      dtype=np.float64) @ lattice
    rho = np.zeros(grid.shape[0])
    for at in atoms:
        for sh in shifts:
            d = grid - (at + sh)
            rho += np.exp(-0.6 * np.einsum("ij,ij->i", d, d))
    return np.ascontiguousarray(grid), rho, 1024, 1000, 1e-6, 29


def ref_case_inputs(name):
    """(grid, rho, norb, thc_cfac, max_it, threshold, rng_seed) of a case of the reference
    k-means fixtures (tests/golden/make_ref_golden.py): a synthetic system by name, c4_<s>
    for system s of the batch, ``limit`` (:func:`limit_case`) and ``limit_full`` (the same
    with a negative threshold, so that every one of the 1,000 iterations runs)."""
    from thcpp_gb300 import synth
    from tests.conftest import system
    if name.startswith("limit"):
        g, r, nmu, mi, th, seed = limit_case()
        return g, r, nmu // 8, 8, mi, (th if name == "limit" else -1.0), seed
    s = synth.c4_system(int(name[3:])) if name.startswith("c4_") else system(name)
    return s.grid, s.density, s.norb, s.thc_cfac, s.max_it, s.threshold, s.rng_seed
