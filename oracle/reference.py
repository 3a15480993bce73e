"""The reference's own k-means, built from its sources -- TEST INFRASTRUCTURE ONLY.

``oracle/ref/Makefile`` compiles the reference's ``src/kmeans.cpp`` unmodified (with a
one-rank MPI stand-in and in-memory datasets in place of the HDF5 orbital file) into
``oracle/_ref/kmeans_ref``.  :func:`kmeans` runs that binary and returns what
``KMeansSolver::kernel`` (``src/kmeans.cpp:187-264``) produced: the interpolating-point
indices and the step table it prints every 10 iterations (iteration, normed difference,
% of labels changed; ``src/kmeans.cpp:238``).

The reference tree is present only where the library is developed; :func:`available` says
whether the binary exists or can be built.  The committed fixtures under ``tests/golden/``
that carry its outputs to machines without the tree are made by
``tests/golden/make_ref_golden.py``.
"""

from __future__ import annotations

import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RECIPE = os.path.join(HERE, "ref")
BINARY = os.path.join(HERE, "_ref", "kmeans_ref")


def reference_dir() -> str:
    """The reference tree the recipe compiles from (the Makefile's REF)."""
    return subprocess.run(["make", "-s", "-C", RECIPE, "reference-dir"], capture_output=True,
                          text=True, check=True).stdout.strip()


def available() -> bool:
    """Whether the reference tree (and so the binary's sources) is present here."""
    try:
        return os.path.exists(os.path.join(reference_dir(), "src", "kmeans.cpp"))
    except (OSError, subprocess.CalledProcessError):
        return False


def build() -> str:
    """Build (or refresh) oracle/_ref/kmeans_ref from the reference's sources."""
    subprocess.run(["make", "-s", "-C", RECIPE], check=True, capture_output=True)
    return BINARY


class RefKMeans:
    def __init__(self, idx, steps, threshold_breached, stdout):
        self.idx = idx                      # N_mu int32, sorted (the reference's output)
        self.steps = steps                  # [(iteration, diff, pct)] every 10 iterations
        self.threshold_breached = threshold_breached
        self.stdout = stdout


_STEP = re.compile(r"^\s+(\d+)\s+([-+0-9.eE]+)\s+([-+0-9.eE]+)\s*$")


def kmeans(grid, rho, norb: int, thc_cfac: int, max_it: int, threshold: float,
           rng_seed: int) -> RefKMeans:
    """Run the reference's KMeansSolver on one rank (N_mu = thc_cfac * norb)."""
    build()
    g = np.ascontiguousarray(grid, np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(rho, np.float64).reshape(-1)
    ng = g.shape[0]
    with tempfile.TemporaryDirectory() as d:
        fin = os.path.join(d, "in.bin")
        fout = os.path.join(d, "idx.bin")
        with open(fin, "wb") as f:
            np.array([ng, norb], np.int64).tofile(f)
            g.tofile(f)
            r.tofile(f)
        p = subprocess.run([BINARY, fin, str(thc_cfac), str(max_it), repr(float(threshold)),
                            str(int(rng_seed)), fout], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"kmeans_ref exited {p.returncode}: {p.stdout[-400:]}"
                               f"{p.stderr[-400:]}")
        idx = np.fromfile(fout, np.int32)
    steps = []
    for line in p.stdout.splitlines():
        m = _STEP.match(line)
        if m:
            steps.append((int(m.group(1)), float(m.group(2)), float(m.group(3))))
    breached = "Threshold not breached" not in p.stdout
    return RefKMeans(idx, steps, breached, p.stdout)


def kmeans_system(system) -> RefKMeans:
    return kmeans(system.grid, system.density, system.norb, system.thc_cfac, system.max_it,
                  system.threshold, system.rng_seed)
