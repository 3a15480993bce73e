"""The oracle still reproduces the committed golden fixtures (regression pin)."""
import os

import numpy as np

import oracle
from thcpp_gb300 import synth

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_tiny_golden():
    g = np.load(os.path.join(HERE, "tiny.npz"))
    s = synth.config("tiny")
    km = oracle.kmeans_system(s)
    assert np.array_equal(km.idx, g["idx"]) and km.iters == int(g["iters"])
    assert km.diff == float(g["diff"])
    r = oracle.isdf_real(s.phi, km.idx, s.mesh, s.coulG)
    assert np.linalg.norm(r["M"] - g["M"]) <= 1e-10 * np.linalg.norm(g["M"])


def test_c1_golden():
    g = np.load(os.path.join(HERE, "c1_idx.npz"))
    km = oracle.kmeans_system(synth.config("c1"))
    assert np.array_equal(km.idx, g["idx"]) and km.iters == int(g["iters"])
