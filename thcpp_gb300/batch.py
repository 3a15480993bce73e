"""Batched factorisations through ``thc_factorize_batched`` (the C4 workload).

The reference factorises one system per run (``src/main.cpp:50-72``); a batch of
independent systems is a sequence of such runs.  ``thc_factorize_batched`` runs the same
k-means + ISDF per system, but spreads the systems over several contexts, each with its own
CUDA stream and host thread, so that the many small, latency-bound kernels of different
systems overlap on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import capi


def system_arrays(s, device=None):
    """Inputs and output buffers of one synthetic system for the C ABI.

    With ``device`` (a torch device) the arrays are device tensors, else numpy arrays.
    """
    init = capi.initial_indices(s.ng, s.nmu, s.rng_seed)
    arrs = dict(grid=np.ascontiguousarray(s.grid), rho=np.ascontiguousarray(s.density),
                init_idx=init, phi=np.ascontiguousarray(s.phi),
                mesh=np.asarray(s.mesh, np.int32), coulG=np.ascontiguousarray(s.coulG),
                out_idx=np.zeros(s.nmu, np.int32), out_orbitals=np.zeros((s.norb, s.nmu, 2)),
                out_M=np.zeros((s.nmu, s.nmu, 2)), out_L=np.zeros((s.nmu, s.nmu, 2)))
    if device is not None:
        import torch
        arrs = {k: (v if k == "mesh" else torch.from_numpy(v).to(device))
                for k, v in arrs.items()}
        # The library's streams do not synchronise with torch's: finish the copies here.
        torch.cuda.synchronize(device)
    return arrs


def batch_entry(s, arrs, shift_rel=-1.0):
    """The thc_system fields of one system (arrays from :func:`system_arrays`)."""
    return dict(grid=arrs["grid"], rho=arrs["rho"], ng=s.ng, nmu=s.nmu,
                init_idx=arrs["init_idx"], max_it=s.max_it, threshold=s.threshold,
                phi=arrs["phi"], norb=s.norb, mesh=arrs["mesh"], coulG=arrs["coulG"],
                shift_rel=shift_rel, out_idx=arrs["out_idx"],
                out_orbitals=arrs["out_orbitals"], out_M=arrs["out_M"], out_L=arrs["out_L"])


def run_sequential(ctx, systems, arrays):
    """One system after the other on one context: the sequential per-system baseline."""
    statuses, times = [], []
    for s, a in zip(systems, arrays):
        _, kst, st = ctx.kmeans(a["grid"], a["rho"], s.nmu, a["init_idx"], s.max_it,
                                s.threshold, out_idx=a["out_idx"], raise_on_error=False)
        ims = 0.0
        if st == capi.THC_OK:
            r = ctx.isdf(a["phi"], a["out_idx"], s.mesh, a["coulG"], out_M=a["out_M"],
                         out_L=a["out_L"], out_orbitals=a["out_orbitals"],
                         raise_on_error=False)
            st = r["status"]
            ims = r["stats"].device_ms
        statuses.append(st)
        times.append((kst.device_ms, ims))
    run_sequential.times = times
    return statuses


def run_batched(systems, arrays, precision, nstreams=4, device=0):
    """All systems through thc_factorize_batched; returns (status, per-system statuses)."""
    entries = [batch_entry(s, a) for s, a in zip(systems, arrays)]
    st, arr = capi.factorize_batched(entries, device=device, precision=precision,
                                     nstreams=nstreams)
    run_batched.errors = [arr[i].error.decode(errors="replace") for i in range(len(systems))]
    return st, [arr[i].status for i in range(len(systems))]
