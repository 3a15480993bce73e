"""Accuracy report of one config against the blocked FP64 GPU oracle (test infrastructure).

    python -m tests.accuracy_report c5 [--refine K] [--prec mixed|fp64] [--pairs 512]
                                       [--slices P,Z,M]

Runs the library's k-means and ISDF on the config exactly as bench.py does (the 216-atom
cell generated on the GPU, its C solved with the shift 1e-10 tr(C)/N_mu and refinement),
keeps the interpolating vectors, frees the library's workspace, then runs
oracle/isdf_torch.py on the same points with the same shift and refinement steps and
prints one JSON line: relative Frobenius errors of M and zeta, the ISDF reconstruction error
of sampled orbital-pair densities for both, cond(C), the device memory the library used and
the device time of the ISDF call (the second of two, so that the autotuner's trials are not
in it).  --slices sets the slice depths of the P, zeta and Coulomb products (mixed path).
"""
import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    import numpy as np
    import torch

    from oracle import isdf_torch
    from thcpp_gb300 import build, capi, synth

    ap = argparse.ArgumentParser()
    ap.add_argument("config")
    ap.add_argument("--refine", type=int, default=None)
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--pairs", type=int, default=512)
    ap.add_argument("--slices", default=None, help="P,Z,M slice depths (2..6)")
    a = ap.parse_args()
    build.build()
    dev = torch.device("cuda", 0)
    t0 = time.time()
    if a.config == "c5":
        with capi.Context(0, capi.THC_PREC_FP64) as g:
            s = synth.config_gpu("c5", g, dev)
        phi, grid, rho, coul = s.phi, s.grid, s.density, s.coulG
    else:
        s = synth.config(a.config)
        phi, grid, rho, coul = (torch.from_numpy(x).to(dev) for x in
                                (s.phi, s.grid, s.density, s.coulG))
    shift_rel = 1e-10 if a.config == "c5" else -1.0
    refine = a.refine if a.refine is not None else (1 if a.config == "c5" else 0)
    prec = capi.THC_PREC_MIXED if a.prec == "mixed" else capi.THC_PREC_FP64
    init = torch.from_numpy(capi.initial_indices(s.ng, s.nmu, s.rng_seed)).to(dev)
    idx = torch.zeros(s.nmu, dtype=torch.int32, device=dev)
    free0, total = torch.cuda.mem_get_info()
    with capi.Context(0, prec) as ctx:
        ctx.kmeans(grid, rho, s.nmu, init, s.max_it, s.threshold, out_idx=idx)
        ctx.set_option("refine", refine)
        slices = None
        if a.slices:
            slices = [int(x) for x in a.slices.split(",")]
            for key, v in zip(("slices_p", "slices_z", "slices_m"), slices):
                ctx.set_option(key, v)
        ctx.isdf(phi, idx, s.mesh, coul, shift_rel)
        r = ctx.isdf(phi, idx, s.mesh, coul, shift_rel)
        torch.cuda.synchronize()
        used_gb = (free0 - torch.cuda.mem_get_info()[0]) / 1e9
        zt = torch.empty((s.nmu, s.ng), dtype=torch.float64, device=dev)
        ctx.interpolating_vectors(s.ng, s.nmu, out=zt)
        st = r["stats"]
        M = r["M"][..., 0] + 1j * r["M"][..., 1]
    torch.cuda.empty_cache()
    idx_h = idx.cpu().numpy()
    ref = isdf_torch.isdf_real(phi, idx_h, s.mesh, coul,
                               shift_rel=shift_rel if shift_rel > 0 else None,
                               shift=0.0 if shift_rel > 0 else st.shift_used, refine=refine)
    em = float(np.linalg.norm(M - ref["M"]) / np.linalg.norm(ref["M"]))
    ez = float(torch.linalg.norm(zt - ref["zeta_t"]) / torch.linalg.norm(ref["zeta_t"]))
    pairs = isdf_torch.sample_pairs(s.norb, a.pairs)
    ep = isdf_torch.pair_density_error(zt, phi, idx_h, pairs)
    ep_ref = isdf_torch.pair_density_error(ref["zeta_t"], phi, idx_h, pairs)
    out = {"config": a.config, "precision": a.prec, "n_g": s.ng, "n_orb": s.norb,
           "n_mu": s.nmu, "cond_C": ref["cond_C"], "shift_rel": shift_rel if shift_rel > 0
           else None, "shift_used": st.shift_used, "refine_steps": refine,
           "rel_err_M": em, "rel_err_zeta": ez, "pair_density_err": ep,
           "pair_density_err_oracle": ep_ref, "pairs_sampled": int(len(pairs)),
           "library_device_memory_gb": round(used_gb, 2), "slices": slices,
           "isdf_device_ms": round(float(st.device_ms), 3), "wall_s": round(time.time() - t0, 1)}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
