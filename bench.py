"""Benchmark: ISDF seconds per system on one GB300 (mixed precision vs all-FP64).

One step = one full factorisation of one synthetic system (k-means interpolating points
+ interpolating vectors + FFT Coulomb matrix + its Cholesky factor) through the C ABI of
libthc_gb300.so.  Workload: the 8-atom diamond conventional cell, 48^3 grid
(N_g = 110,592), N_o = 32, N_mu = 256, k-means max_it 100 / threshold 1e-6.

  value  mixed-precision s/system with inputs resident in HBM (device pointers),
         L2 flushed before every timed step, CUDA events on the library's stream
  e2e    the same through the C ABI with pinned HOST buffers: H2D of the inputs and D2H
         of idx, Orbitals, M and Luv inside the timed region (wall clock)
  fp64   the all-FP64 path (the drop-in) on the same inputs, and the mixed/FP64 M error

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank factorises its own replica of the workload (the path
has no exchange step: replicas only) and rank 0 prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c2": {"workload": "diamond-8atom-48^3-no32-nmu256", "n_g": 110592, "n_orb": 32,
           "n_mu": 256, "mesh": [48, 48, 48]},
    "c3": {"workload": "diamond-64atom-72^3-no256-nmu2048", "n_g": 373248, "n_orb": 256,
           "n_mu": 2048, "mesh": [72, 72, 72]},
    "c4": {"workload": "batch-48-random-cubic-cells-32^3..64^3-no16..200-nmu6..10xno",
           "systems": 48},
    "c5": {"workload": "diamond-216atom-108^3-no864-nmu5184", "n_g": 1259712, "n_orb": 864,
           "n_mu": 5184, "mesh": [108, 108, 108]},
}
WORKLOAD = "c2"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per sliced-GEMM launch, mean of
# the three launches of one factorisation, from one ncu capture of the workload; None where
# no capture was taken.
OZ_TRAFFIC = {"c2": ((43.2 + 170.2) + (341.4 + 95.9) + (295.2 + 4.7)) * 1e6 / 3.0}
CONFIG = dict(WORKLOADS[WORKLOAD], kmeans_max_it=100, kmeans_threshold=1e-6,
              l2="flushed (256 MB write) before every timed step", parallelism="replicas")
METRIC = "ISDF s/system on 1 GB300 (mixed precision; FP64 path reported beside)"


def sliced_gemm_flops(ng, no, nmu, mesh, shifted, refine, slices=(6, 6, 5)):
    """Algorithmic tensor-pipe work of one mixed factorisation: the sum over its sliced
    GEMMs of (slice pairs) x 2 M N K.  P = Phi Phi_mu^T and the Coulomb product (its lower
    half, K = 2 N_c over the half spectrum, Nyquist planes included) always; the solve is
    zeta^T = C^{-1} Z^T with C^{-1} = X^T X formed by a sliced product from N_mu = 512 on
    (the library's threshold), or, with a shift, two products (Y^T = Z (P X)^T, then
    zeta^T = X^T Y) plus refinement's G = X X^T and one N_mu^3 product per step."""
    sp, sz, sm = slices
    pairs = lambda L: L * (L + 1) // 2
    n0, n1, n2 = mesh
    nc2 = 2 * n0 * n1 * (n2 // 2 + 1)
    flops = (pairs(sp) * 2 * nmu * ng * no + pairs(sz) * 2 * nmu * ng * nmu
             + pairs(sm) * 2 * nmu * nmu * nc2 / 2)
    if shifted:
        flops += pairs(sz) * 2 * nmu * ng * nmu + (
            pairs(sz) * 2 * nmu ** 3 * (1 + refine) if refine > 0 else 0)
    elif nmu >= 512:
        flops += pairs(sz) * 2 * nmu ** 3
    return flops


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def aggregate_over_ranks(values, device=None):
    """Max over ranks of per-rank timings (replicas: the slowest rank bounds the job).

    Returns the list unchanged for a single process.  Uses the default process group
    (NCCL on GPUs, gloo on CPU).
    """
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def cpu_reference_step(s, nthreads):
    """The CPU port of the reference path (oracle): C++ k-means + LAPACK/FFT ISDF."""
    import oracle
    t0 = time.perf_counter()
    km = oracle.kmeans_system(s, nthreads=nthreads)
    oracle.isdf_reference(s.phi, km.idx, s.mesh, s.coulG, workers=nthreads)
    return time.perf_counter() - t0


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from thcpp_gb300 import synth
    import oracle
    oracle.build()
    s = synth.config(WORKLOAD)
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_step(s, nthreads)
    ts = [cpu_reference_step(s, nthreads) for _ in range(args.steps)]
    v = float(np.sum(ts) / args.steps)
    line = {"metric": METRIC, "value": v, "unit": "s/system", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * v,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian s/p orbitals)", "config": CONFIG,
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "s/system", "cores": nthreads, "kind": "port",
                             "sample": "full factorisation of the workload per step: C++ "
                                       "k-means restatement (OpenMP) + numpy/scipy zgels, "
                                       "C2C FFT, herk, zpotrf"},
            "e2e": {"value": v, "unit": "s/system", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_c4(args):
    """The batched workload: 48 seeded random cubic systems, thc_factorize_batched against
    the same 48 factorisations one after another on one context (mixed precision).

    The batch spans several CUDA streams, so each step is timed on the host clock around a
    device-wide synchronisation.  Inputs are resident in HBM before timing starts.
    """
    import torch
    from thcpp_gb300 import batch, build, capi, synth
    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nsys = args.c4_systems
    t0 = time.perf_counter()
    systems = [synth.c4_system(i) for i in range(nsys)]
    gen_s = time.perf_counter() - t0
    prec = capi.THC_PREC_MIXED
    seq_arr = [batch.system_arrays(s, dev) for s in systems]
    bat_arr = [batch.system_arrays(s, dev) for s in systems]
    ctx = capi.Context(0, prec)

    def run_seq():
        st = batch.run_sequential(ctx, systems, seq_arr)
        if any(x not in (capi.THC_OK, capi.THC_ERR_NOT_PD) for x in st):
            raise RuntimeError(f"sequential statuses {st}")

    def run_bat():
        st, per = batch.run_batched(systems, bat_arr, prec, nstreams=args.c4_streams)
        if any(x not in (capi.THC_OK, capi.THC_ERR_NOT_PD) for x in per):
            errs = {i: e for i, e in enumerate(batch.run_batched.errors) if per[i] not in (0, 4)}
            raise RuntimeError(f"batched status {st}: {per} {errs}")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(args.steps):
            torch.cuda.synchronize()
            a = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            tot += time.perf_counter() - a
        return tot / args.steps

    launches0 = ctx.kernel_launches
    t_seq = timed(run_seq)
    seq_launches = (ctx.kernel_launches - launches0) // (args.steps + args.warmup)
    t_bat = timed(run_bat)
    tune = ctx.autotune_log()
    same_idx = all(torch.equal(a["out_idx"], b["out_idx"]) for a, b in zip(seq_arr, bat_arr))
    dm = max(float(torch.linalg.norm(a["out_M"] - b["out_M"]) / torch.linalg.norm(a["out_M"]))
             for a, b in zip(seq_arr, bat_arr))
    ctx.close()
    line = {
        "metric": "batched ISDF s/system on 1 GB300 (48 systems, mixed precision)",
        "value": t_bat / nsys, "unit": "s/system", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_bat * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16-sliced/fp32/fp64",
        "data": "synthetic (seeded random cubic cells, Gaussian s/p orbitals)",
        "config": dict(WORKLOADS["c4"], systems=nsys, streams=args.c4_streams,
                       l2="inputs of the batch (several GB) exceed L2",
                       timing="host clock around device-synchronised batches"),
        "sequential_s_per_system": t_seq / nsys,
        "speedup_batched_vs_sequential": t_seq / t_bat,
        "idx_identical": same_idx, "max_rel_diff_M_batched_vs_sequential": dm,
        "gpu_launches": seq_launches,
        "host_generation_s": gen_s,
        "sequential_kmeans_ms_total": sum(t[0] for t in batch.run_sequential.times),
        "sequential_isdf_ms_total": sum(t[1] for t in batch.run_sequential.times),
        "sequential_largest_ms": max(t[0] + t[1] for t in batch.run_sequential.times),
        "autotune": tune,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--paths", default="mixed,fp64,e2e,qrcp",
                    help="comma list of measured paths (a profiling run may keep only 'mixed')")
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS),
                    help="c2 is the benchmark workload; c3 and c4 (batch) are reported separately")
    ap.add_argument("--c4-systems", type=int, default=48)
    ap.add_argument("--c4-streams", type=int, default=8)
    ap.add_argument("--refine", type=int, default=None,
                    help="refinement steps of the shifted solve (default: 1 for c5, else 0)")
    args = ap.parse_args()
    if args.workload == "c4" and args.impl != "reference":
        return run_c4(args)
    global WORKLOAD, CONFIG
    WORKLOAD = args.workload
    CONFIG = dict(WORKLOADS[WORKLOAD], kmeans_max_it=100, kmeans_threshold=1e-6,
                  l2="flushed (256 MB write) before every timed step", parallelism="replicas")
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from thcpp_gb300 import build, capi, synth
    build.build()
    on_device = WORKLOAD == "c5"
    if on_device:
        # 1.26e6 points x 864 Gaussians: generated on the GPU (the host build takes hours).
        with capi.Context(local, capi.THC_PREC_FP64) as gctx:
            s = synth.config_gpu(WORKLOAD, gctx, dev)
    else:
        s = synth.config(WORKLOAD)
    nmu, ng, no = s.nmu, s.ng, s.norb
    init = capi.initial_indices(ng, nmu, s.rng_seed)
    # The 216-atom cell's C is near rank-deficient by construction: its FP64 Cholesky always
    # runs with the diagonal shift 1e-10 tr(C)/N_mu, followed by refinement of zeta.
    shift_rel = 1e-10 if WORKLOAD == "c5" else -1.0
    refine = args.refine if args.refine is not None else (1 if WORKLOAD == "c5" else 0)

    # Device-resident inputs.
    as_dev = (lambda a: a) if on_device else (lambda a: torch.from_numpy(a).to(dev))
    d_grid = as_dev(s.grid)
    d_rho = as_dev(s.density)
    d_phi = as_dev(s.phi)
    d_coul = as_dev(s.coulG)
    d_init = torch.from_numpy(init).to(dev)
    d_idx = torch.zeros(nmu, dtype=torch.int32, device=dev)
    d_M = torch.zeros((nmu, nmu, 2), dtype=torch.float64, device=dev)
    d_L = torch.zeros((nmu, nmu, 2), dtype=torch.float64, device=dev)
    d_orb = torch.zeros((no, nmu, 2), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # A dedicated stream: the library launches on it and the CUDA events are recorded on it.
    stream = torch.cuda.Stream(dev)

    def device_step(ctx):
        _, kst, st = ctx.kmeans(d_grid, d_rho, nmu, d_init, s.max_it, s.threshold, out_idx=d_idx)
        if st:
            raise RuntimeError(f"thc_kmeans status {st}")
        r = ctx.isdf(d_phi, d_idx, s.mesh, d_coul, shift_rel, out_orbitals=d_orb, out_M=d_M,
                     out_L=d_L)
        return kst, r

    def timed(ctx, steps, warmup):
        ctx.set_stream(stream.cuda_stream)
        ctx.set_option("refine", refine)
        for _ in range(warmup):
            device_step(ctx)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = ctx.kernel_launches
        ctx.set_option("profile", 1)
        tot = 0.0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            kst, r = device_step(ctx)
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        launches = ctx.kernel_launches - l0
        return tot / steps, launches, kst, r

    # Mixed precision (the headline).
    ctx = capi.Context(local, capi.THC_PREC_MIXED)
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.nvtx.range_push("mixed")
    ms_mixed, launches, kst, r_mx = timed(ctx, args.steps, args.warmup)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    torch.cuda.synchronize()
    free_b, total_b = torch.cuda.mem_get_info()
    mem_gb = (total_b - free_b) / 1e9      # inputs + the library's grow-only workspace
    M_mixed = d_M.cpu().numpy().copy()
    isdf_st = r_mx["stats"]
    oz_ms, oz_n = ctx.kernel_time("ozgemm")
    km_ms, km_n = ctx.kernel_time("km_assign")
    # Device time per system of each stage of the timed steps (CUDA events the library
    # records around its launches; stages nest: "ozgemm" is the sum of the oz_* products,
    # "dgemm" includes the FP64 GEMMs inside potrf_inv and chol_inverse).
    stage_ms = {}
    for name in ("kmeans", "oz_P", "oz_cinv", "oz_Y", "oz_zeta", "oz_M", "ozgemm", "slice",
                 "fft", "potrf_inv", "chol_inverse", "dgemm", "oz_split_reduce"):
        ms_, n_ = ctx.kernel_time(name)
        if n_:
            stage_ms[name] = round(ms_ / args.steps, 4)
    ctx.set_option("profile", 0)

    paths = set(args.paths.split(","))
    # All-FP64 path on the same inputs.  A failure here (or in any other side leg below) is
    # recorded under an "error" key of that leg and never voids the headline line.
    ms_fp64 = float("nan")
    rel_err = None
    dg_ms = 0.0
    idx_same = None
    leg_errors = {}

    def fp64_leg():
        nonlocal ms_fp64, rel_err, dg_ms, idx_same, ctx
        idx_mx = d_idx.cpu().numpy().copy()
        if on_device:
            # Both paths' workspaces do not fit at once at this size: free the mixed one.
            ctx.close()
        ctx64 = capi.Context(local, capi.THC_PREC_FP64)
        torch.cuda.nvtx.range_push("fp64")
        ms_fp64, launches64, kst64, r64 = timed(ctx64, args.fp64_steps,
                                                0 if on_device else 1)
        torch.cuda.nvtx.range_pop()
        dg_ms, dg_n = ctx64.kernel_time("dgemm")
        ctx64.set_option("profile", 0)
        idx64 = d_idx.cpu().numpy().copy()
        M_fp64 = d_M.cpu().numpy().copy()
        if on_device:
            ctx64.close()
            ctx = capi.Context(local, capi.THC_PREC_MIXED)
        Mc = M_mixed[..., 0] + 1j * M_mixed[..., 1]
        M6 = M_fp64[..., 0] + 1j * M_fp64[..., 1]
        rel_err = float(np.linalg.norm(Mc - M6) / np.linalg.norm(M6))
        idx_same = bool(np.array_equal(idx64, idx_mx))

    if "fp64" in paths:
        try:
            fp64_leg()
        except Exception as e:  # recorded, not fatal: the headline is the mixed path
            leg_errors["fp64"] = f"{type(e).__name__}: {e}"
            if on_device and getattr(ctx, "h", None) is None:
                ctx = capi.Context(local, capi.THC_PREC_MIXED)

    # QRCP interpolating points (the reference's other point selector) on the same orbitals,
    # N_mu pivots over N_g columns; FP64 in both precisions.  Untimed by the step clock.
    qrcp = None

    def qrcp_leg():
        q_ms = []
        for i in range(4):
            rq = ctx.qrcp(d_phi, nmu)
            if i:
                q_ms.append(rq["stats"].device_ms)
        q = float(np.median(q_ms))
        # FP64 FMAs: N_g (N_o + k) per step k (the Gram entry and the projection).
        q_flop = 2.0 * ng * (nmu * no + nmu * (nmu - 1) / 2)
        return {"points": nmu, "s_per_system": q * 1e-3,
                "numerical_rank": int(rq["stats"].numerical_rank),
                "fp64_tflops": q_flop / (q * 1e-3) / 1e12, "fp64_peak_tflops": 1.25,
                "peak_source": "nominal (FP64 is not in the measured peaks)"}

    if "qrcp" in paths and WORKLOAD == "c2":
        try:
            qrcp = qrcp_leg()
        except Exception as e:
            qrcp = {"error": f"{type(e).__name__}: {e}"}

    # End to end through the C ABI with pinned host buffers.
    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.numpy()
    host = (lambda a: a.cpu().numpy()) if on_device else (lambda a: a)
    h_grid, h_rho, h_phi, h_coul = (pinned(host(s.grid)), pinned(host(s.density)),
                                    pinned(host(s.phi)), pinned(host(s.coulG)))
    h_init = pinned(init)
    h_idx = pinned(np.zeros(nmu, np.int32))
    h_M = pinned(np.zeros((nmu, nmu, 2)))
    h_L = pinned(np.zeros((nmu, nmu, 2)))
    h_orb = pinned(np.zeros((no, nmu, 2)))
    ctx.set_stream(None)

    def host_step():
        ctx.kmeans(h_grid, h_rho, nmu, h_init, s.max_it, s.threshold, out_idx=h_idx)
        ctx.isdf(h_phi, h_idx, s.mesh, h_coul, shift_rel, out_orbitals=h_orb, out_M=h_M,
                 out_L=h_L)

    e2e = float("nan")
    if "e2e" in paths:
        torch.cuda.nvtx.range_push("e2e")
        for _ in range(args.warmup):
            host_step()
        e2e = 0.0
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            host_step()
            e2e += time.perf_counter() - t0
        e2e /= args.steps
        torch.cuda.nvtx.range_pop()
    h2d = (h_grid.nbytes + h_rho.nbytes + h_init.nbytes + h_phi.nbytes + h_coul.nbytes
           + h_idx.nbytes)
    d2h = h_idx.nbytes + h_orb.nbytes + h_M.nbytes + h_L.nbytes

    # Max over ranks (replicas: each rank factorised its own copy of the workload).
    t_step, e2e = aggregate_over_ranks([ms_mixed, e2e], device=dev)

    if rank == 0:
        import json as _json
        peaks = {}
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            peaks = _json.load(open(pk))
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        peak_src = "measured" if "bf16_tflops" in peaks else "fallback"
        # Dominant tensor kernel: the sliced GEMMs.
        flops = sliced_gemm_flops(ng, no, nmu, s.mesh, bool(isdf_st.rank_deficient), refine)
        # Aggregate over the timed launches: all their flops over all their time.
        achieved = flops * args.steps / (oz_ms * 1e-3) / 1e12 if oz_n else None
        roof = {"kernel": "ozgemm (sliced-BF16 tensor GEMMs of a factorisation, aggregate)",
                "bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": (achieved / bf16_peak) if achieved else None,
                "peak_source": peak_src, "traffic": OZ_TRAFFIC.get(args.workload),
                "traffic_unit": "bytes per launch",
                "share_of_step": (oz_ms / args.steps) / t_step if oz_n else None}
        cpu = None
        if not args.no_cpu_baseline and not on_device:
            try:
                t_cpu = cpu_reference_step(s, os.cpu_count() or 1)
                cpu = {"value": t_cpu, "unit": "s/system", "cores": os.cpu_count(),
                       "kind": "port",
                       "sample": "1 full factorisation of the workload (C++ k-means "
                                 "restatement + numpy/scipy zgels/FFT/herk/zpotrf) on the "
                                 "host cores"}
            except Exception as e:
                cpu = {"value": None, "error": f"{type(e).__name__}: {e}"}
        line = {
            "metric": METRIC, "value": t_step * 1e-3 / 1.0, "unit": "s/system",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16-sliced/fp32/fp64", "data": "synthetic (seeded Gaussian s/p orbitals)",
            "config": CONFIG,
            "e2e": {"value": e2e, "unit": "s/system", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "fp64": {"s_per_system": ms_fp64 * 1e-3, "speedup_mixed_vs_fp64": ms_fp64 / t_step,
                     "rel_err_M_mixed_vs_fp64": rel_err, "idx_identical": idx_same,
                     "dgemm_ms_per_system": dg_ms / max(args.fp64_steps, 1)},
            "kmeans": {"iterations": kst.iterations, "rechecked_points": int(kst.rechecked),
                       "assign_us_per_iteration": (1e3 * km_ms / km_n) if km_n else None},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "stage_ms_per_system": stage_ms,
        }
        # Conditioning of C at the k-means points (side computation, after the timing; a
        # failure here leaves it null).
        cond = None
        try:
            pm = d_phi[d_idx.long()]
            cmat = (pm @ pm.T) ** 2
            try:
                ev = torch.linalg.eigvalsh(cmat).cpu().numpy()
            except RuntimeError:           # no GPU linear-algebra library in this process
                ev = np.linalg.eigvalsh(cmat.cpu().numpy())
            cond = float(ev[-1] / ev[0]) if float(ev[0]) > 0 else None
        except Exception as e:
            leg_errors["cond_C"] = f"{type(e).__name__}: {e}"
        line["solve"] = {"cond_C": cond,
                         "shift_rel": shift_rel if shift_rel > 0 else None,
                         "shift_used": isdf_st.shift_used, "refine_steps": refine,
                         "rank_deficient": int(isdf_st.rank_deficient)}
        line["device_memory_gb"] = round(mem_gb, 2)
        # The sliced-GEMM autotuner's decisions (shape class -> k-step, tile order, split).
        line["autotune"] = ctx.autotune_log()
        if qrcp:
            line["qrcp"] = qrcp
        if leg_errors:
            line["leg_errors"] = leg_errors
        # Whole-job s/system: ws replicas each factorised one system per step in t_step.
        line["value"] = t_step * 1e-3 / ws
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
