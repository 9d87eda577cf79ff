"""Benchmark of the CI hot path on one GB300.

A step is one mixed-precision block-Davidson solve for the 10 lowest
eigenpairs of the fp-shell 4p+4n M=0 problem (dimension 1,963,461, seeded
synthetic Gaussian TBMEs, lambda = 0.5), from the Hamiltonian resident in HBM
to 10 eigenpairs with residual <= 1e-5 (FP32 H and vectors, FP64 projection,
FP64 refinement).  `value` is seconds per solve (lower is better).
`e2e` times the whole user call through the C ABI: interaction tables from
the host, GPU basis, GPU Hamiltonian build, the solve and the eigenvectors
copied back to host memory.  Also reported: the plain FP64 GPU Davidson (the
reference algorithm: block 10, basis limit 30, one-vector Gram-Schmidt, FP64
everything) and the SpMM kernel against the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference the reference algorithm runs on the host CPU cores with
nothing from the product library (oracle/: the XML and interaction
restatement, basis, row builder, CSB pull-form SpMM and Davidson in C with
OpenMP) on the same problem; each step is one Davidson iteration of one
continuous run, and the value scales the measured seconds per iteration to the
iteration cap at which that algorithm stops on this problem.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "davidson_seconds_to_10_eigenpairs"
NSTATES = 10
TOL = 1e-5
WORKLOAD = dict(workload="fp-shell 4p+4n M=0, lowest 10 eigenpairs, |dE|<=1e-4 MeV, resid<=1e-5",
                space="fp", protons=4, neutrons=4, twoM=0, dimension=1963461, lam=0.5, seed=7,
                l2="inputs larger than L2 (stored H ~15 GB, vectors ~300 MB)")
# Davidson settings of the mixed solve (block vectors per SpMM, basis limit)
MIXED = dict(block=8, lim=96, keep=32, algorithm=1, precond=1, switch_resid=3e-5, refine_lim=32, refine_keep=16)
# the same solver in FP64 (FP64 products, vectors and projections): the
# precision-only baseline, run to the same tolerance
FP64_SAME = dict(block=8, lim=96, keep=32, algorithm=1, precond=1)
# Iterations the reference algorithm (block 10, limit 30) runs on this problem:
# its 400-iteration cap (max(40 * nstates, 200)), which it reaches without
# converging all 10 pairs to 1e-5 (measured with the same algorithm in FP64 on
# the GPU), so CPU samples scaled by it are a lower bound of the CPU solve time.
REF_ITERS_DEFAULT = 400
# DRAM bytes (read + write) of one steady-state k_spmm_f32w<8> launch on this
# workload (launch shape fixed at 8 warps x 8 CTAs per SM, the second launch),
# measured with ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum.
NCU_TRAFFIC_BYTES = {("k_spmm_f32w<8>", "fp44"): 11.86e9 + 64.24e6,
                     # k_tiled, 2 slices per warp, 2 ring slots (the autotuner's choice), second launch
                     ("k_tiled", "fp44"): 8.65e9 + 62.24e6}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for p in self.samples:
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(seconds: float, dist=None, device=None) -> float:
    """Slowest rank's time (replicas: every rank solves its own copy)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


CONFIGS = {"fp44": ("fp", 4, 4, 0, "+", 0.5, 7, "fp44m0s7"), "sd66": ("sd", 6, 6, 0, "+", 0.5, 5, "sd66m0s5"),
           # profiling case: fp44's block lengths (4 protons) with 1,140 neutron blocks (~3 GB stored)
           "fp34": ("fp", 3, 4, 1, "-", 0.5, 7, "fp34m1s7")}


def make_inputs(tmp: str, config: str = "fp44"):
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    sp, nv, zv, tm, par, lam, seed, name = CONFIGS[config]
    return make_system(tmp, SyntheticSystem(sp, nv, zv, tm, par, lam, seed, name=name))[1]


def run_spmm_only(args):
    """SpMM kernel alone (for profiling): build H, time --steps launches."""
    import torch
    import cosmo_gb300 as cg
    torch.cuda.set_device(0)
    tmp = tempfile.mkdtemp(prefix="cg_spmm_")
    prob = cg.Problem(make_inputs(tmp, args.config))
    basis = cg.ManyBodyStates(prob)
    prec = cg.CG_PREC_FP64 if args.precision == "fp64" else cg.CG_PREC_FP32
    H = cg.Hamiltonian(prob, basis, prec)
    tune = None
    if prec == cg.CG_PREC_FP32:
        if args.tuning:
            w, c = (int(v) for v in args.tuning.split("x"))
            cg._check(cg.lib().cg_spmm_set_tuning(H._h, w, c))
            tune = {"warps": w, "ctas_per_sm": c, "fixed": True}
        else:
            tune = H.autotune(args.nvec)
        if args.format:
            H.set_format(cg.CG_FORMAT_TILED if args.format == "tiled" else cg.CG_FORMAT_ROWS)
            tune["format_fixed"] = args.format
        if args.tiled_shape:
            r, st = (int(v) for v in args.tiled_shape.split("x"))
            H.set_tiled_shape(r, st)
            tune["tiled_shape"] = args.tiled_shape
        spmm_s, alg = spmm_roofline(cg, H, args.nvec, reps=args.steps, warm=args.warmup)
    else:
        spmm_s, alg = spmm_roofline(cg, H, args.nvec, reps=args.steps, warm=args.warmup, fp64=True)
    peak, kind = measured_peaks()
    print(json.dumps({"mode": "spmm", "config": args.config, "precision": args.precision, "nvec": args.nvec,
                      "n": H.n, "nnz_full": int(H.info.nnz_full), "build_seconds": H.info.build_seconds,
                      "launch_ms": spmm_s * 1e3, "alg_bytes": alg,
                      "achieved_gbs": alg / spmm_s / 1e9, "peak_gbs": peak, "frac": alg / spmm_s / 1e9 / peak,
                      "tuning": tune}))


def run_batched_only(args):
    """The 64-problem batched solve alone (for profiling): build the batch,
    then --steps solves; prints build and per-solve times."""
    import torch
    import cosmo_gb300 as cg
    from cosmo_gb300.synthetic import batched_sd_systems, make_system
    torch.cuda.set_device(0)
    tmp = tempfile.mkdtemp(prefix="cg_batch_")
    probs = [cg.Problem(make_system(tmp, s)[1]) for s in batched_sd_systems()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = cg.Batch(probs)
    torch.cuda.synchronize()
    build = time.perf_counter() - t0
    times = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        eig, res, nconv, st = b.solve(5)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    print(json.dumps({"mode": "batched", "problems": len(probs), "build_seconds": build, "solve_seconds": times,
                      "iterations_fp32": int(st.iterations_fp32), "iterations_fp64": int(st.iterations_fp64),
                      "states_converged": int(nconv.sum()), "max_resid": float(np.nanmax(res))}))


def spmm_roofline(cg, h, b: int, reps: int = 20, warm: int = 3, fp64: bool = False):
    """Average device time of one SpMM launch (b vectors) from CUDA events on the
    library's stream, and its algorithmic bytes per launch: stored entries x
    (value + 4-byte column) + row pointers + the input and output vectors."""
    import torch
    n = h.n
    esz = 8 if fp64 else 4
    ld = (8 if b <= 8 else 16) if not fp64 else (b + 3) // 4 * 4
    dt = torch.float64 if fp64 else torch.float32
    prec = cg.CG_PREC_FP64 if fp64 else cg.CG_PREC_FP32
    x = torch.randn(n, ld, device="cuda", dtype=dt)
    y = torch.empty(n, ld, device="cuda", dtype=dt)
    torch.cuda.synchronize()
    st = torch.cuda.ExternalStream(h.stream)
    for _ in range(warm):
        h.spmm_device(x.data_ptr(), ld, y.data_ptr(), ld, b, prec)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        h.spmm_device(x.data_ptr(), ld, y.data_ptr(), ld, b, prec)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nnz = int(h.info.nnz_full)
    fi = None if fp64 else h.format_info()
    if fi and fi["format"] == cg.CG_FORMAT_TILED and b <= 8:
        # tiled: 16-bit column + FP32 value per stored entry (padding excluded;
        # a scaled-identity tile reads one value), x read once (8-wide rows),
        # y written, unit descriptors and run offsets
        alg = ((nnz - int(fi["ident_entries"])) * 6 + int(fi["ident_tiles"]) * 8 + n * 8 * 4 + n * b * 4
               + int(fi["meta_bytes"]))
        kernel = "k_tiled"
    else:
        alg = nnz * (esz + 4) + (n + 1) * 8 + n * b * esz * 2
        kernel = ("k_spmm_fp64" if fp64 else f"k_spmm_f32w<{8 if b <= 8 else 16}>")
    del x, y
    spmm_roofline.kernel = kernel
    return ms * 1e-3, alg


def per_state_errors(cg, basis, eig_mixed, vecs_mixed, r64, twom: int):
    """Eigenvalue and <J-J+> error of every mixed-precision state against the
    FP64 solve (states paired in energy order)."""
    jm, _ = cg.jt_expectations(basis, vecs_mixed)
    j6, _ = cg.jt_expectations(basis, r64.vecs)
    return [{"E_fp64": float(r64.eig[i]), "dE": float(eig_mixed[i] - r64.eig[i]), "JJ_fp64": float(j6[i]),
             "dJJ": float(jm[i] - j6[i]), "twoJ": cg.jj_spin(j6[i], twom), "resid_fp64": float(r64.resid[i])}
            for i in range(len(r64.eig))]


def run_ours(args):
    import torch
    import cosmo_gb300 as cg
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp(prefix="cg_bench_")
    xml = make_inputs(tmp)
    prob = cg.Problem(xml)
    basis = cg.ManyBodyStates(prob)
    H = cg.Hamiltonian(prob, basis, cg.CG_PREC_FP32)
    # launch-shape choice, kept in the tuning cache a user's later runs read
    tune_cache = os.path.join(tmp, "spmm_tuning.json")
    tuning = H.autotune(MIXED["block"], cache=tune_cache)
    kw = dict(precision=cg.CG_PREC_FP32, tol_resid=TOL, **MIXED)

    for _ in range(args.warmup):
        cg.davidson_diagonalization(H, NSTATES, want_vectors=False, **kw)
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = cg.launch_count()
    t0 = time.perf_counter()
    results = []
    for _ in range(args.steps):
        results.append(cg.davidson_diagonalization(H, NSTATES, want_vectors=False, **kw))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    launches = cg.launch_count() - l0
    clocks.stop()
    elapsed = max_over_ranks(t1 - t0, dist, "cuda")
    per_solve = elapsed / args.steps
    last = results[-1]

    # end to end through the C ABI: host interaction -> basis -> H -> solve -> eigenvectors to host
    e2e_times = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        p2 = cg.Problem(xml)
        b2 = cg.ManyBodyStates(p2)
        h2 = cg.Hamiltonian(p2, b2, cg.CG_PREC_FP32)
        h2.autotune(MIXED["block"], cache=tune_cache)  # cached choice, no timing
        r2 = cg.davidson_diagonalization(h2, NSTATES, want_vectors=True, **kw)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - s0)
        h2d = int(p2.info.n_one_body) * 16 + int(p2.info.n_two_body) * 24
        d2h = r2.vecs.nbytes + 3 * 8 * NSTATES
        mixed_vecs, mixed_eig = r2.vecs, r2.eig
        del h2, b2, p2
    e2e = statistics.median(e2e_times)

    # SpMM roofline (FP32 mixed kernel, block of 10 vectors)
    spmm_s, alg_bytes = spmm_roofline(cg, H, MIXED["block"])
    # the product's dominant traffic is one 32-byte vector gather per stored
    # entry; its ceiling is the device's random-gather rate over a table the
    # size of the vector block (L2 resident)
    gathers = int(H.info.nnz_full)
    g_peak = cg.gather_ceiling(int(H.n), 1)
    kernel_name = spmm_roofline.kernel
    fmt_info = H.format_info()
    rows_ms = None
    if fmt_info["format"] == cg.CG_FORMAT_TILED:
        # the row-wise kernel on the same matrix, for comparison (and its gather rate)
        H.set_format(cg.CG_FORMAT_ROWS)
        rows_s, _ = spmm_roofline(cg, H, MIXED["block"])
        H.set_format(cg.CG_FORMAT_TILED)
        rows_ms = rows_s * 1e3
        spmm_roofline.kernel = kernel_name
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / spmm_s / 1e9
    # the same launch against the bytes of a stored FP32 value + 16-bit
    # tile-local row and column per entry (every one of the nnz_full entries,
    # scaled-identity ones included) plus x and y of the b vectors: the layout
    # of the reference's CSB with FP32 values, which this kernel's own layout
    # (16-bit column only, scaled-identity tiles as one value) undercuts
    csb_bytes = int(H.info.nnz_full) * 8 + 2 * int(H.n) * MIXED["block"] * 4

    # FP64 GPU Davidson on an FP64 matrix: (1) the same solver in FP64 to the
    # same tolerance (the precision-only baseline), (2) the reference control
    # flow (block 10, limit 30, one-vector Gram-Schmidt) to its iteration cap
    fp64 = None
    if not args.skip_fp64:
        H64 = cg.Hamiltonian(prob, basis, cg.CG_PREC_FP64)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        r64 = cg.davidson_diagonalization(H64, NSTATES, want_vectors=True, precision=cg.CG_PREC_FP64,
                                          tol_resid=TOL, **FP64_SAME)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - s0
        fp64 = dict(workload="same matrix stored in FP64, same solver (block 8, limit 64, keep 32, residual-driven) "
                             "with FP64 products, vectors and projections, to the same tolerance",
                    seconds=t64, iterations=int(r64.stats.iterations), converged=int(r64.stats.converged),
                    spmm_seconds=r64.stats.spmm_seconds, max_resid=float(r64.resid.max()),
                    precision_only_speedup=t64 / per_solve,
                    per_state=per_state_errors(cg, basis, mixed_eig, mixed_vecs, r64, 0))
        fp64["max_abs_dE"] = max(abs(x["dE"]) for x in fp64["per_state"])
        fp64["max_abs_dJJ"] = max(abs(x["dJJ"]) for x in fp64["per_state"])
        del r64
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        r0 = cg.davidson_diagonalization(H64, NSTATES, want_vectors=False, precision=cg.CG_PREC_FP64,
                                         tol_resid=TOL, maxiter=args.fp64_maxiter)
        torch.cuda.synchronize()
        t0r = time.perf_counter() - s0
        fp64["reference_control_flow"] = dict(
            seconds=t0r, iterations=int(r0.stats.iterations), converged=int(r0.stats.converged),
            spmm_seconds=r0.stats.spmm_seconds, speedup=t0r / per_solve,
            max_abs_dE_converged=float(np.abs(r0.eig - last.eig)[r0.resid <= TOL].max(initial=0.0)),
            note="the reference algorithm (block 10, limit 30, one-vector Gram-Schmidt, critc stall test) in FP64; "
                 "it stops at its iteration cap with the converged count shown")
        del H64, r0

    # CPU baseline: the reference algorithm restated in C (oracle), FP64 CSB, on
    # this host's cores, bounded sample scaled to a full solve
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline_from_gpu_matrix(H, fp64["reference_control_flow"]["iterations"] if fp64 else None)

    hinfo = {"n": int(H.n), "nnz_full": int(H.info.nnz_full), "nnz_upper": int(H.info.nnz_upper),
             "build_seconds": H.info.build_seconds, "device_bytes": int(H.info.device_bytes)}
    batched = None
    virtual = None
    sd66 = None
    if rank == 0 and not args.skip_batched:
        batched = batched_subbench(cg)
    if rank == 0 and not args.skip_sd66:
        sd66 = sd66_subbench(cg)
    if rank == 0 and not args.skip_virtual:
        del H
        torch.cuda.empty_cache()
        virtual = virtual_subbench(cg, fp64["reference_control_flow"]["iterations"] if fp64 else None)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": per_solve, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_solve * 1e3, "higher_is_better": False,
        "scaling": "replicas", "vs_baseline": None, "dtype": "fp32 storage / fp64 projection",
        "data": "synthetic (seeded Gaussian TBMEs)", "config": WORKLOAD,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": NCU_TRAFFIC_BYTES.get((kernel_name, "fp44")),
                     "kernel": kernel_name,
                     "peak_source": peak_kind, "launch_ms": spmm_s * 1e3, "alg_bytes": alg_bytes},
        "roofline_csb_layout": {"achieved": csb_bytes / spmm_s / 1e9, "peak": peak, "unit": "GB/s",
                                "frac": csb_bytes / spmm_s / 1e9 / peak, "alg_bytes": csb_bytes,
                                "kernel": kernel_name,
                                "note": "same launch; bytes of an FP32 value + u16 row + u16 column per entry "
                                        "(all nnz_full entries) + x + y"},
        "gather_roofline": ({"achieved": gathers / (rows_ms * 1e-3), "peak": g_peak, "unit": "gathers/s",
                             "frac": gathers / (rows_ms * 1e-3) / g_peak, "kernel": "k_spmm_f32w<8>",
                             "launch_ms": rows_ms,
                             "note": "row-wise kernel on the same matrix: 32-byte L2 gathers of the 8-vector "
                                     "block, probe over an n-row table"} if rows_ms else
                            {"achieved": gathers / spmm_s, "peak": g_peak, "unit": "gathers/s",
                             "frac": gathers / spmm_s / g_peak,
                             "note": "32-byte gathers of the 8-vector block, probe over an n-row table"}),
        "spmm_format": {k: (int(v) if not isinstance(v, bool) else v) for k, v in fmt_info.items()},
        "clocks": clocks.summary(),
        "spmm_tuning": {k: v for k, v in tuning.items() if k != "candidates"},
        "solve": {"iterations": int(last.stats.iterations), "refine_iterations": int(last.stats.refine_iterations),
                  "matvecs": int(last.stats.matvecs), "converged": int(last.stats.converged),
                  "max_resid": float(last.resid.max()), "spmm_seconds": last.stats.spmm_seconds,
                  "eig": [round(float(x), 8) for x in last.eig]},
        "hamiltonian": hinfo,
        "fp64_gpu_davidson": fp64,
        "cpu_baseline": cpu,
        "batched_sd64": batched,
        "sd66_fp64_block4": sd66,
        "virtual_fp55": virtual,
    }
    if fp64:
        line["speedup_vs_fp64_gpu"] = fp64["seconds"] / per_solve
        line["speedup_vs_fp64_gpu_reference_control_flow"] = fp64["reference_control_flow"]["seconds"] / per_solve
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def batched_subbench(cg):
    """64 independent sd-shell problems (dimensions 0..67,251), lowest 5
    eigenpairs each to resid <= 1e-5: the batched lockstep solve (one CUDA graph
    launch per iteration for all problems) against the same problems solved one
    after another with the single-problem mixed solver."""
    import torch
    from cosmo_gb300.synthetic import batched_sd_systems, make_system
    tmp = tempfile.mkdtemp(prefix="cg_batch_")
    probs = [cg.Problem(make_system(tmp, s)[1]) for s in batched_sd_systems()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = cg.Batch(probs)
    build = time.perf_counter() - t0
    dims = b.dims()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eig, res, nconv, st = b.solve(5)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    wanted = int(sum(min(5, int(d)) for d in dims))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in probs:
        bb = cg.ManyBodyStates(p)
        if bb.n <= 64:  # the batched path solves these exactly as well
            continue
        h = cg.Hamiltonian(p, bb, cg.CG_PREC_FP32)
        cg.davidson_diagonalization(h, 5, want_vectors=False, precision=cg.CG_PREC_FP32, tol_resid=TOL,
                                    block=5, lim=30)
    torch.cuda.synchronize()
    seq = time.perf_counter() - t0
    return {"problems": len(probs), "rows": int(dims.sum()), "max_dim": int(dims.max()),
            "build_seconds": build, "solve_seconds": min(times), "build_plus_solve_seconds": build + min(times),
            "iterations_fp32": int(st.iterations_fp32), "iterations_fp64": int(st.iterations_fp64),
            "graph_launches": int(st.graph_launches), "kernels_per_graph": int(st.graph_kernels),
            "spmm_autotuned_shape": {"warps_per_cta": int(st.spmm_warps), "ctas_per_sm": int(st.spmm_ctas_per_sm),
                                     "tune_seconds": float(st.spmm_tune_seconds)},
            "launches": int(st.launches), "states_converged": int(nconv.sum()), "states_wanted": wanted,
            "max_resid": float(np.nanmax(res)),
            "sequential_build_plus_solve_seconds": seq,
            "speedup_vs_sequential": seq / (build + min(times))}


def sd66_subbench(cg):
    """sd-shell 6p+6n M=0 (n = 93,710): plain FP64 stored H and block Davidson
    for the 10 lowest eigenpairs with block 4 and basis limit 40, as the
    reference control flow on the GPU, as the residual-driven solver in FP64,
    and the mixed solve; the same reference control flow on the host cores
    (oracle restatement, all threads) run to its own stop, not sampled."""
    import torch
    from oracle import oracle as O
    tmp = tempfile.mkdtemp(prefix="cg_sd66_")
    xml = make_inputs(tmp, "sd66")
    prob = cg.Problem(xml)
    basis = cg.ManyBodyStates(prob)
    out = {"workload": "sd-shell 6p+6n M=0, FP64 CSB, lowest 10 eigenpairs, block 4, basis limit 40",
           "n": int(basis.n)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h64 = cg.Hamiltonian(prob, basis, cg.CG_PREC_FP64)
    torch.cuda.synchronize()
    out["gpu_build_seconds"] = time.perf_counter() - t0
    runs = {}
    for name, kw in (("fp64_reference_control_flow", dict(algorithm=0)),
                     ("fp64_residual_driven", dict(algorithm=1, keep=20, precond=1))):
        cg.davidson_diagonalization(h64, NSTATES, want_vectors=False, precision=cg.CG_PREC_FP64, tol_resid=TOL,
                                    block=4, lim=40, **kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = cg.davidson_diagonalization(h64, NSTATES, want_vectors=False, precision=cg.CG_PREC_FP64, tol_resid=TOL,
                                        block=4, lim=40, **kw)
        torch.cuda.synchronize()
        runs[name] = r
        out[name] = {"seconds": time.perf_counter() - t0, "iterations": int(r.stats.iterations),
                     "converged": int(r.stats.converged), "max_resid": float(r.resid.max())}
    h32 = cg.Hamiltonian(prob, basis, cg.CG_PREC_FP32)
    kw = dict(precision=cg.CG_PREC_FP32, tol_resid=TOL, **MIXED)
    cg.davidson_diagonalization(h32, NSTATES, want_vectors=False, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rm = cg.davidson_diagonalization(h32, NSTATES, want_vectors=False, **kw)
    torch.cuda.synchronize()
    ref = runs["fp64_residual_driven"]
    out["mixed"] = {"seconds": time.perf_counter() - t0, "iterations": int(rm.stats.iterations),
                    "converged": int(rm.stats.converged), "max_abs_dE_vs_fp64": float(np.abs(rm.eig - ref.eig).max())}

    def nearest(eig, resid):
        """converged pairs matched to the nearest FP64 eigenvalue (a control
        flow that stalls a state can converge a higher one in its place), and
        how many of the 10 lowest FP64 states no converged pair matches"""
        ok = np.asarray(resid) <= TOL
        e = np.asarray(eig)[ok]
        if not len(e):
            return 0.0, NSTATES
        d = np.abs(e[:, None] - ref.eig[None, :])
        return float(d.min(axis=1).max()), int(NSTATES - len(set(d.argmin(axis=1).tolist())))
    r0 = runs["fp64_reference_control_flow"]
    dmax, miss = nearest(r0.eig, r0.resid)
    out["fp64_reference_control_flow"].update(max_abs_dE_converged_vs_nearest_fp64=dmax,
                                              lowest_states_not_found=miss)
    out["eig"] = [round(float(x), 8) for x in ref.eig]
    # the reference control flow on the host cores, run to its own stop
    rp, c, v = h64.upper_rows()
    csb = O.CSB(rp, c, v)
    del rp, c, v
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    rc = csb.davidson(NSTATES, block=4, lim=40, critr=TOL, nthreads=cores)
    cpu_s = time.perf_counter() - t0
    dmax, miss = nearest(rc["eig"], rc["resid"])
    out["cpu_reference_control_flow"] = {
        "seconds": cpu_s, "iterations": int(rc["iterations"]), "converged": int((rc["resid"] <= TOL).sum()),
        "cores": cores, "kind": "port", "max_abs_dE_converged_vs_nearest_fp64": dmax,
        "lowest_states_not_found": miss}
    out["speedup_gpu_reference_control_flow_vs_cpu"] = cpu_s / out["fp64_reference_control_flow"]["seconds"]
    out["speedup_mixed_vs_cpu"] = cpu_s / out["mixed"]["seconds"]
    return out


def virtual_subbench(cg, fp64_iters):
    """fp-shell 5p+5n M=0 (n = 18,600,516) with the on-the-fly product: the
    products alone, the mixed solve (FP32 products, FP64 projection and
    refinement) to 10 eigenpairs, and the plain FP64 on-the-fly Davidson (the
    reference algorithm) timed over a bounded sample of iterations."""
    import torch
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    tmp = tempfile.mkdtemp(prefix="cg_fp55_")
    xml = make_system(tmp, SyntheticSystem("fp", 5, 5, 0, "+", 0.5, 8, name="fp55m0s8"))[1]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prob = cg.Problem(xml)
    basis = cg.ManyBodyStates(prob)
    hv = cg.Hamiltonian(prob, basis, cg.CG_PREC_FP32, virtual=True)
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    n = hv.n
    conn = int(hv.info.nnz_full)
    st = torch.cuda.ExternalStream(hv.stream)

    def product_ms(prec, vb, reps):
        dt = torch.float32 if prec == cg.CG_PREC_FP32 else torch.float64
        x = torch.randn(n, vb, dtype=dt, device="cuda")
        y = torch.zeros(n, vb, dtype=dt, device="cuda")
        torch.cuda.synchronize()
        hv.spmm_device(x.data_ptr(), vb, y.data_ptr(), vb, vb, prec)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            hv.spmm_device(x.data_ptr(), vb, y.data_ptr(), vb, vb, prec)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms32 = product_ms(cg.CG_PREC_FP32, 8, 5)
    ms64 = product_ms(cg.CG_PREC_FP64, 4, 2)
    msdf = product_ms(cg.CG_PREC_REFINE, 4, 2)  # double-float (refinement) product
    kw = dict(precision=cg.CG_PREC_FP32, tol_resid=TOL, **MIXED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = cg.davidson_diagonalization(hv, NSTATES, want_vectors=True, **kw)
    torch.cuda.synchronize()
    mixed = time.perf_counter() - t0
    # the same solver in FP64 on the FP64 on-the-fly product, to the same tolerance
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r64 = cg.davidson_diagonalization(hv, NSTATES, want_vectors=True, precision=cg.CG_PREC_FP64, tol_resid=TOL,
                                      **FP64_SAME)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    states = per_state_errors(cg, basis, r.eig, r.vecs, r64, 0)
    fp64_same = {"seconds": t64, "iterations": int(r64.stats.iterations), "converged": int(r64.stats.converged),
                 "spmm_seconds": r64.stats.spmm_seconds, "max_resid": float(r64.resid.max()),
                 "precision_only_speedup": t64 / mixed, "per_state": states,
                 "max_abs_dE": max(abs(x["dE"]) for x in states), "max_abs_dJJ": max(abs(x["dJJ"]) for x in states)}
    del r64
    # the reference control flow in FP64 on the on-the-fly product: a bounded sample of iterations
    t0 = time.perf_counter()
    rr = cg.davidson_diagonalization(hv, NSTATES, want_vectors=False, precision=cg.CG_PREC_FP64, maxiter=4)
    torch.cuda.synchronize()
    per_it = (time.perf_counter() - t0) / max(1, int(rr.stats.iterations))
    its = fp64_iters or REF_ITERS_DEFAULT
    return {"workload": "fp-shell 5p+5n M=0, lowest 10 eigenpairs, resid<=1e-5, on-the-fly product",
            "n": int(n), "connections_per_product": conn, "table_bytes": int(hv.info.device_bytes),
            "setup_seconds": setup, "fp32_product_ms_8vec": ms32, "fp64_product_ms_4vec": ms64,
            "double_float_product_ms_4vec": msdf,
            "product_timing_note": "device API calls: pack kernel + product, staging buffer allocated per call",
            "fp32_connection_vectors_per_s": conn * 8 / (ms32 * 1e-3),
            "fp64_connection_vectors_per_s": conn * 4 / (ms64 * 1e-3),
            "mixed_solve_seconds": mixed, "mixed_iterations": int(r.stats.iterations),
            "mixed_refine_iterations": int(r.stats.refine_iterations), "mixed_converged": int(r.stats.converged),
            "mixed_max_resid": float(r.resid.max()), "eig": [round(float(x), 8) for x in r.eig],
            "fp64_same_solver": fp64_same,
            "fp64_reference_control_flow": {
                "seconds_per_iteration": per_it, "estimated_seconds": per_it * its,
                "sample": f"{int(rr.stats.iterations)} iterations of the reference algorithm (block 10, lim 30) in "
                          f"FP64 on the on-the-fly product, scaled to {its} iterations (its cap, reached without "
                          f"convergence on fp 4+4)",
                "speedup_estimate": per_it * its / mixed}}


REF_ALGO = ("the reference control flow (DavidsonDiagonalization defaults: block 10, basis limit 30, "
            "thresholds 1e-15/1e-12/1e-8) on an FP64 CSB pull-form product")


def reference_davidson_sample(csb, warm: int, timed: int, cores: int, budget: float = 600.0):
    """One continuous run of the reference Davidson (oracle restatement, all
    host threads) for warm + timed iterations; the mean duration of the timed
    iterations (after the first `warm`), with the counts actually run."""
    r = csb.davidson(NSTATES, nthreads=cores, maxiter=warm + timed, time_budget=budget)
    ends = np.asarray(r["iter_end"])
    k = len(ends)
    if k == 0:
        raise RuntimeError("reference Davidson sample ran no iteration")
    w = min(warm, k - 1)
    dur = np.diff(np.concatenate([[0.0], ends]))[w:]
    return float(dur.mean()), {"iterations_run": k, "timed_iterations": int(len(dur)), "warmup_iterations": w,
                               "collapses": int(r["collapses"]), "sample_seconds": float(dur.sum())}


def sample_text(per: float, info: dict, its: int, cores: int) -> str:
    return (f"one continuous run of {REF_ALGO}, {cores} host threads: iterations {info['warmup_iterations'] + 1}.."
            f"{info['iterations_run']} ({info['timed_iterations']} iterations, {info['collapses']} basis collapses "
            f"in the run) measured at {per:.3f} s/iteration; value = that x {its}, the iteration cap at which this "
            f"algorithm stops on this problem without converging all 10 pairs to resid<=1e-5 (GPU FP64 run of the "
            f"same control flow), so a lower bound of its time to tolerance")


def cpu_baseline_from_gpu_matrix(H, ref_iters, warm: int = 3, timed: int = 12):
    """The bench line's cpu_baseline: the oracle's reference Davidson on the
    GPU-built matrix (its upper triangle copied to the host)."""
    from oracle import oracle as O
    rp, c, v = H.upper_rows()
    csb = O.CSB(rp, c, v)
    del rp, c, v
    cores = os.cpu_count() or 1
    per, info = reference_davidson_sample(csb, warm, timed, cores)
    its = ref_iters if ref_iters else REF_ITERS_DEFAULT
    return {"value": per * its, "unit": "s", "cores": cores, "kind": "port", "sample": sample_text(per, info, its, cores),
            "seconds_per_iteration": per, **info}


def run_reference(args):
    """The reference's CPU path on the host cores, with nothing from the
    product library: the oracle's own XML/interaction restatement, the oracle
    basis and row builder (C, OpenMP), the reference-layout CSB and the
    reference Davidson.  Each step is one Davidson iteration of one continuous
    run (warm-up iterations untimed)."""
    rank, world, local = env_rank()
    if rank != 0:
        return
    from oracle import interaction as OI
    from oracle import oracle as O
    tmp = tempfile.mkdtemp(prefix="cg_ref_")
    xml = make_inputs(tmp, args.config)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    sysd, k1, v1, k2, v2 = OI.operator_terms(xml)
    t1 = time.perf_counter()
    z = O.basis(sysd.sps, sysd.nv + sysd.zv, sysd.twom, sysd.nv - sysd.zv, sysd.parity)
    t2 = time.perf_counter()
    rp, c, v = O.build_upper(len(sysd.sps), k1, v1, k2, v2, z, nthreads=cores)
    csb = O.CSB(rp, c, v)
    t3 = time.perf_counter()
    nnz = int(rp[-1])
    del rp, c, v, z
    per, info = reference_davidson_sample(csb, args.warmup, args.steps, cores)
    its = args.ref_iters
    value = per * its
    loaded = sorted({ln.split()[-1] for ln in open("/proc/self/maps") if ln.rstrip().endswith(".so")
                     and HERE in ln})
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": False,
            "config": WORKLOAD,
            "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port",
                             "sample": sample_text(per, info, its, cores)},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "seconds_per_iteration": per, **info,
            "setup_seconds": {"interaction": t1 - t0, "basis": t2 - t1, "csb_build": t3 - t2},
            "nnz_upper": nnz, "repo_libraries_loaded": [os.path.relpath(x, HERE) for x in loaded]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--fp64-maxiter", type=int, default=400)
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-virtual", action="store_true")
    ap.add_argument("--skip-sd66", action="store_true")
    ap.add_argument("--ref-iters", type=int, default=REF_ITERS_DEFAULT)
    ap.add_argument("--mode", default="solve", choices=["solve", "spmm", "batched"])
    ap.add_argument("--config", default="fp44", choices=sorted(CONFIGS))
    ap.add_argument("--nvec", type=int, default=10)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--tuning", default=None, help="fixed launch shape WARPSxCTAS for --mode spmm")
    ap.add_argument("--format", default=None, choices=["rows", "tiled"], help="fixed SpMM storage for --mode spmm")
    ap.add_argument("--tiled-shape", default=None, help="tiled product shape SLICESxSTAGES for --mode spmm")
    args = ap.parse_args()
    if args.mode == "spmm":
        run_spmm_only(args)
    elif args.mode == "batched":
        run_batched_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
