"""Benchmark: q->0 Tamm-Dancoff BSE build + diagonalization + eps2 on one GB300.

Workload (one "step" = one BSE solve): the magnetic spinful 4-orbital honeycomb model
(2 sites x 2 spins, exchange splitting 0.5 eV, SOC 0.05 eV, random NNN hoppings
sigma = 0.1 eV, seed 1234) on a 24x24 grid, 2 valence x 2 conduction bands, N_BSE = 2304,
Rytova-Keldysh W + bare 2-D exchange, eps2 on 2000 points over 0-8 eV with 0.05 eV
broadening.  Mixed precision: complex64 kernel build and FP32 eigensolve, FP64
Rayleigh-Ritz refinement of the lowest 256 excitons.  Inputs are synthetic (seeded).

value  = device time per solve (CUDA events on the library's stream), inputs resident
e2e    = the same solve through the C ABI with host buffers: context creation (model
         upload), solve, copy-back of eigenvalues and eps, destroy -- wall clock
Other keys: the plain FP64 GPU path (cuSOLVER zheevd) on the same problem, the max
eigenvalue error of the mixed path against it, the roofline of the dominant kernel (the
tridiagonal reduction of the own eigensolver; the kernel build as a second figure), the
eigensolve rate in the 14.7 N^3 flop unit, the CPU oracle baseline and the SM clocks
sampled during the timed region.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

OMEGA = np.arange(2000) * 8.0 / 2000
GAMMA = 0.05
WORKLOAD = "magnetic4_24x24_2v2c"
METRIC = "BSE build+diag wall time and eps2 grad time at N_BSE; error vs FP64"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.dev = device_index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().strip().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _l2_flush_buffer():
    import torch
    return torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2


def _flush(buf):
    buf.zero_()
    import torch
    torch.cuda.synchronize()


def _problem(pkg_synth, grid=24, **kw):
    return pkg_synth.magnetic4_problem(grid=grid, **kw)


def _model_bytes(m):
    return int(sum(a.nbytes for a in (m.r_cart, m.weights, m.h_r, m.centres, m.lattice, m.k_cart, m.g_cart)))


def cpu_oracle_solve_ms(orc, prob, reps=1):
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        orc.solve(prob, OMEGA, GAMMA)
        ts.append((time.perf_counter() - t0) * 1e3)
    return min(ts)


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    orc = entry.load_oracle()
    prob = _problem(synth)
    cores = int(orc.lib().oracle_num_threads())
    for _ in range(args.warmup):
        orc.solve(prob, OMEGA, GAMMA)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.solve(prob, OMEGA, GAMMA)
        ts.append((time.perf_counter() - t0) * 1e3)
    total = sum(ts)
    ms = total / args.steps
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_bse": prob.n_bse, "n_g": prob.ng, "precision": "fp64",
                   "l2": "inputs resident in host memory; CPU run"},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port",
                         "sample": f"full solve of the {WORKLOAD} workload (N_BSE={prob.n_bse}) per step: "
                                   "C++ OpenMP restatement of the reference loops + LAPACK zheevd (scipy)"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    ws, rank, local = _dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BSE_BENCH_GLOO") is None else "gloo")
    import torch
    torch.cuda.set_device(local)
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    gpu.load().bse_set_device(local)
    solver = {"own": 0, "cusolver": 1}[args.solver]
    prob = _problem(synth)
    mixed = dict(precision=1, n_refine=256, eig_solver=solver)
    flush = _l2_flush_buffer()

    # --- device-resident timing (value) ---
    ctx = gpu.BSEContext(prob, **mixed)
    for _ in range(args.warmup):
        ctx.solve(OMEGA, GAMMA)
    ctx.reset_kernel_launches()
    step_ms, build_ms, eig_ms, tri_ms = [], [], [], []
    _barrier(ws)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t_host0 = time.perf_counter()
    for _ in range(args.steps):
        _flush(flush)                                 # outside the solve's events
        E_mixed, e2_mixed, _ = ctx.solve(OMEGA, GAMMA)
        st = ctx.stage_times()
        step_ms.append(st["solve"])
        build_ms.append(st["build"])
        eig_ms.append(st["eig"])
        tri_ms.append(st["eig_tridiag"])
    torch.cuda.synchronize()
    host_s = time.perf_counter() - t_host0
    clk = clocks.stop()
    launches = ctx.kernel_launches()
    stage = ctx.stage_times()
    ctx.close()
    _barrier(ws)
    dev_total = _max_over_ranks(ws, sum(step_ms))
    ms_per_step = dev_total / args.steps
    value = ms_per_step / ws          # whole-job time per solve (each rank solves one problem per step)

    # --- end to end through the C ABI with host buffers (e2e) ---
    e2e_ms = []
    for _ in range(max(1, args.steps)):
        _flush(flush)
        t0 = time.perf_counter()
        with gpu.BSEContext(prob, **mixed) as c2:
            c2.solve(OMEGA, GAMMA)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = _max_over_ranks(ws, sum(e2e_ms)) / len(e2e_ms) / ws
    from bse_gb300.capi import Marshalled
    mm = Marshalled(prob)
    h2d = _model_bytes(mm) + OMEGA.nbytes
    d2h = mm.n_exc * 8 + 2 * OMEGA.nbytes

    # --- plain FP64 GPU path (cuSOLVER zheevd) and the error of the mixed path ---
    with gpu.BSEContext(prob, precision=0, eig_solver=1) as c64:
        c64.solve(OMEGA, GAMMA)
        t64 = []
        for _ in range(max(1, min(3, args.steps))):
            _flush(flush)
            E64, e2_64, _ = c64.solve(OMEGA, GAMMA)
            t64.append(c64.stage_times()["solve"])
    fp64_ms = float(np.median(t64))
    nref = 256
    err_ref = float(np.abs(E_mixed[:nref] - E64[:nref]).max())
    err_all = float(np.abs(E_mixed - E64).max())
    eps2_err = float(np.linalg.norm(e2_mixed - e2_64) / np.linalg.norm(e2_64))

    # --- rooflines.  Dominant kernel (own solver): the one-stage tridiagonal reduction, which reads
    # and rewrites the trailing (n-k-1)^2 block of full complex64 storage for every reflector k:
    # 2 * 8 B * sum_m m^2 per launch.  The 42 MB matrix stays in L2 (ncu: 0.34 MB of DRAM traffic
    # per launch), so the HBM denominator overstates what bounds it; the figure shows how far the
    # latency-bound sweep is from streaming.  Second figure: the build kernel (HBM store of H). ---
    N = prob.n_bse
    nb = prob.model.nw * prob.model.n_spin
    build_bytes = N * N * 8 + 16 * prob.nk * nb * (prob.params.nv + prob.params.nc)   # full c64 store (own solver)
    build_avg_ms = float(np.mean(build_ms))
    tri_bytes = 16 * (N - 1) * N * (2 * N - 1) // 6
    tri_avg_ms = float(np.mean(tri_ms))
    eig_avg_ms = float(np.mean(eig_ms))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    # --- eps2 gradient: 12 hopping/onsite parameters + r0, hand-written adjoint (FP64 forward) ---
    grad_ms = None
    if not args.no_grad:
        from bse_gb300.adjoint import ParamModel, backward, gpu_forward
        from bse_gb300.synth import MAGNETIC4_NOMINAL
        pm = ParamModel.magnetic4()
        wts = np.random.default_rng(11).uniform(0.0, 1.0, size=len(OMEGA))
        fwd = gpu_forward(pm, prob, MAGNETIC4_NOMINAL, 10.0, OMEGA, GAMMA)      # warm-up
        backward(pm, fwd["prob"], fwd, OMEGA, wts, GAMMA)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fwd = gpu_forward(pm, prob, MAGNETIC4_NOMINAL, 10.0, OMEGA, GAMMA)
        backward(pm, fwd["prob"], fwd, OMEGA, wts, GAMMA)
        torch.cuda.synchronize()
        grad_ms = (time.perf_counter() - t0) * 1e3

    # --- CPU baseline (oracle, rank 0) ---
    cpu = None
    if rank == 0 and not args.no_cpu:
        orc = entry.load_oracle()
        cpu_ms = cpu_oracle_solve_ms(orc, prob)
        cpu = {"value": cpu_ms, "unit": "ms", "cores": int(orc.lib().oracle_num_threads()), "kind": "port",
               "sample": f"one full CPU solve of {WORKLOAD} (N_BSE={N}): C++ OpenMP restatement of the "
                         "reference loops + LAPACK zheevd (scipy)"}

    build_gbs = build_bytes / (build_avg_ms * 1e-3) / 1e9
    if args.solver == "own" and N <= 8192:
        tri_gbs = tri_bytes / (tri_avg_ms * 1e-3) / 1e9
        roof = {"kernel": "tridiag_fused_kernel<float2>", "bound": "hbm", "achieved": tri_gbs, "peak": peak,
                "peak_source": peak_src, "unit": "GB/s", "frac": tri_gbs / peak,
                "traffic": 42947840 + 5654784 if N == 2304 else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at N_BSE=2304 "
                                  "(profiles/tridiag_fused_kernel_magnetic4_24x24.md): the 42 MB matrix is read "
                                  "from DRAM once and then stays in L2",
                "alg_bytes_per_launch": int(tri_bytes), "avg_launch_ms": tri_avg_ms}
    else:
        roof = {"kernel": "build_kernel<4,float>", "bound": "hbm", "achieved": build_gbs, "peak": peak,
                "peak_source": peak_src, "unit": "GB/s", "frac": build_gbs / peak, "traffic": None,
                "alg_bytes_per_launch": int(build_bytes), "avg_launch_ms": build_avg_ms}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64+fp64-refine", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_bse": N, "n_k": prob.nk, "n_g": prob.ng, "nw": prob.model.nw,
                       "nv": prob.params.nv, "nc": prob.params.nc, "n_omega": len(OMEGA), "gamma": GAMMA,
                       "precision": "mixed", "n_refine": nref, "eig_solver": args.solver,
                       "parallelism": f"replicas x{ws}",
                       "l2": "flushed between steps (256 MB write); H is 42 MB"},
            "e2e": {"value": e2e_value, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "roofline": roof,
            "roofline_build": {"kernel": "build_kernel<4,float>", "bound": "hbm", "achieved": build_gbs, "peak": peak,
                               "peak_source": peak_src, "unit": "GB/s", "frac": build_gbs / peak, "traffic": None,
                               "alg_bytes_per_launch": int(build_bytes), "avg_launch_ms": build_avg_ms},
            "eig_rate": {"unit": "TFLOP/s", "flop_per_solve": 14.7 * N ** 3, "eig_ms": eig_avg_ms,
                         "value": 14.7 * N ** 3 / (eig_avg_ms * 1e-3) / 1e12,
                         "note": "14.7 N^3 = zhetrd 16/3 + D&C 4/3 + zunmtr 8 (N^3 real flops), the LAPACK-equivalent count"},
            "stages_ms": stage,
            "eps2_grad_ms": grad_ms,
            "eps2_grad_config": "d(sum_s w_s eps2(w_s))/d(12 hopping/onsite, r0), FP64 forward + hand-written adjoint, N_BSE=2304",
            "fp64_gpu_ms": fp64_ms,
            "speedup_vs_fp64_gpu": fp64_ms / ms_per_step,
            "max_eig_err_ev": {"refined_lowest_256": err_ref, "all": err_all},
            "eps2_rel_l2_vs_fp64": eps2_err,
            "host_wall_s": host_s,
            "clocks": clk,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_batch(args):
    """64 seeded 2- to 4-band models, grids 12x12 .. 30x30 (N_BSE 144 .. 3600): aggregate time of
    one batched solve (bse_solve_many, 8 host workers) against the same solves one after another."""
    import torch
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    probs = synth.random_batch_problems(n_models=64, seed=77)
    ctxs = [gpu.BSEContext(p, precision=1, n_refine=64, eig_solver=0) for p in probs]
    gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=8)          # warm-up (workspaces, library modules)
    torch.cuda.synchronize()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=8)
        torch.cuda.synchronize()
        ts.append((time.perf_counter() - t0) * 1e3)
    t0 = time.perf_counter()
    for c in ctxs:
        c.solve(OMEGA, GAMMA)
    seq = (time.perf_counter() - t0) * 1e3
    ns = [p.n_bse for p in probs]
    for c in ctxs:
        c.close()
    print(json.dumps({"metric": "batched BSE build+diag+eps2 wall time (64 models)", "value": float(np.median(ts)),
                      "unit": "ms", "steps": args.steps, "higher_is_better": False, "n_gpus": 1,
                      "config": {"workload": "batch64_rand_2to4band_12to30grid", "n_models": len(probs),
                                 "n_bse_min": min(ns), "n_bse_max": max(ns), "n_bse_sum": sum(ns),
                                 "precision": "mixed", "n_refine": 64, "workers": 8},
                      "sequential_ms": seq, "models_per_s": len(probs) / (float(np.median(ts)) / 1e3)}))
    return 0


def run_large(args):
    """8-orbital model, 4v x 4c, complex64 BSE matrix, FP64 refinement of the lowest 256:
    a mixed solve at 48x48 (N_BSE = 36864) with its FP64 residual bound, and FP64 (cuSOLVER
    zheevd) vs mixed solves at 12x12 and 24x24 (N_BSE = 2304, 9216) for the same-size eigenvalue
    errors and the N^3 extrapolation of the plain FP64 GPU time to N_BSE = 36864."""
    import torch
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    out = {"metric": "BSE build+diag wall time at N_BSE=36864 (mixed) vs plain FP64 GPU path", "unit": "ms",
           "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
           "config": {"workload": "orb8_48x48_4v4c", "precision": "mixed", "n_refine": 256, "eig_solver": "own"}}
    small = {}
    for grid in (12, 24):
        prob = synth.orb8_problem(grid=grid)
        with gpu.BSEContext(prob, precision=0, eig_solver=1) as c64:
            c64.solve(OMEGA, GAMMA)
            E64, e2_64, _ = c64.solve(OMEGA, GAMMA)
            t64 = c64.stage_times()["solve"]
        with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as cm:
            cm.solve(OMEGA, GAMMA)
            Em, e2m, _ = cm.solve(OMEGA, GAMMA)
            tm = cm.stage_times()
            dg = cm.diagnostics()
        small[prob.n_bse] = {"fp64_cusolver_ms": t64, "mixed_own_ms": tm["solve"], "mixed_stages_ms": tm,
                             "max_err_refined_256_ev": float(np.abs(Em[:256] - E64[:256]).max()),
                             "max_err_all_ev": float(np.abs(Em - E64).max()),
                             "eps2_rel_l2": float(np.linalg.norm(e2m - e2_64) / np.linalg.norm(e2_64)),
                             "max_refined_residual_ev": dg["max_refined_residual"], "clusters": dg["clusters"]}
        print(json.dumps({"n_bse": prob.n_bse, **small[prob.n_bse]}), file=sys.stderr, flush=True)
    prob = synth.orb8_problem(grid=48)
    with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as cm:
        t0 = time.perf_counter()
        cm.solve(OMEGA, GAMMA)
        first = (time.perf_counter() - t0) * 1e3
        if args.steps > 1:
            cm.solve(OMEGA, GAMMA)
        st = cm.stage_times()
        dg = cm.diagnostics()
    n1, n2 = 2304, 9216
    expo = math.log(small[n2]["fp64_cusolver_ms"] / small[n1]["fp64_cusolver_ms"]) / math.log(n2 / n1)
    fp64_est = small[n2]["fp64_cusolver_ms"] * (36864 / n2) ** 3
    out.update({"value": st["solve"], "ms_per_step": st["solve"], "first_solve_wall_ms": first, "stages_ms": st,
                "n_bse": prob.n_bse, "max_refined_residual_ev": dg["max_refined_residual"],
                "clusters": dg["clusters"], "fp64_cusolver_ms_extrapolated_n3": fp64_est,
                "fp64_growth_exponent_2304_9216": expo, "speedup_vs_fp64_gpu_extrapolated": fp64_est / st["solve"],
                "smaller_sizes": small})
    print(json.dumps(out))
    return 0


def run_coupled(args):
    """Full BSE (tamm_dancoff = 0, coupling block of add_coupling_part) on the magnetic4 24x24 2v2c
    model: FP64 build of the 2N = 4608 matrix and the structure-preserving solve (Cholesky of
    [[A, B], [B*, A*]], own eigensolver on L^H J L) through bse_solve, cuSOLVER heevd of the same
    L^H J L as the cross-check; the CPU oracle (the reference's route: eig_gen of the 2N x 2N matrix,
    inverse overlap spectrum) is timed on the 12x12 model (2N = 1152) and scaled by N^3."""
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    prob = synth.magnetic4_problem(grid=24)
    N = prob.n_bse
    with gpu.BSEContext(prob, tamm_dancoff=0, precision=0, eig_solver=0) as c:
        for _ in range(max(args.warmup, 1)):
            c.solve(OMEGA, GAMMA)
        ts = []
        for _ in range(max(args.steps, 1)):
            E, e2, _ = c.solve(OMEGA, GAMMA)
            ts.append(c.stage_times()["solve"])
        st = c.stage_times()
    with gpu.BSEContext(prob, tamm_dancoff=0, precision=0, eig_solver=1) as c2:
        c2.solve(OMEGA, GAMMA)
        E2, e2b, _ = c2.solve(OMEGA, GAMMA)
        t_cus = c2.stage_times()["solve"]
    # mixed precision: FP32 solve of -L^-1 J L^-H, FP64 refinement of the lowest 256 positive pairs
    with gpu.BSEContext(prob, tamm_dancoff=0, precision=1, eig_solver=0, n_refine=256) as c3:
        c3.solve(OMEGA, GAMMA)
        tm = []
        for _ in range(max(args.steps, 1)):
            Em, e2m, _ = c3.solve(OMEGA, GAMMA)
            tm.append(c3.stage_times()["solve"])
        stm = c3.stage_times()
        dgm = c3.diagnostics()
    out = {"metric": "full-BSE (coupling block) build+diag+eps wall time at N_BSE=2304 (2N=4608, FP64)",
           "value": float(np.median(ts)), "unit": "ms", "higher_is_better": False, "n_gpus": 1,
           "steps": len(ts), "data": "synthetic", "dtype": "c128",
           "config": {"workload": "magnetic4_24x24_2v2c_full_bse", "n_bse": N, "matrix": 2 * N,
                      "precision": "fp64", "eig_solver": "own"},
           "stages_ms": st, "cusolver_solve_ms": t_cus,
           "own_vs_cusolver_max_abs_dE_ev": float(np.abs(E - E2).max()),
           "own_vs_cusolver_eps2_rel_l2": float(np.linalg.norm(e2 - e2b) / np.linalg.norm(e2b)),
           "mixed": {"solve_ms": float(np.median(tm)), "stages_ms": stm, "n_refine": 256,
                     "max_err_refined_256_ev": float(np.abs(Em[N:N + 256] - E[N:N + 256]).max()),
                     "max_err_all_ev": float(np.abs(Em - E).max()),
                     "eps2_rel_l2_vs_fp64": float(np.linalg.norm(e2m - e2) / np.linalg.norm(e2)),
                     "max_refined_residual_ev": dgm["max_refined_residual"],
                     "speedup_vs_fp64": float(np.median(ts)) / float(np.median(tm))}}
    if not args.no_cpu:
        orc = entry.load_oracle()
        small = synth.magnetic4_problem(grid=12)
        t0 = time.perf_counter()
        orc.solve(small, OMEGA, GAMMA, tamm_dancoff=0)
        t_cpu = (time.perf_counter() - t0) * 1e3
        out["cpu_baseline"] = {"value": t_cpu * (N / small.n_bse) ** 3, "unit": "ms", "kind": "port",
                               "cores": orc.lib().oracle_num_threads(),
                               "sample": f"oracle full-BSE solve of the 12x12 model (2N = {2 * small.n_bse}) in "
                                         f"{t_cpu:.0f} ms, scaled by (N/{small.n_bse})^3"}
    print(json.dumps(out))
    return 0


def run_rpa(args):
    """RPA screened interaction (w_kind = BSE_W_RPA, Dyson eps^-1, 64 sphere points) on the magnetic4
    24x24 2v2c model: the W tables (chi0 for the 2209 grid Delta k), then the mixed solve; the model-W
    workload beside it, and the oracle's RPA W table timed on the 8x8 model."""
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    prob = synth.magnetic4_problem(grid=24)
    kw = dict(w_kind=3, rpa_order=1, rpa_points=64, rpa_seed=1, precision=1, n_refine=256)
    with gpu.BSEContext(prob, **kw) as c:
        for _ in range(max(args.warmup, 1)):
            c.solve(OMEGA, GAMMA)
        ts, tt = [], []
        for _ in range(max(args.steps, 1)):
            E, e2, _ = c.solve(OMEGA, GAMMA)
            st = c.stage_times()
            ts.append(st["solve"])
            tt.append(st["tables"])
    with gpu.BSEContext(prob, precision=1, n_refine=256) as c2:
        c2.solve(OMEGA, GAMMA)
        E2, e22, _ = c2.solve(OMEGA, GAMMA)
        st2 = c2.stage_times()
    out = {"metric": "BSE build+diag wall time with the RPA screened interaction at N_BSE=2304", "unit": "ms",
           "value": float(np.median(ts)), "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
           "config": {"workload": "magnetic4_24x24_2v2c_rpa", "n_bse": prob.n_bse, "n_g": prob.ng,
                      "rpa_order": 1, "rpa_points": 64, "precision": "mixed", "n_refine": 256},
           "rpa_tables_ms": float(np.median(tt)), "stages_ms": st, "model_w_solve_ms": st2["solve"],
           "model_w_tables_ms": st2["tables"], "lowest_exciton_ev_rpa": float(E[0]), "lowest_exciton_ev_model_w": float(E2[0])}
    if not args.no_cpu:
        orc = entry.load_oracle()
        small = synth.magnetic4_problem(grid=8)
        t0 = time.perf_counter()
        orc.rpa_w(small, 0.0, 1, 64, 1)
        out["cpu_rpa_w_ms_8x8"] = (time.perf_counter() - t0) * 1e3
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--solver", default="own", choices=["own", "cusolver"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--workload", default="magnetic4", choices=["magnetic4", "batch", "large", "coupled", "rpa"])
    args = ap.parse_args()
    if args.workload == "rpa":
        return run_rpa(args)
    if args.workload == "coupled":
        return run_coupled(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "large":
        return run_large(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
