"""Benchmark: q->0 Tamm-Dancoff BSE build + diagonalization + eps2 on one GB300.

Headline workload (one "step" = one BSE solve): the 8-orbital model (random Hermitian onsite
blocks, nearest / next-nearest hoppings, seed 2024, gap ~1.5 eV) on a 48x48 grid, 4 valence x 4
conduction bands, N_BSE = 36864, Rytova-Keldysh W + bare 2-D exchange, eps2 on 2000 points over
0-8 eV with 0.05 eV broadening.  Mixed precision: complex64 kernel build, FP32 eigensolve (the
dense -> band products on the tensor cores), FP64 Rayleigh-Ritz refinement of the lowest 256
excitons.  Inputs are synthetic (seeded); the 10.9 GB matrix is far larger than L2.

value  = device time per solve (CUDA events on the library's stream), model resident
e2e    = the same solve through the C ABI with host buffers, every step: context creation (model
         upload from host memory), solve, copy-back of the eigenvalues and eps, destroy
Other keys: the roofline of the dominant kernel (the tensor-core trailing update of the two-stage
reduction, HBM-bound) with its tensor-pipe rate, the eigensolve rate in the 14.7 N^3 flop unit,
the plain FP64 GPU path at N_BSE = 36864 (measured by `--workload fp64check`, committed under
profiles/) and the mixed path's errors against it, the same comparison live at N_BSE = 2304
(magnetic 4-orbital model, 24x24), the eps2 gradient time, the 64-model batch, the CPU oracle
baseline and the SM clocks sampled during the timed region.
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
WORKLOAD = "orb8_48x48_4v4c"          # N_BSE = 36864
WORKLOAD_SMALL = "magnetic4_24x24_2v2c"  # N_BSE = 2304
METRIC = "BSE build+diag wall time and eps2 grad time at N_BSE; error vs FP64"
FP64_LARGE_PROFILE = os.path.join(ROOT, "profiles", "fp64_vs_mixed_orb8_48x48.md")
# DRAM traffic / algorithmic bytes of tc_update_kernel, one ncu-captured launch at m = 8192
UPD_TRAFFIC_RATIO = (613.634560 + 478.541824) / (16 * 8192 ** 2 / 1e6)


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


def cpu_sample_large(orc, synth, prob_small=None):
    """One bounded CPU sample for the N_BSE = 36864 workload: the oracle's whole solve of the same
    8-orbital model on a 12x12 grid (N_BSE = 2304), its stages scaled to N_BSE = 36864 -- the band,
    build and spectrum stages by (36864 / 2304)^2 (their work is per exciton pair), the dense
    eigensolve (LAPACK zheevd) by (36864 / 2304)^3.  Returns (estimated ms, stage ms, sample text)."""
    prob = prob_small if prob_small is not None else synth.orb8_problem(grid=12)
    tm = {}
    t0 = time.perf_counter()
    orc.solve(prob, OMEGA, GAMMA, timings=tm)
    wall = (time.perf_counter() - t0) * 1e3
    r = 36864 / prob.n_bse
    quad = (tm["bands"] + tm["build"] + tm["eps"]) * 1e3
    eig = tm["eig"] * 1e3
    est = quad * r ** 2 + eig * r ** 3
    text = (f"oracle solve of orb8 12x12 (N_BSE={prob.n_bse}) in {wall:.0f} ms (bands+build+eps {quad:.0f} ms, "
            f"zheevd {eig:.0f} ms), scaled to N_BSE=36864: x{r ** 2:.0f} and x{r ** 3:.0f}")
    return est, {"bands_build_eps_ms": quad, "zheevd_ms": eig, "wall_ms": wall}, text


def fp64_large_record():
    """The plain FP64 GPU solve at N_BSE = 36864 and the mixed path's errors against it, as measured
    by `bench.py --workload fp64check` (one JSON line kept in the profile file)."""
    try:
        for ln in open(FP64_LARGE_PROFILE):
            ln = ln.strip()
            if ln.startswith("{") and '"fp64check"' in ln:
                return json.loads(ln)
    except OSError:
        pass
    return None


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    orc = entry.load_oracle()
    small = synth.orb8_problem(grid=12)
    cores = int(orc.lib().oracle_num_threads())
    for _ in range(args.warmup):
        cpu_sample_large(orc, synth, small)
    ts = []
    text = ""
    for _ in range(args.steps):
        est, _, text = cpu_sample_large(orc, synth, small)
        ts.append(est)
    ms = sum(ts) / len(ts)
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_bse": 36864, "n_g": small.ng, "precision": "fp64",
                   "l2": "inputs resident in host memory; CPU run"},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port",
                         "sample": "per step: " + text + "; C++ OpenMP restatement of the reference loops "
                                   "+ LAPACK zheevd (scipy OpenBLAS)"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _diag_full(gpu, ctx):
    out = np.zeros(12)
    ctx._check(ctx.lib.bse_diagnostics(ctx.h, out.ctypes.data_as(gpu._dp), 12))
    return out


def _small_comparison(gpu, synth, steps, flush):
    """magnetic4 24x24 (N_BSE = 2304): mixed solve vs the plain FP64 GPU path, live."""
    prob = synth.magnetic4_problem(grid=24)
    with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as c:
        c.solve(OMEGA, GAMMA)
        tm = []
        for _ in range(steps):
            _flush(flush)
            Em, e2m, _ = c.solve(OMEGA, GAMMA)
            tm.append(c.stage_times()["solve"])
    with gpu.BSEContext(prob, precision=0, eig_solver=1) as c64:
        c64.solve(OMEGA, GAMMA)
        t64 = []
        for _ in range(max(1, min(3, steps))):
            _flush(flush)
            E64, e2_64, _ = c64.solve(OMEGA, GAMMA)
            t64.append(c64.stage_times()["solve"])
    mixed_ms, fp64_ms = float(np.median(tm)), float(np.median(t64))
    return {"workload": WORKLOAD_SMALL, "n_bse": prob.n_bse, "mixed_ms": mixed_ms, "fp64_gpu_ms": fp64_ms,
            "fp64_path": "cuSOLVER zheevd on the complex128 matrix (bse_solve, precision fp64)",
            "speedup_vs_fp64_gpu": fp64_ms / mixed_ms,
            "max_eig_err_ev": {"refined_lowest_256": float(np.abs(Em[:256] - E64[:256]).max()),
                               "all": float(np.abs(Em - E64).max())},
            "eps2_rel_l2_vs_fp64": float(np.linalg.norm(e2m - e2_64) / np.linalg.norm(e2_64))}


def _batch_figure(gpu, synth, steps):
    """64 seeded 2- to 4-band models (N_BSE 144 .. 3600): one bse_solve_many over them."""
    import torch
    probs = synth.random_batch_problems(n_models=64, seed=77)
    ctxs = [gpu.BSEContext(p, precision=1, n_refine=64, eig_solver=0) for p in probs]
    try:
        gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=8)
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=8)
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
    finally:
        for c in ctxs:
            c.close()
    ms = float(np.median(ts))
    return {"workload": "batch64_rand_2to4band_12to30grid", "wall_ms": ms, "models_per_s": len(probs) / (ms / 1e3),
            "n_bse_sum": int(sum(p.n_bse for p in probs))}


def run_gpu(args):
    ws, rank, local = _dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BSE_BENCH_GLOO") is None else "gloo")
    import torch
    torch.cuda.set_device(local)
    os.environ["BSE_KERNEL_TIMING"] = "1"     # per-launch events around the tensor-core products
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    from bse_gb300.capi import Marshalled
    gpu.load().bse_set_device(local)
    prob = synth.orb8_problem(grid=48)
    N = prob.n_bse
    mixed = dict(precision=1, n_refine=256, eig_solver=0)
    mm = Marshalled(prob, **mixed)
    h2d = _model_bytes(mm) + OMEGA.nbytes
    d2h = mm.n_exc * 8 + 2 * OMEGA.nbytes
    flush = _l2_flush_buffer()

    # --- K steps, each through the C ABI with host buffers: create (model upload), solve, copy-back,
    # destroy.  value = the solve's device time (events on the library stream), e2e = the wall time ---
    for _ in range(args.warmup):
        with gpu.BSEContext(prob, **mixed) as c:
            c.solve(OMEGA, GAMMA)
    dev_ms, e2e_ms, stages, kts = [], [], [], []
    launches = 0
    _barrier(ws)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t_host0 = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        with gpu.BSEContext(prob, **mixed) as c:
            E_mixed, e2_mixed, _ = c.solve(OMEGA, GAMMA)
            st = c.stage_times()
            kts.append(_diag_full(gpu, c))
            launches += c.kernel_launches()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        dev_ms.append(st["solve"])
        stages.append(st)
    torch.cuda.synchronize()
    host_s = time.perf_counter() - t_host0
    clk = clocks.stop()
    _barrier(ws)
    ms_per_step = _max_over_ranks(ws, sum(dev_ms)) / args.steps
    value = ms_per_step / ws            # whole-job time per solve (one problem per rank and step)
    e2e_value = _max_over_ranks(ws, sum(e2e_ms)) / args.steps / ws
    stage_avg = {k: float(np.mean([s[k] for s in stages])) for k in stages[0]}
    dg = kts[-1]

    # --- rooflines from the per-launch events of the timed steps ---
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
    k_arr = np.array(kts)
    upd_ms, upd_n, upd_bytes, upd_flops = (k_arr[:, 8 + i].sum() for i in range(4))
    hemm_ms, hemm_n, hemm_bytes, hemm_flops = (k_arr[:, 4 + i].sum() for i in range(4))
    roof = None
    if upd_n > 0:
        gbs = upd_bytes / (upd_ms * 1e-3) / 1e9
        # tensor work actually issued: six BF16 products of the real-folded complex update
        # (M = m rows, N = 2 m real columns, K = 4 kk) = 6 * 2 * m * 2m * 4kk = 96 m^2 kk = 6 * flops_alg
        tflops = 6.0 * upd_flops / (upd_ms * 1e-3) / 1e12
        roof = {"kernel": "tc_update_kernel (tcgen05 kind::f16, TMA)", "bound": "hbm", "achieved": gbs, "peak": hbm,
                "peak_source": src, "unit": "GB/s", "frac": gbs / hbm,
                "traffic": UPD_TRAFFIC_RATIO * upd_bytes / upd_n,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at m = 8192 "
                                  "(profiles/tc_update_hemm_kernels_m8192.md): 1.014 x the algorithmic bytes, "
                                  "scaled to the average launch here (traffic grows with the 16 m^2 bytes)",
                "alg_bytes_per_launch": upd_bytes / upd_n, "avg_launch_ms": upd_ms / upd_n,
                "launches_per_solve": upd_n / args.steps,
                "alg_bytes_unit": "16 m^2 per launch: the m x m complex64 trailing matrix read and written once",
                "tensor": {"achieved": tflops, "peak": bf16, "unit": "TFLOP/s", "frac": tflops / bf16,
                           "note": "BF16 tensor flops issued (6 split products) vs the measured dense BF16 peak"}}
    hemm_fig = None
    if hemm_n > 0:
        gbs = hemm_bytes / (hemm_ms * 1e-3) / 1e9
        hemm_fig = {"kernel": "tc_hemm_kernel", "bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                    "frac": gbs / hbm, "alg_bytes_per_launch": hemm_bytes / hemm_n, "avg_launch_ms": hemm_ms / hemm_n,
                    "total_ms_per_solve": hemm_ms / args.steps}
    eig_ms = stage_avg["eig"]

    # --- secondary figures (after the timed region) ---
    small = _small_comparison(gpu, synth, max(1, min(5, args.steps)), flush)
    grad_ms = None
    if not args.no_grad:
        from bse_gb300.adjoint import ParamModel, backward, gpu_forward
        from bse_gb300.synth import MAGNETIC4_NOMINAL
        pm = ParamModel.magnetic4()
        p2 = synth.magnetic4_problem(grid=24)
        wts = np.random.default_rng(11).uniform(0.0, 1.0, size=len(OMEGA))
        fwd = gpu_forward(pm, p2, MAGNETIC4_NOMINAL, 10.0, OMEGA, GAMMA)      # warm-up
        backward(pm, fwd["prob"], fwd, OMEGA, wts, GAMMA)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fwd = gpu_forward(pm, p2, MAGNETIC4_NOMINAL, 10.0, OMEGA, GAMMA)
        backward(pm, fwd["prob"], fwd, OMEGA, wts, GAMMA)
        torch.cuda.synchronize()
        grad_ms = (time.perf_counter() - t0) * 1e3
    batch = None if args.no_batch else _batch_figure(gpu, synth, 3)
    fp64_large = fp64_large_record()

    cpu = None
    if rank == 0 and not args.no_cpu:
        orc = entry.load_oracle()
        est, parts, text = cpu_sample_large(orc, synth)
        cpu = {"value": est, "unit": "ms", "cores": int(orc.lib().oracle_num_threads()), "kind": "port",
               "sample": text + "; C++ OpenMP restatement of the reference loops + LAPACK zheevd (scipy OpenBLAS)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64+fp64-refine", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_bse": N, "n_k": prob.nk, "n_g": prob.ng, "nw": prob.model.nw,
                       "nv": prob.params.nv, "nc": prob.params.nc, "n_omega": len(OMEGA), "gamma": GAMMA,
                       "precision": "mixed", "n_refine": 256, "eig_solver": "own",
                       "parallelism": f"replicas x{ws}",
                       "l2": "inputs larger than L2 (the complex64 BSE matrix is 10.9 GB)"},
            "e2e": {"value": e2e_value, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "roofline": roof,
            "roofline_hemm": hemm_fig,
            "eig_rate": {"unit": "TFLOP/s", "flop_per_solve": 14.7 * N ** 3, "eig_ms": eig_ms,
                         "value": 14.7 * N ** 3 / (eig_ms * 1e-3) / 1e12,
                         "note": "14.7 N^3 = zhetrd 16/3 + D&C 4/3 + zunmtr 8 (N^3 real flops), the LAPACK-equivalent count"},
            "stages_ms": stage_avg,
            "max_refined_residual_ev": float(dg[0]),
            "fp64_gpu_n36864": fp64_large,
            "n2304_mixed_vs_fp64": small,
            "eps2_grad_ms": grad_ms,
            "eps2_grad_config": "d(sum_s w_s eps2(w_s))/d(12 hopping/onsite, r0), FP64 forward + hand-written adjoint, "
                                "magnetic4 24x24 (N_BSE=2304)",
            "batch64": batch,
            "host_wall_s": host_s,
            "clocks": clk,
        }
        if fp64_large:
            line["speedup_vs_fp64_gpu"] = fp64_large["fp64_gpu_ms"] / ms_per_step
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


def run_fp64check(args):
    """The plain FP64 GPU path at N_BSE = 36864 (orb8 48x48): bse_solve in FP64 with cuSOLVER zheevd
    on the complex128 matrix, against the mixed path on the same problem: its time, the mixed
    path's eigenvalue errors (refined lowest 256 and all) and the eps2 relative L2 error.  One JSON
    line (kept in the profile file that the default run reads)."""
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    prob = synth.orb8_problem(grid=48)
    with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as cm:
        cm.solve(OMEGA, GAMMA)
        Em, e2m, _ = cm.solve(OMEGA, GAMMA)
        tm = cm.stage_times()
        dg = cm.diagnostics()
    print(json.dumps({"mixed_ms": tm["solve"], "stages_ms": tm}), file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    with gpu.BSEContext(prob, precision=0, eig_solver=1) as c64:
        E64, e2_64, _ = c64.solve(OMEGA, GAMMA)
        t64 = c64.stage_times()
    wall64 = (time.perf_counter() - t0) * 1e3
    out = {"fp64check": True, "workload": WORKLOAD, "n_bse": prob.n_bse,
           "fp64_gpu_ms": t64["solve"], "fp64_wall_ms": wall64, "fp64_stages_ms": t64,
           "fp64_path": "bse_solve, precision fp64: complex128 build + cuSOLVER zheevd (eigenvectors for the oscillators)",
           "mixed_ms": tm["solve"], "mixed_stages_ms": tm, "speedup_vs_fp64_gpu": t64["solve"] / tm["solve"],
           "max_eig_err_ev": {"refined_lowest_256": float(np.abs(Em[:256] - E64[:256]).max()),
                              "all": float(np.abs(Em - E64).max())},
           "eps2_rel_l2_vs_fp64": float(np.linalg.norm(e2m - e2_64) / np.linalg.norm(e2_64)),
           "max_refined_residual_ev": dg["max_refined_residual"]}
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
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--workload", default="orb8_48", choices=["orb8_48", "batch", "fp64check", "coupled", "rpa"])
    args = ap.parse_args()
    if args.workload == "rpa":
        return run_rpa(args)
    if args.workload == "coupled":
        return run_coupled(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "fp64check":
        return run_fp64check(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
