"""Small fixed workloads for kernel profiling (ncu) of this library.

    python bethe-salpeter-equation_gb300/profile_case.py --case solve2304
        one mixed-precision solve of the 4-orbital magnetic model, 24x24 grid (N_BSE = 2304),
        own eigensolver (tridiagonal reduction, bisection, inverse iteration, WY back-transform)
    python bethe-salpeter-equation_gb300/profile_case.py --case solve9216
        one mixed-precision solve of the 8-orbital model, 24x24 grid (N_BSE = 9216), own eigensolver
        (two-stage reduction: panel QR + cuBLAS rank-2NB updates, bulge chasing), ~7 GB on the device
    python bethe-salpeter-equation_gb300/profile_case.py --case solve4096
        the same at 16x16 (N_BSE = 4096), ~2 GB on the device, for kernel captures
    python bethe-salpeter-equation_gb300/profile_case.py --case build9216
        the complex64 kernel build of the 8-orbital model, 24x24 grid (N_BSE = 9216, H = 680 MB,
        larger than L2), lower triangle as the cuSOLVER path writes it and full storage

Each case runs one warm-up pass first, so `ncu -k regex:<kernel> -s <skip> -c 1` captures a
warm launch.  The process holds at most ~2 GB of device memory.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import __graft_entry__ as entry  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True, choices=["solve2304", "solve4096", "solve9216", "build9216"])
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args()
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    gpu = import_module("bse_gb300.gpu")
    omega = np.arange(2000) * 8.0 / 2000
    if args.case == "solve2304":
        prob = synth.magnetic4_problem(grid=24)
        with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as ctx:
            for _ in range(args.reps):
                ctx.solve(omega, 0.05)
            print({k: round(v, 3) for k, v in ctx.stage_times().items()})
    elif args.case in ("solve4096", "solve9216"):
        prob = synth.orb8_problem(grid=16 if args.case == "solve4096" else 24)
        with gpu.BSEContext(prob, precision=1, n_refine=256, eig_solver=0) as ctx:
            for _ in range(args.reps):
                ctx.solve(omega, 0.05)
            print({k: round(v, 3) for k, v in ctx.stage_times().items()})
    else:
        prob = synth.orb8_problem(grid=24)
        for solver in (1, 0):       # cuSOLVER path: lower triangle; own solver: full storage
            with gpu.BSEContext(prob, precision=1, n_refine=0, eig_solver=solver) as ctx:
                ctx.compute_bands()
                for _ in range(args.reps):
                    ctx.build_kernel()
                print(solver, {k: round(v, 3) for k, v in ctx.stage_times().items() if k in ("tables", "build")})


if __name__ == "__main__":
    main()
