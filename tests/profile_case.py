"""Fixed workloads for ncu captures of this library (a test-side helper, not part of the package).

    python tests/profile_case.py --case solve2304    one mixed solve of the magnetic 4-orbital model,
        24x24 (N_BSE = 2304): one-stage reduction, bisection, inverse iteration; ~0.3 GB on the device
    python tests/profile_case.py --case solve4096    the 8-orbital model at 16x16 (N_BSE = 4096),
        two-stage reduction; ~2 GB on the device
    python tests/profile_case.py --case solve9216    the same at 24x24 (N_BSE = 9216); ~7 GB
    python tests/profile_case.py --case build9216    the complex64 kernel build at 24x24 (H = 680 MB,
        larger than L2), lower triangle (cuSOLVER path) and full storage; ~2 GB
    python tests/profile_case.py --case tc8192       the tensor-core hemm and update of the two-stage
        reduction alone on an 8192 x 8192 complex64 matrix; ~1.2 GB

Each solve case runs --reps passes (the first is a warm-up).  Capture with the clocks left alone,
e.g. ncu --set full --clock-control none -k regex:<kernel> -s <skip> -c 1 python tests/profile_case.py
--case solve4096, after the same command has run to completion without ncu.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))     # the repository root
import __graft_entry__ as entry  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True, choices=["solve2304", "solve4096", "solve9216", "build9216", "tc8192"])
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
    elif args.case == "tc8192":
        import ctypes as C
        lib = gpu.load()
        lib.bse_test_tc_hemm.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
        lib.bse_test_tc_rank2k.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
        m = 8192
        rng = np.random.default_rng(0)
        A = np.ascontiguousarray((rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))).astype(np.complex64))
        V = np.ascontiguousarray((rng.normal(size=(32, m)) + 1j * rng.normal(size=(32, m))).astype(np.complex64))
        W = np.ascontiguousarray((rng.normal(size=(32, m)) + 1j * rng.normal(size=(32, m))).astype(np.complex64))
        Y = np.zeros((32, m), np.complex64)
        for _ in range(args.reps):
            print("hemm", lib.bse_test_tc_hemm(m, 32, A.ctypes.data, m, V.ctypes.data, Y.ctypes.data),
                  "update", lib.bse_test_tc_rank2k(m, 32, A.ctypes.data, m, V.ctypes.data, W.ctypes.data))
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
