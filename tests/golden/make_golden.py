"""Generate the golden vectors in tests/golden/ from the CPU oracle.

The reference publishes no outputs and cannot be built here, so these fixtures freeze
the oracle's FP64 results on two small seeded workloads (regression vectors for the
restatement; the GPU parity tests compare against the live oracle):
  hbn4_golden.npz   hBN-like 2-band model, 4x4 grid, RK W + bare 2-D V, N = 16
  coll3_golden.npz  collinear two-channel model, 3x3 grid, N = 9 (H is 36 x 36)
  hbn4_full_golden.npz  the hbn4 workload as a full BSE (tamm_dancoff = 0: coupling block,
                    2N = 32 eigenvalues, non-TDA spectrum)
  coll3_full_golden.npz the coll3 workload as a full BSE (8N = 72 matrix, both 4N spin blocks)
Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402


def main():
    entry.load_package()
    from importlib import import_module
    synth = import_module("bse_gb300.synth")
    orc = entry.load_oracle()
    omega = np.arange(200) * 8.0 / 200
    gamma = 0.05
    r = orc.solve(synth.hbn_problem(grid=4), omega, gamma)
    np.savez(os.path.join(HERE, "hbn4_golden.npz"), omega=omega, gamma=gamma, E=r["E"], eps2=r["eps2"],
             eps1=r["eps1"], absH=np.abs(r["H"]))
    r = orc.solve(synth.collinear_problem(grid=3), omega, gamma)
    np.savez(os.path.join(HERE, "coll3_golden.npz"), omega=omega, gamma=gamma, E=r["E"], eps2=r["eps2"],
             eps1=r["eps1"])
    r = orc.solve(synth.hbn_problem(grid=4), omega, gamma, tamm_dancoff=0)
    np.savez(os.path.join(HERE, "hbn4_full_golden.npz"), omega=omega, gamma=gamma, E=r["E"], eps2=r["eps2"],
             eps1=r["eps1"], absH=np.abs(r["H"]), absf=np.abs(r["f"]))
    r = orc.solve(synth.collinear_problem(grid=3), omega, gamma, tamm_dancoff=0)
    np.savez(os.path.join(HERE, "coll3_full_golden.npz"), omega=omega, gamma=gamma, E=r["E"], eps2=r["eps2"],
             eps1=r["eps1"], absH=np.abs(r["H"]))
    print("wrote golden vectors")


if __name__ == "__main__":
    main()
