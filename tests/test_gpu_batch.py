"""Batched solves (bse_solve_many): many uneven models on one GPU from several host threads."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(1000) * 8.0 / 1000
GAMMA = 0.05


def test_solve_many_equals_individual_solves(synth, oracle, gpu):
    probs = synth.random_batch_problems(n_models=8, seed=5, grid_range=(4, 9))
    ctxs = [gpu.BSEContext(p, precision=1, n_refine=32) for p in probs]
    try:
        singles = [c.solve(OMEGA, GAMMA)[1] for c in ctxs]
        e2, _ = gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=4)
        e2b, _ = gpu.solve_many(ctxs, OMEGA, GAMMA, n_workers=3)
    finally:
        for c in ctxs:
            c.close()
    for i, s in enumerate(singles):
        assert np.array_equal(e2[i], s)
        assert np.array_equal(e2b[i], s)
    for i in (0, 5):
        ref = oracle.solve(probs[i], OMEGA, GAMMA)
        assert np.linalg.norm(e2[i] - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])


def test_solve_many_rejects_bad_arguments(gpu):
    lib = gpu.load()
    import ctypes as C
    assert lib.bse_solve_many(None, 1, None, 0, 0.05, None, None, 1) == -1
    arr = (C.c_void_p * 1)(None)
    assert lib.bse_solve_many(arr, 1, None, 0, 0.05, None, None, 1) == -1
