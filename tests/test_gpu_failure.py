"""Failure detection without a GPU fault: every wait of the solver on another block (grid and
flag barriers of the cooperative reductions, the bulge chase's sweep dependencies) is bounded, and
the H(k) Jacobi eigensolver has a sweep cap.  The test overrides BSE_TEST_SPIN_LIMIT (polls before a
wait gives up) and BSE_TEST_JACOBI_SWEEPS (the sweep cap), read at bse_create, make these limits
run out on purpose: the waiting block raises the error word and returns, every other block sees the
word at its next wait and returns, and the host reports BSE_ERR_NOT_CONVERGED.  The device stays
usable: a fresh context afterwards solves normally.  Nothing here faults, traps or hangs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(400) * 8.0 / 400
GAMMA = 0.05
NOT_CONVERGED = -4


@pytest.mark.parametrize("mode,precision", [("fused", 1), ("fused", 0), ("twostage", 1)])
def test_barrier_limit_runs_out(synth, gpu, monkeypatch, mode, precision):
    prob = synth.magnetic4_problem(grid=12)          # N_BSE = 576: hundreds of barriers per reduction
    monkeypatch.setenv("BSE_TRIDIAG_MODE", mode)
    with gpu.BSEContext(prob, precision=precision, n_refine=32) as ctx:
        E_ref, e2_ref, _ = ctx.solve(OMEGA, GAMMA)
    monkeypatch.setenv("BSE_TEST_SPIN_LIMIT", "1")
    with gpu.BSEContext(prob, precision=precision, n_refine=32) as ctx:
        with pytest.raises(gpu.BSEError) as ei:
            ctx.solve(OMEGA, GAMMA)
        assert ei.value.status == NOT_CONVERGED
        assert "timed out" in str(ei.value)
    monkeypatch.delenv("BSE_TEST_SPIN_LIMIT")
    with gpu.BSEContext(prob, precision=precision, n_refine=32) as ctx:   # the device is still usable
        E, e2, _ = ctx.solve(OMEGA, GAMMA)
    assert np.array_equal(E, E_ref) and np.array_equal(e2, e2_ref)


def test_jacobi_sweep_cap_runs_out(synth, gpu, monkeypatch):
    prob = synth.hbn_problem(grid=6)
    monkeypatch.setenv("BSE_TEST_JACOBI_SWEEPS", "0")
    with gpu.BSEContext(prob) as ctx:
        with pytest.raises(gpu.BSEError) as ei:
            ctx.compute_bands()
        assert ei.value.status == NOT_CONVERGED
        assert "sweep cap" in str(ei.value)
    monkeypatch.delenv("BSE_TEST_JACOBI_SWEEPS")
    with gpu.BSEContext(prob) as ctx:
        E, _, _ = ctx.solve(OMEGA, GAMMA)
    assert np.all(np.isfinite(E))
