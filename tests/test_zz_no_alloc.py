"""The allocation-free dielectric function, bse_eps_noalloc, against bse_eps.

bse_eps_noalloc exists for callers that cannot call cudaMalloc (a framework that holds the
device memory in its own pool, or a pipeline that must not synchronise the device): it
stages its inputs and outputs in one fixed device array instead of allocating.  This file
runs last (pytest collects files alphabetically) and must also pass alone in a fresh
process, where its first call is the one that sets the array up.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(2000) * 8.0 / 2000
GAMMA = 0.05
CONV = (1.602176634 * 1000) / 8.8541878176


def _reference_outputs(gpu, prob):
    """Eigenvalues, oscillator strengths and eps from the context entry points."""
    with gpu.BSEContext(prob) as ctx:
        E, _, _ = ctx.solve(OMEGA, GAMMA)
        f = ctx.oscillators()
        e2, e1 = ctx.eps(OMEGA, GAMMA)
    F = CONV / (prob.model.volume * prob.nk)          # small-q prefactor of bse_eps
    return E, f, F, e2, e1


def _noalloc(lib, E, f, F):
    from bse_gb300.capi import ptr
    E = np.ascontiguousarray(E, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.complex128)
    e2 = np.full(len(OMEGA), np.nan)
    e1 = np.full(len(OMEGA), np.nan)
    st = lib.bse_eps_noalloc(len(E), ptr(E), ptr(f), F, ptr(OMEGA), len(OMEGA), GAMMA, ptr(e2), ptr(e1), None)
    assert st == 0, lib.bse_last_error(None)
    return e2, e1


def test_noalloc_matches_bse_eps_two_calls(synth, gpu):
    lib = gpu.load()
    cases = [_reference_outputs(gpu, synth.hbn_problem(grid=12)),
             _reference_outputs(gpu, synth.magnetic4_problem(grid=8))]
    # two calls in a row on different inputs: the second must not see the first's contents
    for E, f, F, e2_ref, e1_ref in cases:
        e2, e1 = _noalloc(lib, E, f, F)
        assert np.linalg.norm(e2 - e2_ref) <= 1e-12 * np.linalg.norm(e2_ref)
        assert np.linalg.norm(e1 - e1_ref) <= 1e-12 * np.linalg.norm(e1_ref)


def test_noalloc_rejects_oversize(gpu):
    lib = gpu.load()
    from bse_gb300.capi import ptr
    n = 131072 + 1
    E = np.zeros(n)
    f = np.zeros(n, np.complex128)
    e2 = np.zeros(len(OMEGA))
    st = lib.bse_eps_noalloc(n, ptr(E), ptr(f), 1.0, ptr(OMEGA), len(OMEGA), GAMMA, ptr(e2), None, None)
    assert st == -1
    assert b"131072" in lib.bse_last_error(None)
