"""The allocation-free dielectric function, bse_eps_noalloc, against bse_eps.

bse_eps_noalloc exists for callers that cannot call cudaMalloc (code inside a framework that
holds the device memory in its own pool): it stages its inputs and outputs in one fixed device
array instead of allocating.  This file
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


def test_noalloc_at_the_limits(gpu):
    """131072 excitons and 16384 frequencies fill every region of the fixed array: the result
    equals the sum of two half-size calls (which leave the regions' ends unused) and a direct
    numpy evaluation on every 64th frequency."""
    lib = gpu.load()
    from bse_gb300.capi import ptr
    n, nw = 131072, 16384
    rng = np.random.default_rng(4)
    E = np.ascontiguousarray(rng.uniform(0.5, 8.0, n))
    f = np.ascontiguousarray(rng.normal(size=n) + 1j * rng.normal(size=n))
    om = np.ascontiguousarray(np.arange(nw) * 9.0 / nw)
    F = 1e-3

    def call(Ep, fp):
        Ep, fp = np.ascontiguousarray(Ep), np.ascontiguousarray(fp)
        e2 = np.full(nw, np.nan)
        e1 = np.full(nw, np.nan)
        st = lib.bse_eps_noalloc(len(Ep), ptr(Ep), ptr(fp), F, ptr(om), nw, GAMMA, ptr(e2), ptr(e1), None)
        assert st == 0, lib.bse_last_error(None)
        return e2, e1

    e2, e1 = call(E, f)
    a2, a1 = call(E[: n // 2], f[: n // 2])
    b2, b1 = call(E[n // 2:], f[n // 2:])
    assert np.abs(e2 - (a2 + b2)).max() <= 1e-12 * np.abs(e2).max()
    assert np.abs(e1 - (a1 + b1 - 1.0)).max() <= 1e-12 * np.abs(e1).max()
    w = om[::64]
    d = w[:, None] - E[None, :]
    den = d * d + GAMMA * GAMMA
    f2 = np.abs(f) ** 2
    ref2 = F * (f2[None, :] * GAMMA / den).sum(axis=1)
    ref1 = 1.0 - F * (f2[None, :] * d / den).sum(axis=1)
    assert np.abs(e2[::64] - ref2).max() <= 1e-10 * np.abs(ref2).max()
    assert np.abs(e1[::64] - ref1).max() <= 1e-10 * np.abs(ref1).max()


def test_noalloc_rejects_too_many_frequencies(gpu):
    lib = gpu.load()
    from bse_gb300.capi import ptr
    E = np.ones(4)
    f = np.ones(4, np.complex128)
    om = np.zeros(16385)
    e2 = np.zeros(16385)
    st = lib.bse_eps_noalloc(4, ptr(E), ptr(f), 1.0, ptr(om), 16385, GAMMA, ptr(e2), None, None)
    assert st == -1
    assert b"16384" in lib.bse_last_error(None)
