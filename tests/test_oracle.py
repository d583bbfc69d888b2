"""CPU tests of the FP64 oracle: known-answer tests that pin the restatement.

The reference ships no tests, fixtures or golden outputs and cannot be built here
(Armadillo/LAPACK absent), so the oracle is pinned by:
  - the independent-particle limit (ipa=1): eigenvalues are the sorted transitions
    E_c(k) - E_v(k-q) exactly (common_diagonalization, bse.version13.cpp:3346-3365);
  - the analytic two-band honeycomb model E = +-sqrt(D^2 + t^2 |f(k)|^2);
  - Hermiticity of H and gauge invariance of its spectrum and of eps2;
  - an independent numpy evaluation of the kernel in factorised form (tests/factorised.py);
  - the Lorentzian sum rule int eps2 dw = pi F sum |f|^2 and eps2 >= 0;
  - committed golden vectors (tests/golden/, made by tests/golden/make_golden.py).
"""
import math
import os

import numpy as np
import pytest

from factorised import build_factorised

HERE = os.path.dirname(os.path.abspath(__file__))
OMEGA = np.arange(2000) * 8.0 / 2000


def test_two_band_analytic(synth, oracle):
    prob = synth.hbn_problem(grid=12)
    ec, ev, _, _ = oracle.bands(prob)
    lat = prob.model.lattice
    a1, a2 = lat[:, 0], lat[:, 1]
    for arr, shift, sgn in ((ec, np.zeros(3), 1), (ev, np.array(prob.params.q), -1)):
        k = prob.k_cart - shift
        f = 1 + np.exp(-1j * k @ a1) + np.exp(-1j * k @ a2)
        e = sgn * np.sqrt(1.0 + (2.8 * np.abs(f)) ** 2)
        assert np.abs(arr[0, :, 0] - e).max() < 1e-12


def test_ipa_eigenvalues_are_transitions(synth, oracle):
    prob = synth.magnetic4_problem(grid=6)
    prob.params = prob.params.replace(ipa=1)
    ec, ev, _, _ = oracle.bands(prob)
    r = oracle.solve(prob, OMEGA, 0.05)
    trans = (ec[0][:, :, None] - ev[0][:, None, :])     # [k][c][v]
    assert np.abs(np.sort(trans.ravel()) - r["E"]).max() < 1e-13
    H = r["H"]
    assert np.abs(H - np.diag(np.diag(H))).max() == 0.0


@pytest.mark.parametrize("name", ["hbn", "magnetic4", "collinear", "cubic3d", "orb8"])
def test_hermitian(synth, oracle, name):
    prob = {"hbn": lambda: synth.hbn_problem(grid=6), "magnetic4": lambda: synth.magnetic4_problem(grid=4),
            "collinear": lambda: synth.collinear_problem(grid=4), "cubic3d": lambda: synth.cubic3d_problem(grid=3),
            "orb8": lambda: synth.orb8_problem(grid=3)}[name]()
    H, _ = oracle.build(prob)
    assert np.abs(H - H.conj().T).max() < 1e-12 * np.abs(H).max()


def _random_phases(bands, seed):
    ec, ev, cc, cv = bands
    rng = np.random.default_rng(seed)
    pc = np.exp(1j * rng.uniform(0, 2 * np.pi, cc.shape[:2]))[..., None]
    pv = np.exp(1j * rng.uniform(0, 2 * np.pi, cv.shape[:2]))[..., None]
    return ec, ev, cc * pc, cv * pv


@pytest.mark.parametrize("name", ["hbn", "magnetic4", "orb8"])
def test_gauge_invariance(synth, oracle, name):
    prob = {"hbn": lambda: synth.hbn_problem(grid=6), "magnetic4": lambda: synth.magnetic4_problem(grid=4),
            "orb8": lambda: synth.orb8_problem(grid=3)}[name]()
    bands = oracle.bands(prob)
    r0 = oracle.solve(prob, OMEGA, 0.05, band_states=bands)
    r1 = oracle.solve(prob, OMEGA, 0.05, band_states=_random_phases(bands, 3))
    assert np.abs(r0["E"] - r1["E"]).max() < 1e-11
    assert np.linalg.norm(r0["eps2"] - r1["eps2"]) < 1e-10 * np.linalg.norm(r0["eps2"])


@pytest.mark.parametrize("name", ["hbn", "magnetic4", "collinear", "cubic3d", "orb8"])
def test_factorised_kernel_agrees(synth, oracle, name):
    """The reference-order loops (oracle) and the factorised lattice-sum form (what the
    CUDA kernels evaluate) give the same H and rho."""
    prob = {"hbn": lambda: synth.hbn_problem(grid=5), "magnetic4": lambda: synth.magnetic4_problem(grid=4),
            "collinear": lambda: synth.collinear_problem(grid=4), "cubic3d": lambda: synth.cubic3d_problem(grid=3),
            "orb8": lambda: synth.orb8_problem(grid=3)}[name]()
    bands = oracle.bands(prob)
    H, rho = oracle.build(prob, bands)
    H2, rho2 = build_factorised(prob, bands)
    assert np.abs(rho - rho2).max() < 1e-12 * max(1, np.abs(rho).max())
    assert np.abs(H - H2).max() < 1e-11 * np.abs(H).max()


def test_sum_rule_and_positivity(synth, oracle):
    prob = synth.hbn_problem(grid=8)
    om = np.linspace(-200.0, 200.0, 400001)
    r = oracle.solve(prob, om, 0.05)
    assert r["eps2"].min() > -1e-15
    integral = np.trapezoid(r["eps2"], om)
    expect = math.pi * r["F"] * np.sum(np.abs(r["f"]) ** 2)
    # Lorentzian tails beyond +-200 eV carry 2*gamma/(pi*200) of the weight
    assert abs(integral - expect) < 2e-3 * expect


def test_exchange_sign_and_dipole(synth, oracle):
    """Bare exchange raises and the direct term lowers the lowest exciton of the two-band model."""
    prob = synth.hbn_problem(grid=8)
    ref = oracle.solve(prob, OMEGA, 0.05)
    ipa = oracle.solve(prob.__class__(prob.model, prob.k_cart, prob.g_cart, prob.params.replace(ipa=1)), OMEGA, 0.05)
    assert ref["E"][0] < ipa["E"][0] - 0.1        # bound exciton below the gap
    assert np.abs(ref["f"]).max() > 0


def test_golden_vectors(synth, oracle):
    g = np.load(os.path.join(HERE, "golden", "hbn4_golden.npz"))
    prob = synth.hbn_problem(grid=4)
    r = oracle.solve(prob, g["omega"], float(g["gamma"]))
    assert np.abs(r["E"] - g["E"]).max() < 1e-12
    assert np.abs(r["eps2"] - g["eps2"]).max() < 1e-12 * np.abs(g["eps2"]).max()
    assert np.abs(np.abs(r["H"]) - g["absH"]).max() < 1e-12 * g["absH"].max()
    g2 = np.load(os.path.join(HERE, "golden", "coll3_golden.npz"))
    prob2 = synth.collinear_problem(grid=3)
    r2 = oracle.solve(prob2, g2["omega"], float(g2["gamma"]))
    assert np.abs(r2["E"] - g2["E"]).max() < 1e-12
    assert np.abs(r2["eps2"] - g2["eps2"]).max() < 1e-12 * np.abs(g2["eps2"]).max()
