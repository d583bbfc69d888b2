"""CPU tests of the oracle's full BSE (tamm_dancoff = 0: the coupling block of
add_coupling_part, bse.version13.cpp:2929-3040, and the non-TDA spectrum, 3504-3522 and
3607-3620).  They pin the restatement the GPU path is checked against:
  - the resonant block and rho_cv are the Tamm-Dancoff ones, the anti-resonant blocks are
    -conj(A) (2917-2923) and -conj(B)^T (3035-3038), B is symmetric up to the O(q) shift of
    the exchange phases;
  - the coupling block equals the factorised lattice-sum form the CUDA kernel evaluates;
  - the three routes to the spectrum agree: the reference's eig_gen + inverse overlap matrix,
    the J-normalised sum over pairs, and direct linear solves of (w - H + i gamma) x = J rho;
  - eigenvalues come in +-E pairs, the J-norm of each eigenvector has the sign of E;
  - gauge invariance of the spectrum and of eps2 (decisions Q25, Q26);
  - with B = 0 the positive half of the spectrum is the Tamm-Dancoff one.
"""
import os

import numpy as np
import pytest

from factorised import coupling_factorised

OMEGA = np.arange(400) * 8.0 / 400
GAMMA = 0.05


def _prob(synth, name):
    return {"hbn6": lambda: synth.hbn_problem(grid=6), "hbn8": lambda: synth.hbn_problem(grid=8),
            "cubic3": lambda: synth.cubic3d_problem(grid=3), "orb8_3": lambda: synth.orb8_problem(grid=3),
            "mag4_4": lambda: synth.magnetic4_problem(grid=4), "coll3": lambda: synth.collinear_problem(grid=3),
            "coll4": lambda: synth.collinear_problem(grid=4)}[name]()


def _random_phases(bands, seed):
    ec, ev, cc, cv = bands
    rng = np.random.default_rng(seed)
    pc = np.exp(1j * rng.uniform(0, 2 * np.pi, cc.shape[:2]))[..., None]
    pv = np.exp(1j * rng.uniform(0, 2 * np.pi, cv.shape[:2]))[..., None]
    return ec, ev, cc * pc, cv * pv


@pytest.mark.parametrize("name", ["hbn6", "cubic3", "mag4_4", "coll3"])
def test_block_structure(synth, oracle, name):
    """Collinear models: the resonant part is the spin-rotated 4N x 4N Tamm-Dancoff matrix and
    the coupling part is rotated the same way (spin_transformation 3096-3105)."""
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    H, rho = oracle.build(prob, bands, tamm_dancoff=0)
    Ht, rhot = oracle.build(prob, bands)
    NA, NR = Ht.shape[0], rhot.shape[0]
    g0 = prob.ng // 2
    assert H.shape == (2 * NA, 2 * NA) and rho.shape == (2 * NR, prob.ng)
    A, B = H[:NA, :NA], H[:NA, NA:]
    assert np.array_equal(A, Ht) and np.array_equal(rho[:NR], rhot)
    assert np.array_equal(H[NA:, NA:], -A.conj())
    assert np.array_equal(H[NA:, :NA], -B.conj().T)
    # B^T = B up to the q-shift of the exchange phases e^{i(G+q).tau} (q = 1e-5 x)
    assert np.abs(B - B.T).max() < 1e-8 * np.abs(B).max()
    # dipole column of rho_vc: i q.<v|r|c> = -conj(i q.<c|r|v>)  (Q25)
    assert np.abs(rho[NR:, g0] + rho[:NR, g0].conj()).max() < 1e-14


@pytest.mark.parametrize("name", ["hbn6", "cubic3", "orb8_3", "mag4_4", "coll3", "coll4"])
def test_coupling_factorised_agrees(synth, oracle, name):
    """The oracle's loops over stored all-pairs densities and the factorised form (what the
    CUDA coupling kernel evaluates) give the same B."""
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    H, _ = oracle.build(prob, bands, tamm_dancoff=0)
    NA = H.shape[0] // 2
    B = coupling_factorised(prob, bands)
    assert np.abs(B - H[:NA, NA:]).max() < 1e-12 * np.abs(B).max()


@pytest.mark.parametrize("name", ["hbn6", "cubic3", "mag4_4"])
def test_spectrum_routes_agree(synth, oracle, name):
    prob = _prob(synth, name)
    H, rho = oracle.build(prob, tamm_dancoff=0)
    N = prob.n_bse
    F = oracle.prefactor(prob)
    r = rho[:, prob.ng // 2]
    res = oracle.solve_coupled(H, r, F, OMEGA, GAMMA)
    E = res["E"]
    # M = J H positive definite here: real spectrum in +-E pairs, J-norm sign = sign(E)
    J = np.r_[np.ones(N), -np.ones(N)]
    assert np.linalg.eigvalsh(J[:, None] * H).min() > 0
    assert np.abs(res["E_imag"]).max() < 1e-10 * np.abs(E).max()
    assert np.abs(E[:N][::-1] + E[N:]).max() < 1e-9 * np.abs(E).max()
    assert np.array_equal(res["jnorm_sign"], np.sign(E))
    # J-normalised pair sum == augmentation-matrix route
    chi = (np.sign(E) * np.abs(res["f"]) ** 2 / (OMEGA[:, None] - E[None, :] + 1j * GAMMA)).sum(axis=1)
    e2 = (1 - F * chi).imag
    assert np.linalg.norm(e2 - res["eps2"]) < 1e-10 * np.linalg.norm(res["eps2"])
    # == direct resolvent rho^H (w - H + i gamma)^{-1} J rho
    for w in OMEGA[::40]:
        x = np.linalg.solve((w + 1j * GAMMA) * np.eye(2 * N) - H, J * r)
        ref = (1 - F * (r.conj() @ x)).imag
        s = np.searchsorted(OMEGA, w)
        assert abs(ref - res["eps2"][s]) < 1e-10 * np.abs(res["eps2"]).max()


@pytest.mark.parametrize("name", ["hbn6", "cubic3"])
def test_gauge_invariance(synth, oracle, name):
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    r0 = oracle.solve(prob, OMEGA, GAMMA, band_states=bands, tamm_dancoff=0)
    r1 = oracle.solve(prob, OMEGA, GAMMA, band_states=_random_phases(bands, 5), tamm_dancoff=0)
    assert np.abs(r0["E"] - r1["E"]).max() < 1e-10
    assert np.linalg.norm(r0["eps2"] - r1["eps2"]) < 1e-9 * np.linalg.norm(r0["eps2"])


def test_no_coupling_limit(synth, oracle):
    """B = 0: the positive eigenvalues are the Tamm-Dancoff ones and eps2 is the TDA spectrum
    plus the anti-resonant term -F sum |f|^2 gamma / ((w + E)^2 + gamma^2)."""
    prob = _prob(synth, "hbn6")
    H, rho = oracle.build(prob, tamm_dancoff=0)
    N = prob.n_bse
    H[:N, N:] = 0
    H[N:, :N] = 0
    F = oracle.prefactor(prob)
    res = oracle.solve_coupled(H, rho[:, prob.ng // 2], F, OMEGA, GAMMA)
    tda = oracle.solve(prob, OMEGA, GAMMA)
    assert np.abs(res["E"][N:] - tda["E"]).max() < 1e-10
    anti = F * (np.abs(tda["f"]) ** 2 * GAMMA / ((OMEGA[:, None] + tda["E"][None, :]) ** 2 + GAMMA ** 2)).sum(axis=1)
    assert np.abs(res["eps2"] - (tda["eps2"] - anti)).max() < 1e-10 * np.abs(tda["eps2"]).max()


def test_ipa_ignores_coupling(synth, oracle):
    """ipa = 1 has no kernel: tamm_dancoff = 0 changes nothing (3346-3365, 3490-3493)."""
    prob = _prob(synth, "hbn6")
    a = oracle.solve(prob, OMEGA, GAMMA, ipa=1)
    b = oracle.solve(prob, OMEGA, GAMMA, ipa=1, tamm_dancoff=0)
    assert np.array_equal(a["E"], b["E"]) and np.array_equal(a["eps2"], b["eps2"])


def test_collinear_blocks(synth, oracle):
    """Collinear full BSE: both 4N x 4N spin blocks (H0 = {1,2}, H1 = {0,3} of every quadrant,
    3151-3172) keep the full-BSE structure; at 4x4 both are positive definite, the eigenvalues
    are the union of the blocks' and the spectrum comes from H1 with rho = (rho_cv; rho_vc)."""
    prob = _prob(synth, "coll4")
    H, rho = oracle.build(prob, tamm_dancoff=0)
    N = prob.n_bse
    H0, H1 = oracle.split_blocks_coupled(H, N)
    for Hb in (H0, H1):
        n2 = Hb.shape[0] // 2
        M = np.r_[np.ones(n2), -np.ones(n2)][:, None] * Hb
        assert np.abs(M - M.conj().T).max() < 1e-12 * np.abs(M).max()
        assert np.linalg.eigvalsh(M).min() > 0
    r = oracle.solve(prob, OMEGA, GAMMA, tamm_dancoff=0)
    assert r["E"].shape == (8 * N,) and r["f"].shape == (4 * N,)
    E0 = np.sort(np.linalg.eigvals(H0).real)
    assert np.abs(r["E"][:4 * N] - E0).max() < 1e-10
    res = oracle.solve_coupled(H1, rho[:, prob.ng // 2], oracle.prefactor(prob), OMEGA, GAMMA)
    assert np.array_equal(r["eps2"], res["eps2"])
    # spin-rotation invariance of the spectrum of the spin-conserving block: the coupled H1
    # equals the un-rotated blocks {0,3}
    Ht, _ = oracle.build(prob)
    b1 = np.r_[0:N, 3 * N:4 * N]
    assert np.array_equal(H1[:2 * N, :2 * N], Ht[np.ix_(b1, b1)])


def test_golden_vectors(synth, oracle):
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hbn4_full_golden.npz"))
    r = oracle.solve(synth.hbn_problem(grid=4), g["omega"], float(g["gamma"]), tamm_dancoff=0)
    assert np.abs(r["E"] - g["E"]).max() < 1e-12
    assert np.abs(r["eps2"] - g["eps2"]).max() < 1e-12 * np.abs(g["eps2"]).max()
    assert np.abs(np.abs(r["H"]) - g["absH"]).max() < 1e-12 * g["absH"].max()


def test_single_transition_closed_form(synth, oracle):
    """One k point, 1v x 1c: H = [[a, b], [-b*, -a]] has the eigenvalues +-sqrt(a^2 - |b|^2)."""
    prob = synth.hbn_problem(grid=1)
    H, _ = oracle.build(prob, tamm_dancoff=0)
    assert H.shape == (2, 2)
    a, b = H[0, 0].real, H[0, 1]
    r = oracle.solve(prob, OMEGA, GAMMA, tamm_dancoff=0)
    e = np.sqrt(a * a - abs(b) ** 2)
    assert np.abs(r["E"] - np.array([-e, e])).max() < 1e-12 * a
    X = r["A"]
    jn = np.einsum("il,i,il->l", X.conj(), np.array([1.0, -1.0]), X).real
    assert np.allclose(jn, [-1, 1], atol=1e-12)
