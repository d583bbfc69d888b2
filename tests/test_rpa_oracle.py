"""CPU tests of the oracle's RPA screened interaction (adding_screening = 1, the insulator branch
of pull_coulomb_potentials, bse.version13.cpp:2597-2690, with Dielectric_Function::pull_values
2214-2315) -- the oracle half of the RPA-W row; the CUDA kernels for it are not built yet.
Known answers:
  - chi0 at omega = 0 is Hermitian and negative semidefinite (eta = 0);
  - first order: eps^-1 = 1 + v chi0; Dyson: (1 - v chi0) eps^-1 = 1;
  - the static response of a Hermitian model is real: chi0_{-G,-G'}(-q) = chi0_GG'(q)^*, also for
    a magnetic model (decision Q30), and the W table keeps W_{-G,-G'}(-dk) = W_GG'(dk)^* including
    the sphere-averaged dk = 0 entry (Q28);
  - 0 < eps^-1_00 < 1 (screening), W Hermitian at every dk != 0;
  - the BSE matrix built with the RPA W is Hermitian, and its spectrum and eps2 are gauge invariant.
"""
import numpy as np
import pytest

OMEGA = np.arange(400) * 8.0 / 400
GAMMA = 0.05


def _prob(synth, name):
    return {"hbn6": lambda: synth.hbn_problem(grid=6), "cubic3": lambda: synth.cubic3d_problem(grid=3),
            "mag4_4": lambda: synth.magnetic4_problem(grid=4)}[name]()


def _neg_g(prob):
    """index of -G for every G of the (symmetric) G list"""
    G = prob.g_cart
    idx = np.array([np.argmin(np.linalg.norm(G + g, axis=1)) for g in G])
    assert np.allclose(G[idx], -G)
    return idx


def _v(prob, q):
    import factorised as fz
    vol, area, normal, lz = fz._geometry(prob.model.lattice)
    return fz._coulomb(prob.params, q + prob.g_cart, normal, lz)


@pytest.mark.parametrize("name", ["hbn6", "cubic3", "mag4_4"])
def test_chi0_and_dyson(synth, oracle, name):
    prob = _prob(synth, name)
    q = prob.k_cart[1] - prob.k_cart[0]
    ng = prob.ng
    chi0, einv = oracle.rpa_eps_inv(prob, q, 0.0, 1)
    _, einv0 = oracle.rpa_eps_inv(prob, q, 0.0, 0)
    v = _v(prob, q)
    assert np.abs(chi0 - chi0.conj().T).max() < 1e-14 * np.abs(chi0).max()
    assert np.linalg.eigvalsh(chi0).max() < 1e-12 * np.abs(chi0).max()
    assert np.abs((np.eye(ng) - v[:, None] * chi0) @ einv - np.eye(ng)).max() < 1e-12
    assert np.abs(einv0 - (np.eye(ng) + v[:, None] * chi0)).max() < 1e-12
    e00 = einv[ng // 2, ng // 2]
    assert 0 < e00.real < 1 and abs(e00.imag) < 1e-12


@pytest.mark.parametrize("name", ["hbn6", "mag4_4"])
def test_static_response_is_real(synth, oracle, name):
    """chi0_{-G,-G'}(-q) = chi0_GG'(q)^* (Q30: exact without time-reversal symmetry)."""
    prob = _prob(synth, name)
    q = prob.k_cart[2] - prob.k_cart[0]
    ng_idx = _neg_g(prob)
    cp, _ = oracle.rpa_eps_inv(prob, q, 0.0, 1)
    cm, _ = oracle.rpa_eps_inv(prob, -q, 0.0, 1)
    assert np.abs(cm[np.ix_(ng_idx, ng_idx)] - cp.conj()).max() < 1e-12 * np.abs(cp).max()


@pytest.mark.parametrize("name", ["hbn6", "mag4_4"])
def test_w_table_symmetries(synth, oracle, name):
    prob = _prob(synth, name)
    W = oracle.rpa_w(prob, eta=0.0, order=1, n_points=16, seed=3)
    nk, ng = prob.nk, prob.ng
    idx = _neg_g(prob)
    scale = np.abs(W).max()
    for i in range(nk):
        for j in range(nk):
            # reality of the static W(r, r'), the pair (j, i) holding -dk
            assert np.abs(W[j, i][np.ix_(idx, idx)] - W[i, j].conj()).max() < 1e-10 * scale
            if i != j:
                assert np.abs(W[i, j] - W[i, j].conj().T).max() < 1e-10 * scale
    # screening: W_00(dk) below the bare v(dk) for dk != 0
    dk = prob.k_cart[1] - prob.k_cart[0]
    assert 0 < W[1, 0][ng // 2, ng // 2].real < _v(prob, dk)[ng // 2]
    # seeded: the same seed gives the same table, another seed changes only dk = 0
    W2 = oracle.rpa_w(prob, eta=0.0, order=1, n_points=16, seed=3)
    W3 = oracle.rpa_w(prob, eta=0.0, order=1, n_points=16, seed=4)
    assert np.array_equal(W, W2)
    off = ~np.eye(nk, dtype=bool)
    assert np.array_equal(W[off], W3[off]) and not np.array_equal(W[0, 0], W3[0, 0])


@pytest.mark.parametrize("name", ["hbn6", "mag4_4"])
def test_bse_with_rpa_w(synth, oracle, name):
    prob = _prob(synth, name)
    W = oracle.rpa_w(prob, eta=0.0, order=1, n_points=16, seed=5)
    bands = oracle.bands(prob)
    H, _ = oracle.build(prob, bands, w_table=W)
    assert np.abs(H - H.conj().T).max() < 1e-12 * np.abs(H).max()
    rng = np.random.default_rng(9)
    ec, ev, cc, cv = bands
    ph = (cc * np.exp(1j * rng.uniform(0, 2 * np.pi, cc.shape[:2]))[..., None],
          cv * np.exp(1j * rng.uniform(0, 2 * np.pi, cv.shape[:2]))[..., None])
    r0 = oracle.solve(prob, OMEGA, GAMMA, band_states=bands, w_table=W)
    r1 = oracle.solve(prob, OMEGA, GAMMA, band_states=(ec, ev) + ph, w_table=W)
    assert np.abs(r0["E"] - r1["E"]).max() < 1e-10
    assert np.linalg.norm(r0["eps2"] - r1["eps2"]) < 1e-9 * np.linalg.norm(r0["eps2"])
