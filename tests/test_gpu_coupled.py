"""GPU parity of the full BSE (tamm_dancoff = 0): the CUDA coupling-block build and the
structure-preserving solve against the oracle's reference-route restatement (eig_gen of the
2N x 2N matrix and the inverse-overlap spectrum, bse.version13.cpp:2929-3040, 3326,
3504-3522, 3607-3620).

Tolerances: H elements and rho 1e-11 relative, eigenvalues 1e-8 eV, |f|^2 per pair 1e-8
relative to max |f|^2, eps2 relative L2 1e-8, eigenvector residual ||H x - E x|| 1e-8 * ||H||,
J-norm x^H J x = sign(E) to 1e-9.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(2000) * 8.0 / 2000
GAMMA = 0.05
SOLVERS = {"own": 0, "cusolver": 1}


def _prob(synth, name):
    return {"hbn8": lambda: synth.hbn_problem(grid=8), "cubic4": lambda: synth.cubic3d_problem(grid=4),
            "mag8": lambda: synth.magnetic4_problem(grid=8), "orb8_3": lambda: synth.orb8_problem(grid=3),
            "coll3": lambda: synth.collinear_problem(grid=3), "coll4": lambda: synth.collinear_problem(grid=4)}[name]()


@pytest.mark.parametrize("name", ["hbn8", "cubic4", "mag8", "orb8_3", "coll3", "coll4"])
def test_coupled_build_matches_oracle(synth, oracle, gpu, name):
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    H_ref, rho_ref = oracle.build(prob, bands, tamm_dancoff=0)
    with gpu.BSEContext(prob, tamm_dancoff=0) as ctx:
        ctx.set_bands(*bands)
        H, rho = ctx.build_kernel(want_h=True, want_rho=True)
    nh = 2 * (3 * (prob.model.n_spin - 1) + 1) * prob.n_bse
    assert H.shape == H_ref.shape == (nh, nh)
    assert np.abs(H - H_ref).max() < 1e-11 * np.abs(H_ref).max()
    assert np.abs(rho - rho_ref).max() < 1e-11 * max(1.0, np.abs(rho_ref).max())


@pytest.mark.parametrize("solver", ["own", "cusolver"])
@pytest.mark.parametrize("name", ["hbn8", "cubic4", "mag8", "coll4"])
def test_coupled_solve_matches_oracle(synth, oracle, gpu, name, solver):
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    ref = oracle.solve(prob, OMEGA, GAMMA, band_states=bands, tamm_dancoff=0)
    with gpu.BSEContext(prob, tamm_dancoff=0, eig_solver=SOLVERS[solver]) as ctx:
        ctx.set_bands(*bands)
        ctx.build_kernel()
        E, _ = ctx.diagonalize()
        f = ctx.oscillators()
        e2, e1 = ctx.eps(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    # |f|^2 per pair (phases are a gauge) where the level is separated from its neighbours;
    # collinear: the pairs of the optically active block H1 (the second half of E)
    E = E[len(E) - len(f):]
    gap = np.minimum(np.r_[np.inf, np.diff(E)], np.r_[np.diff(E), np.inf])
    sep = gap > 1e-6
    f2, f2r = np.abs(f) ** 2, np.abs(ref["f"]) ** 2
    assert np.abs(f2[sep] - f2r[sep]).max() < 1e-8 * f2r.max()
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])
    assert np.linalg.norm(e1 - ref["eps1"]) < 1e-8 * np.linalg.norm(ref["eps1"])


@pytest.mark.parametrize("solver", ["own", "cusolver"])
@pytest.mark.parametrize("name", ["hbn8", "coll4"])
def test_coupled_vectors(synth, oracle, gpu, solver, name):
    """a_out: the eigenvectors of H = [[A, B], [-B^H, -A*]] (collinear: of the optically active
    block H1), J-normalised (x^H J x = sign E), and f = rho^H x from them equals the oscillators."""
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    H_ref, rho_ref = oracle.build(prob, bands, tamm_dancoff=0)
    if prob.model.n_spin == 2:
        H_ref = oracle.split_blocks_coupled(H_ref, prob.n_bse)[1]
    N = H_ref.shape[0] // 2
    J = np.r_[np.ones(N), -np.ones(N)]
    with gpu.BSEContext(prob, tamm_dancoff=0, eig_solver=SOLVERS[solver]) as ctx:
        ctx.set_bands(*bands)
        ctx.build_kernel()
        E, X = ctx.diagonalize(want_vectors=True)
        E = E[len(E) - X.shape[1]:]
        f = ctx.oscillators()
    res = np.linalg.norm(H_ref @ X - X * E[None, :], axis=0)
    assert res.max() < 1e-8 * np.abs(H_ref).max() * 2 * N
    jn = np.einsum("il,i,il->l", X.conj(), J, X).real
    assert np.abs(jn - np.sign(E)).max() < 1e-9
    f2 = X.T @ np.conj(rho_ref[:, prob.ng // 2])
    assert np.abs(f2 - f).max() < 1e-9 * np.abs(f).max()


def test_coupled_bse_solve_entry_point(synth, oracle, gpu):
    prob = _prob(synth, "mag8")
    ref = oracle.solve(prob, OMEGA, GAMMA, tamm_dancoff=0)
    with gpu.BSEContext(prob, tamm_dancoff=0) as ctx:
        E, e2, e1 = ctx.solve(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


def test_coupled_not_positive_definite_is_an_error(synth, gpu):
    """orb8 at 3x3 has a negative Tamm-Dancoff exciton: [[A, B], [B*, A*]] is indefinite and
    the solve returns BSE_ERR_BAD_INPUT (the context stays usable: rebuild and retry)."""
    prob = _prob(synth, "orb8_3")
    with gpu.BSEContext(prob, tamm_dancoff=0) as ctx:
        ctx.compute_bands()
        ctx.build_kernel()
        with pytest.raises(gpu.BSEError) as ei:
            ctx.diagonalize()
        assert ei.value.status == -1 and "positive definite" in str(ei.value)
        ctx.build_kernel()
        with pytest.raises(gpu.BSEError):
            ctx.diagonalize()


@pytest.mark.parametrize("name", ["hbn8", "mag8", "coll4"])
def test_coupled_mixed_matches_oracle(synth, oracle, gpu, name):
    """BSE_MIXED full BSE: FP32 Cholesky / inverse and the own FP32 solve of -L^-1 J L^-H, FP64
    refinement of the lowest n_refine positive pairs on the definite pencil (J, M).  Refined
    eigenvalues within 1e-8 eV; the others within the FP32 error of mu = -1/E, 1e-6 E^2 / E_min;
    eps2 relative L2 1e-4."""
    prob = _prob(synth, name)
    bands = oracle.bands(prob)
    ref = oracle.solve(prob, OMEGA, GAMMA, band_states=bands, tamm_dancoff=0)
    n_ref = 32
    with gpu.BSEContext(prob, tamm_dancoff=0, precision=1, n_refine=n_ref) as ctx:
        ctx.set_bands(*bands)
        ctx.build_kernel()
        E, _ = ctx.diagonalize()
        f = ctx.oscillators()
        e2, _ = ctx.eps(OMEGA, GAMMA)
        dg = ctx.diagnostics()
    Er = ref["E"]
    N = len(f) // 2            # positive pairs of the optically active block
    off = len(E) - len(f)      # collinear: that block's values follow the spin-flip block's
    assert np.abs(E[off + N:off + N + n_ref] - Er[off + N:off + N + n_ref]).max() < 1e-8
    emin = np.abs(Er).min()
    assert np.all(np.abs(E - Er) <= np.maximum(1e-5, 1e-6 * Er ** 2 / emin))
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])
    # Rayleigh-Ritz in the span of the FP32 stage's vectors: the refined eigenvalues are second
    # order in that subspace's FP32 error (checked to 1e-8 eV above), their residuals
    # ||M x - E J x|| first order, a few eps32 * max|E|
    assert dg["n_refined"] == n_ref and dg["max_refined_residual"] < 1e-6 * np.abs(Er).max()


def test_coupled_mixed_limits(synth, gpu):
    prob = _prob(synth, "hbn8")
    with pytest.raises(gpu.BSEError):
        gpu.BSEContext(prob, tamm_dancoff=0, precision=1, eig_solver=1)
    with gpu.BSEContext(prob, tamm_dancoff=0, precision=1, n_refine=8) as ctx:
        ctx.compute_bands()
        ctx.build_kernel()
        with pytest.raises(gpu.BSEError) as ei:
            ctx.diagonalize(want_vectors=True)
        assert "eigenvectors" in str(ei.value)
