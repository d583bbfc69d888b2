"""GPU parity: the CUDA library (through the C ABI) against the CPU FP64 oracle.

Tolerances (eV for energies, relative for matrices / spectra):
  FP64 path:   band energies 1e-11, gauge-fixed band vectors 1e-9, H elements 1e-11 * max|H|,
               BSE eigenvalues 1e-8 eV (the 1e-6 eV FP64 target with margin), eps2 rel L2 1e-8
  MIXED path:  H elements 2e-6 * max|H| (complex64 storage), refined eigenvalues 1e-6 eV,
               unrefined eigenvalues 1e-6 * ||H||_2 (the backward error class of an FP32
               eigensolver; ||H||_2 = max |E|), eps2 rel L2 1e-4
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(2000) * 8.0 / 2000     # 0-8 eV, 2000 points (the config-1 grid)
GAMMA = 0.05


def _problems(synth):
    return {
        "hbn12": synth.hbn_problem(grid=12),
        "mag8": synth.magnetic4_problem(grid=8),
        "coll6": synth.collinear_problem(grid=6),
        "cubic4": synth.cubic3d_problem(grid=4),
        "orb8_4": synth.orb8_problem(grid=4),
    }


@pytest.fixture(scope="module")
def problems(synth):
    return _problems(synth)


@pytest.mark.parametrize("name", ["hbn12", "mag8", "coll6", "cubic4", "orb8_4"])
def test_bands_match_oracle(problems, oracle, gpu, name):
    prob = problems[name]
    ref = oracle.bands(prob)
    with gpu.BSEContext(prob) as ctx:
        ctx.compute_bands()
        got = ctx.get_bands()
    for r, g, tol in zip(ref, got, (1e-11, 1e-11, 1e-9, 1e-9)):
        assert np.abs(r - g).max() < tol


@pytest.mark.parametrize("name", ["hbn12", "mag8", "coll6", "cubic4", "orb8_4"])
def test_build_matches_oracle_fp64(problems, oracle, gpu, name):
    prob = problems[name]
    bands = oracle.bands(prob)
    H_ref, rho_ref = oracle.build(prob, bands)
    with gpu.BSEContext(prob) as ctx:
        ctx.set_bands(*bands)
        H, rho = ctx.build_kernel(want_h=True, want_rho=True)
    scale = np.abs(H_ref).max()
    assert np.abs(H - H_ref).max() < 1e-11 * scale
    assert np.abs(rho - rho_ref).max() < 1e-11 * max(1.0, np.abs(rho_ref).max())


@pytest.mark.parametrize("name", ["hbn12", "mag8", "coll6"])
def test_build_matches_oracle_mixed(problems, oracle, gpu, name):
    prob = problems[name]
    bands = oracle.bands(prob)
    H_ref, _ = oracle.build(prob, bands)
    with gpu.BSEContext(prob, precision=1) as ctx:
        ctx.set_bands(*bands)
        H, _ = ctx.build_kernel(want_h=True)
    assert np.abs(H - H_ref).max() < 2e-6 * np.abs(H_ref).max()


SOLVERS = {"own": 0, "cusolver": 1}


@pytest.mark.parametrize("solver", ["own", "cusolver"])
@pytest.mark.parametrize("name", ["hbn12", "mag8", "coll6", "cubic4", "orb8_4"])
def test_solve_fp64(problems, oracle, gpu, name, solver):
    prob = problems[name]
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, eig_solver=SOLVERS[solver]) as ctx:
        E, e2, e1 = ctx.solve(OMEGA, GAMMA)
        f = ctx.oscillators()
    assert np.abs(E - ref["E"]).max() < 1e-8
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])
    assert np.linalg.norm(e1 - ref["eps1"]) < 1e-8 * np.linalg.norm(ref["eps1"])
    # |f|^2 summed over (near-)degenerate groups is gauge invariant
    assert abs(np.sum(np.abs(f) ** 2) - np.sum(np.abs(ref["f"]) ** 2)) < 1e-9 * np.sum(np.abs(ref["f"]) ** 2)


@pytest.mark.parametrize("solver", ["own", "cusolver"])
@pytest.mark.parametrize("name,n_refine", [("hbn12", 64), ("mag8", 64), ("coll6", 32)])
def test_solve_mixed(problems, oracle, gpu, name, n_refine, solver):
    prob = problems[name]
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, precision=1, n_refine=n_refine, eig_solver=SOLVERS[solver]) as ctx:
        E, e2, _ = ctx.solve(OMEGA, GAMMA)
    n_opt = len(ref["E_opt"])
    E_opt = E[-n_opt:]
    assert np.abs(E_opt[:n_refine] - ref["E_opt"][:n_refine]).max() < 1e-6
    assert np.abs(E - ref["E"]).max() < max(1e-5, 1e-6 * np.abs(ref["E"]).max())
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])


@pytest.mark.parametrize("solver", ["own", "cusolver"])
def test_ipa_limit_exact(synth, gpu, solver):
    """ipa = 1: H = diag(E_c(k) - E_v(k-q)) and the eigenvalues are those transitions, sorted
    (common_diagonalization ipa branch, bse.version13.cpp:3346-3365)."""
    prob = synth.magnetic4_problem(grid=8)
    with gpu.BSEContext(prob, ipa=1, eig_solver=SOLVERS[solver]) as ctx:
        ctx.compute_bands()
        ec, ev, _, _ = ctx.get_bands()
        E, _, _ = ctx.solve(OMEGA, GAMMA)
    nk, nc, nv = prob.nk, prob.params.nc, prob.params.nv
    trans = (ec[0][:, :, None] - ev[0][:, None, :]).reshape(nk, nc * nv)
    assert np.abs(np.sort(trans.ravel()) - E).max() < 1e-12


def test_random_k_list_pair_tables(synth, oracle, gpu):
    """A k list that is not a lattice uses per-pair Delta-k tables."""
    prob = synth.hbn_problem(grid=4)
    rng = np.random.default_rng(5)
    from bse_gb300.model import reciprocal_vectors
    kc = rng.uniform(-1, 1, size=(20, 3))
    kc[:, 2] = 0
    prob.k_cart = kc @ reciprocal_vectors(prob.model.lattice).T
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob) as ctx:
        E, e2, _ = ctx.solve(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


@pytest.mark.parametrize("solver", ["own", "cusolver"])
def test_stage_api_sequence(synth, oracle, gpu, solver):
    """build -> diagonalize -> oscillators -> eps through the separate entry points."""
    prob = synth.hbn_problem(grid=8)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, eig_solver=SOLVERS[solver]) as ctx:
        ctx.build_kernel()
        E, A = ctx.diagonalize(want_vectors=True)
        f = ctx.oscillators()
        e2, e1 = ctx.eps(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    # eigenvectors: unit norm, orthogonal, and A^H H A = diag(E)
    assert np.abs(A.conj().T @ A - np.eye(A.shape[0])).max() < 1e-9
    H = ref["H"]
    assert np.abs(A.conj().T @ H @ A - np.diag(E)).max() < 1e-8 * np.abs(E).max()
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


@pytest.mark.parametrize("solver", ["own", "cusolver"])
def test_degenerate_spectrum_weights(synth, oracle, gpu, solver):
    """hBN in the independent-particle limit has exactly degenerate transitions (grid symmetry):
    the eigenvectors inside each degenerate group must stay orthogonal, or the eps2 weights of
    the group are wrong."""
    prob = synth.hbn_problem(grid=12)
    prob.params = prob.params.replace(ipa=1)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, eig_solver=SOLVERS[solver]) as ctx:
        E, e2, _ = ctx.solve(OMEGA, GAMMA)
        f = ctx.oscillators()
    assert np.abs(E - ref["E"]).max() < 1e-10
    assert abs(np.sum(np.abs(f) ** 2) - np.sum(np.abs(ref["f"]) ** 2)) < 1e-9 * np.sum(np.abs(ref["f"]) ** 2)
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


@pytest.mark.parametrize("mode", ["fused", "shared", "redundant", "twostage"])
def test_tridiagonal_barrier_modes(synth, oracle, gpu, monkeypatch, mode):
    """Every variant of the tridiagonal reduction (one-stage with the working vectors in shared
    memory, or with per-block copies in global memory, both one grid barrier per reflector, or
    two barriers with shared vectors; the two-stage dense -> band -> tridiagonal path of the
    largest matrices) gives the oracle's spectrum."""
    monkeypatch.setenv("BSE_TRIDIAG_MODE", mode)
    prob = synth.orb8_problem(grid=4)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    for precision, tol in ((0, 1e-8), (1, None)):
        with gpu.BSEContext(prob, precision=precision, eig_solver=0, n_refine=64) as ctx:
            E, e2, _ = ctx.solve(OMEGA, GAMMA)
        if tol is None:
            assert np.abs(E[:64] - ref["E"][:64]).max() < 1e-6
            assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])
        else:
            assert np.abs(E - ref["E"]).max() < tol
            assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


@pytest.mark.parametrize("grid", [13, 7])
def test_two_stage_vectors_ragged(synth, oracle, gpu, monkeypatch, grid):
    """Two-stage reduction at orders that are not multiples of the band width (169, 49), FP64:
    all eigenvalues, all back-transformed eigenvectors (orthonormal, A^H H A = diag(E)), eps2."""
    monkeypatch.setenv("BSE_TRIDIAG_MODE", "twostage")
    prob = synth.hbn_problem(grid=grid)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, eig_solver=0) as ctx:
        ctx.build_kernel()
        E, A = ctx.diagonalize(want_vectors=True)
        f = ctx.oscillators()
        e2, _ = ctx.eps(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    assert np.abs(A.conj().T @ A - np.eye(A.shape[0])).max() < 1e-9
    H = ref["H"]
    assert np.abs(A.conj().T @ H @ A - np.diag(E)).max() < 1e-8 * np.abs(E).max()
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


def test_two_stage_degenerate_and_collinear(synth, oracle, gpu, monkeypatch):
    """Two-stage reduction on exactly degenerate spectra (hBN IPA limit) and on the collinear
    spin-block layout, FP64 and mixed precision with refinement."""
    monkeypatch.setenv("BSE_TRIDIAG_MODE", "twostage")
    prob = synth.hbn_problem(grid=12)
    prob.params = prob.params.replace(ipa=1)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    with gpu.BSEContext(prob, eig_solver=0) as ctx:
        E, e2, _ = ctx.solve(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-10
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])
    prob = synth.collinear_problem(grid=6)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    for precision in (0, 1):
        with gpu.BSEContext(prob, precision=precision, eig_solver=0, n_refine=64) as ctx:
            E, e2, _ = ctx.solve(OMEGA, GAMMA)
        if precision == 0:
            assert np.abs(E - ref["E"]).max() < 1e-8
            assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])
        else:
            # the refinement covers the optically active block, the last n_opt eigenvalues
            n_opt = len(ref["E_opt"])
            assert np.abs(E[-n_opt:][:64] - ref["E_opt"][:64]).max() < 1e-6
            assert np.abs(E - ref["E"]).max() < max(1e-5, 1e-6 * np.abs(ref["E"]).max())
            assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])


def test_two_stage_repeatable_mixed(synth, gpu, monkeypatch):
    """The concurrent bulge chase gives bit-identical tridiagonals run after run and agrees with
    the one-stage reduction to FP32 accuracy (N=2304: sweeps of 72 steps, ~24 running at once)."""
    prob = synth.orb8_problem(grid=12)
    monkeypatch.setenv("BSE_TRIDIAG_MODE", "shared")
    with gpu.BSEContext(prob, precision=1, eig_solver=0, n_refine=0) as ctx:
        E1, _, _ = ctx.solve(OMEGA, GAMMA)
    monkeypatch.setenv("BSE_TRIDIAG_MODE", "twostage")
    runs = []
    for _ in range(3):
        with gpu.BSEContext(prob, precision=1, eig_solver=0, n_refine=0) as ctx:
            E, _, _ = ctx.solve(OMEGA, GAMMA)
        runs.append(E)
    for E in runs[1:]:
        assert np.array_equal(E, runs[0])
    assert np.abs(runs[0] - E1).max() < max(1e-5, 1e-6 * np.abs(E1).max())


def test_refinement_pencil_modes(synth, oracle, gpu, monkeypatch):
    """The FP64 refinement's projected pencil (S, M) solved by iterative refinement from the FP32
    Ritz vectors (default), by the dense FP64 solver, and by cuSOLVER heevd gives the same refined
    eigenvalues (the magnetic model has exactly degenerate pairs, which form clusters)."""
    prob = synth.magnetic4_problem(grid=12)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    Es = {}
    for mode in ("", "dense", "cusolver"):
        monkeypatch.setenv("BSE_REFINE_EIG", mode)
        with gpu.BSEContext(prob, precision=1, eig_solver=0, n_refine=64) as ctx:
            E, e2, _ = ctx.solve(OMEGA, GAMMA)
            diag = ctx.diagnostics()
        assert np.abs(E[:64] - ref["E"][:64]).max() < 1e-8
        assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])
        assert diag["max_refined_residual"] < 1e-3
        Es[mode] = E[:64]
    assert np.abs(Es[""] - Es["dense"]).max() < 1e-10
    assert np.abs(Es[""] - Es["cusolver"]).max() < 1e-10
