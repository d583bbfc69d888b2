"""GPU parity of the RPA screened interaction (w_kind = BSE_W_RPA: adding_screening = 1,
pull_coulomb_potentials 2597-2690, Dielectric_Function::pull_values 2214-2315) against the
oracle's restatement (decisions Q28-Q30).  Tolerances: H elements 1e-10 relative (FP64),
2e-6 (mixed); eigenvalues 1e-8 eV; eps2 relative L2 1e-8."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(1000) * 8.0 / 1000
GAMMA = 0.05


def _prob(synth, name):
    return {"hbn6": lambda: synth.hbn_problem(grid=6), "mag4_4": lambda: synth.magnetic4_problem(grid=4),
            "coll4": lambda: synth.collinear_problem(grid=4), "cubic3": lambda: synth.cubic3d_problem(grid=3)}[name]()


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("name", ["hbn6", "mag4_4", "coll4", "cubic3"])
def test_rpa_build_matches_oracle(synth, oracle, gpu, name, order):
    prob = _prob(synth, name)
    kw = dict(w_kind=3, rpa_order=order, rpa_points=8, rpa_seed=7)
    bands = oracle.bands(prob)
    H_ref, _ = oracle.build(prob, bands, **kw)
    with gpu.BSEContext(prob, **kw) as ctx:
        ctx.set_bands(*bands)
        H, _ = ctx.build_kernel(want_h=True)
    assert np.abs(H - H_ref).max() < 1e-10 * np.abs(H_ref).max()


@pytest.mark.parametrize("name", ["hbn6", "coll4"])
def test_rpa_solve_matches_oracle(synth, oracle, gpu, name):
    prob = _prob(synth, name)
    kw = dict(w_kind=3, rpa_order=1, rpa_points=8, rpa_seed=3)
    bands = oracle.bands(prob)
    ref = oracle.solve(prob, OMEGA, GAMMA, band_states=bands, **kw)
    with gpu.BSEContext(prob, **kw) as ctx:
        ctx.set_bands(*bands)
        ctx.build_kernel()
        E, _ = ctx.diagonalize()
        ctx.oscillators()
        e2, _ = ctx.eps(OMEGA, GAMMA)
    assert np.abs(E - ref["E"]).max() < 1e-8
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-8 * np.linalg.norm(ref["eps2"])


def test_rpa_mixed_build(synth, oracle, gpu):
    prob = _prob(synth, "hbn6")
    kw = dict(w_kind=3, rpa_order=1, rpa_points=8, rpa_seed=3)
    bands = oracle.bands(prob)
    H_ref, _ = oracle.build(prob, bands, **kw)
    with gpu.BSEContext(prob, precision=1, **kw) as ctx:
        ctx.set_bands(*bands)
        H, _ = ctx.build_kernel(want_h=True)
    assert np.abs(H - H_ref).max() < 2e-6 * np.abs(H_ref).max()


def test_rpa_full_bse_build(synth, oracle, gpu):
    """RPA W with the coupling block: the coupling pairs the states through conj(W), its own table."""
    prob = _prob(synth, "hbn6")
    kw = dict(w_kind=3, rpa_order=1, rpa_points=8, rpa_seed=3, tamm_dancoff=0)
    bands = oracle.bands(prob)
    H_ref, _ = oracle.build(prob, bands, **kw)
    with gpu.BSEContext(prob, **kw) as ctx:
        ctx.set_bands(*bands)
        H, _ = ctx.build_kernel(want_h=True)
    assert np.abs(H - H_ref).max() < 1e-10 * np.abs(H_ref).max()
