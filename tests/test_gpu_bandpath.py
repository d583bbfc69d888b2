"""GPU band structure along a path (Hamiltonian_TB::pull_bands, bse.version13.cpp:823-875):
the band kernel on the path's k points against the oracle's band subset at the same points
(band energies 1e-11 eV)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["hbn", "magnetic4", "collinear"])
def test_band_path_matches_oracle(tmp_path, synth, oracle, gpu, name):
    from bse_gb300 import bandpath, w90io
    from bse_gb300.model import Problem
    prob = {"hbn": lambda: synth.hbn_problem(grid=3), "magnetic4": lambda: synth.magnetic4_problem(grid=3),
            "collinear": lambda: synth.collinear_problem(grid=3)}[name]()
    B = 2 * np.pi * np.linalg.inv(prob.model.lattice).T
    segs = [(np.zeros(3), B @ [0.5, 0, 0], 21), (B @ [0.5, 0, 0], B @ [1 / 3, 1 / 3, 0], 15)]
    ev, ec = bandpath.band_structure(prob, segs, out_path=str(tmp_path / "bands.dat"))
    pts = w90io.band_path_points(segs)
    ref_prob = Problem(model=prob.model, k_cart=pts, g_cart=prob.g_cart,
                       params=prob.params.replace(q=(0.0, 0.0, 0.0), small_momentum=0, ipa=1))
    ec_r, ev_r, _, _ = oracle.bands(ref_prob)
    assert np.abs(ev - ev_r).max() < 1e-11 and np.abs(ec - ec_r).max() < 1e-11
    assert len((tmp_path / "bands.dat").read_text().splitlines()) == len(pts)
