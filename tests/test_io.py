"""Reference input formats: Wannier90 hr.dat / centres.xyz, lattice, atoms and k-list files."""
import numpy as np
import pytest


@pytest.mark.parametrize("name", ["hbn", "magnetic4", "collinear", "cubic3d"])
def test_w90_round_trip(tmp_path, pkg, synth, name):
    from bse_gb300 import w90io
    m = {"hbn": synth.hbn_model, "magnetic4": synth.magnetic4_model, "collinear": synth.collinear_model,
         "cubic3d": synth.cubic3d_model}[name]()
    paths = w90io.write_model_files(m, str(tmp_path), name)
    m2 = w90io.read_model_files(paths, m.nw, m.n_r, n_atoms=m.nw, n_spin=m.n_spin, dim=m.dim)
    assert np.allclose(m2.lattice, m.lattice, atol=1e-15)
    assert (m2.r_cryst == m.r_cryst).all()
    assert np.abs(m2.h_r - m.h_r).max() < 1e-15
    assert np.abs(m2.centres - m.centres).max() < 1e-15
    k = np.random.default_rng(0).normal(size=(7, 3))
    assert np.abs(m2.hk(k) - m.hk(k)).max() < 1e-13


def test_hr_header_mismatch_raises(tmp_path, pkg, synth):
    from bse_gb300 import w90io
    m = synth.hbn_model()
    paths = w90io.write_model_files(m, str(tmp_path), "x")
    with pytest.raises(ValueError):
        w90io.read_hr(paths["hr"], m.nw + 1, m.n_r)


def test_lattice_file_row_is_vector(tmp_path, pkg):
    from bse_gb300 import w90io
    lat = np.array([[1.0, 2, 3], [4, 5, 6], [7, 8, 10]])
    p = tmp_path / "lat"
    p.write_text("1 2 3\n4 5 6\n7 8 10\n")
    got = w90io.read_lattice(str(p))
    assert np.allclose(got[:, 0], [1, 2, 3]) and np.allclose(got[:, 2], [7, 8, 10])
