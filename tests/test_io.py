"""Reference file formats: Wannier90 hr.dat / centres.xyz, lattice, atoms, k-list and spectrum files."""
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


def test_spectrum_file_round_trip(tmp_path, synth, oracle):
    """The reference's dielectric-function file (3644-3656): eps_xx round-trips, yy = zz = (0,0),
    the last column is Im(eps_xx)/3 (Q16)."""
    from bse_gb300 import w90io
    omega = np.arange(50) * 8.0 / 50
    r = oracle.solve(synth.hbn_problem(grid=3), omega, 0.05)
    path = tmp_path / "eps.dat"
    w90io.write_spectrum(str(path), omega, r["eps2"], r["eps1"])
    om, eps = w90io.read_spectrum(str(path))
    assert np.allclose(om, omega) and np.allclose(eps.imag, r["eps2"], rtol=1e-9, atol=1e-12)
    assert np.allclose(eps.real, r["eps1"], rtol=1e-9, atol=1e-12)
    lines = path.read_text().splitlines()
    assert lines[0].startswith("### omega")
    f = lines[10].split()
    assert len(f) == 7 and f[3] == "(0,0)" and f[5] == "(0,0)"
    assert abs(float(f[6]) - r["eps2"][9] / 3) < 1e-9 * max(1.0, abs(r["eps2"][9]))
