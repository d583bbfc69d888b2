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


def test_band_path_files(tmp_path, synth, oracle):
    """Band-structure path (Hamiltonian_TB::pull_bands, 823-875): segment file, crystal -> cartesian
    conversion, inclusive interpolation, and the bands-file layout (valence top-down then conduction
    per spin row), with the oracle's band subset as the energies."""
    from bse_gb300 import w90io
    from bse_gb300.model import Problem
    prob = synth.magnetic4_problem(grid=4)
    B = 2 * np.pi * np.linalg.inv(prob.model.lattice).T        # columns b_i
    f = tmp_path / "kpath.dat"
    f.write_text("0 0 0  0.5 0 0  5\n0.5 0 0  0.333333333333 0.333333333333 0  4\n")
    segs = w90io.read_band_path(str(f), 2, crystal=True, reciprocal=B)
    pts = w90io.band_path_points(segs)
    assert pts.shape == (9, 3)
    assert np.allclose(pts[0], 0) and np.allclose(pts[4], B @ [0.5, 0, 0]) and np.allclose(pts[5], B @ [0.5, 0, 0])
    assert np.allclose(pts[2], 0.5 * (B @ [0.5, 0, 0]))
    path_prob = Problem(model=prob.model, k_cart=pts, g_cart=prob.g_cart,
                        params=prob.params.replace(q=(0.0, 0.0, 0.0), small_momentum=0, ipa=1))
    ec, ev, _, _ = oracle.bands(path_prob)
    out = tmp_path / "bands.dat"
    w90io.write_bands(str(out), ev, ec, prob.model.n_spin)
    rows = [list(map(float, line.split())) for line in out.read_text().splitlines()]
    nv, nc = prob.params.nv, prob.params.nc
    assert len(rows) == 9 and len(rows[0]) == nv + nc
    assert np.allclose(rows[3][:nv], ev[0, 3]) and np.allclose(rows[3][nv:], ec[0, 3])
    assert all(r[nv - 1] <= prob.params.fermi_energy < r[nv] for r in rows)


def test_band_structure_needs_the_gpu(synth, gpu):
    """No CPU fallback: without a device the GPU band structure raises."""
    from bse_gb300 import bandpath
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    prob = synth.hbn_problem(grid=3)
    with pytest.raises(gpu.BSEError):
        bandpath.band_structure(prob, [(np.zeros(3), np.array([0.5, 0, 0]), 4)])
