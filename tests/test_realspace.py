"""Real-space Wannier functions (the reference's Real_space_wannier and the real-space dipole
matrix elements, bse.version13.cpp:1081-1212, 1503-1675): the XSF reader/writer of the package and
the oracle's restatement of M, on the CPU.

  - XSF files round-trip, carry 22 header lines before the grid (what the reference skips) and
    follow the reference's names;
  - the vectorised dipole sums equal a literal transcription of the reference's loop nest;
  - for Gaussian functions narrow against the cell, M_ab(q + G) -> delta_ab exp(i (q+G).tau_a)
    exp(-sigma^2 |q+G|^2 / 2): the point-like exponential factor of the device path
    (function_building_exponential_factor, 1459-1501) times the Gaussian's form factor;
  - the small-q branch gives i qhat.<w_a|r|w_a> = i qhat.tau_a, the same for every G.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import realspace  # noqa: E402


@pytest.fixture(scope="module")
def w90io():
    import __graft_entry__ as entry
    entry.load_package()
    from bse_gb300 import w90io as m
    return m


def test_xsf_roundtrip_and_names(w90io, tmp_path):
    rng = np.random.default_rng(3)
    d = rng.normal(size=(6, 5, 4))
    axes = np.array([[3.0, 0.1, 0.0], [0.0, 4.0, 0.2], [0.0, 0.0, 5.0]])
    p = tmp_path / w90io.xsf_name("wf", 0)
    w90io.write_xsf_datagrid(p, d, [0.1, -0.2, 0.3], axes)
    lines = open(p).read().split("\n")
    assert lines[22].split() == ["6", "5", "4"]          # after the 22 lines the reference skips
    d2, origin, ax2 = w90io.read_xsf_datagrid(p)
    assert np.abs(d2 - d).max() <= 1e-8 * np.abs(d).max()
    assert np.allclose(origin, [0.1, -0.2, 0.3]) and np.allclose(ax2, axes)
    assert w90io.xsf_name("wf", 0) == "wf_00001.xsf"
    assert w90io.xsf_name("wf", 11, spinor=True, spin=0) == "wfup_00012.xsf"
    assert w90io.xsf_name("wf", 11, spinor=True, spin=1) == "wfdown_00012.xsf"


def test_read_wannier_xsf_order(w90io, tmp_path):
    rng = np.random.default_rng(4)
    seed = str(tmp_path / "sw")
    ref = rng.normal(size=(2, 3, 4, 4, 2))
    for s in range(2):
        for w in range(3):
            w90io.write_xsf_datagrid(w90io.xsf_name(seed, w, True, s), ref[s, w], [0, 0, 0], np.eye(3) * 2)
    data, origin, axes = w90io.read_wannier_xsf(seed, 3, spinor=True)
    assert data.shape == ref.shape and np.abs(data - ref).max() <= 1e-8 * np.abs(ref).max()


def _random_rsw(seed, cells=(3, 2, 1), per_cell=(3, 2, 2), nw=2, n_spin=1):
    rng = np.random.default_rng(seed)
    grid = tuple(c * p for c, p in zip(cells, per_cell))
    f = rng.normal(size=(n_spin, nw) + grid)
    axes = np.array([[cells[0] * 1.0, 0.2, 0.0], [0.1, cells[1] * 1.1, 0.0], [0.0, 0.3, cells[2] * 0.9]])
    vol = abs(np.linalg.det(axes)) / np.prod(cells)
    return realspace.RealSpaceWannier(f, cells, vol, [-0.3, 0.2, 0.1], axes)


def test_normalisation():
    rsw = _random_rsw(5, n_spin=2)
    norms = np.einsum("swxyz,swxyz->sw", rsw.f, rsw.f) * rsw.factor
    assert np.abs(norms - 1).max() < 1e-13


def test_vectorised_dipole_matches_literal_loops():
    rsw = _random_rsw(6)
    n_int = (3, 3, 1)
    for qg in ([0.0, 0.0, 0.0], [0.7, -1.3, 0.4]):
        for w1, w2 in ((0, 0), (0, 1), (1, 0)):
            a = rsw.dipole(w1, w2, qg, n_int)
            b = realspace.dipole_literal(rsw, w1, w2, np.asarray(qg), n_int)
            assert np.abs(a - b).max() < 1e-12 * max(1.0, np.abs(b).max())


def _gaussians(sigma=0.07, per_cell=16, cells=(3, 3, 3)):
    """Two Gaussian functions in the middle cell of a 3 x 3 x 3 simple cubic supercell (a = 1):
    the grid starts at (-1, -1, -1), so the cell holding them spans [0, 1)^3 and their tails lie
    inside the grid.  The corner nearest to zero is then that of cell (1, 1, 1)."""
    taus = np.array([[0.25, 0.25, 0.5], [0.75, 0.75, 0.5]])
    grid = tuple(c * per_cell for c in cells)
    origin = np.array([-1.0, -1.0, -1.0])
    X, Y, Z = np.meshgrid(*(np.arange(n) / per_cell for n in grid), indexing="ij")
    r = origin + np.stack([X, Y, Z], axis=-1)
    f = np.stack([np.exp(-np.sum((r - t) ** 2, axis=-1) / (4 * sigma ** 2)) for t in taus])[None]
    rsw = realspace.RealSpaceWannier(f, cells, 1.0, origin, np.diag(np.asarray(cells, dtype=float)))
    return rsw, taus


def test_point_like_limit():
    sigma = 0.07
    rsw, taus = _gaussians(sigma)
    # the reference adds origin_unitcell (cell indices) to a cartesian position in the phase of M
    # (quirk Q32): exp(i q.(1, 1, 1)) multiplies every element here
    assert np.allclose(rsw.origin_unitcell, 1.0)
    q = np.array([0.02, -0.01, 0.0])
    quirk = np.exp(1j * q.sum())
    g_list = 2 * np.pi * np.array([[0, 0, 0], [1, 0, 0], [0, -1, 1]], dtype=float)
    M = rsw.m_q(q, g_list, np.eye(3), (3, 3, 3))
    for g, G in enumerate(g_list):
        k = q + G
        for a in range(2):
            expect = quirk * np.exp(1j * k @ taus[a]) * np.exp(-sigma ** 2 * (k @ k) / 2)
            assert abs(M[g, a, a] - expect) < 1e-6, (g, a, M[g, a, a], expect)
        # off the diagonal: the home-cell pair and three translated copies of w_0 sit 0.71 from
        # w_1, each overlapping by exp(-d^2 / 8 sigma^2) ~ 2.9e-6
        off = 4 * np.exp(-0.5 / (8 * sigma ** 2))
        assert abs(M[g, 0, 1]) < 1.2 * off and abs(M[g, 1, 0]) < 1.2 * off


def test_small_q_branch_is_the_dipole():
    rsw, taus = _gaussians()
    q = np.array([3e-5, 4e-5, 0.0])
    qhat = q / np.linalg.norm(q)
    g_list = 2 * np.pi * np.array([[0, 0, 0], [1, 1, 0]], dtype=float)
    M = rsw.m_q(q, g_list, np.eye(3), (3, 3, 3), small_q=True)
    quirk = np.exp(1j * q.sum())
    for a in range(2):
        assert abs(M[0, a, a] - quirk * 1j * (qhat @ taus[a])) < 1e-6
    assert np.abs(M[0] - M[1]).max() == 0.0                 # G does not enter (kept from the reference)


def test_k_pair_matrix_elements():
    rsw = _random_rsw(7)
    k_list = np.array([[0.0, 0.0, 0.0], [0.5, 0.1, 0.0]])
    g_list = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    q = np.array([0.01, 0.0, 0.0])
    lat = np.eye(3)
    Mk = rsw.m_k1k2(q, k_list, g_list, lat, (3, 3, 1))
    for s1 in range(2):
        for s2 in range(2):
            assert np.allclose(Mk[:, s1, s2], rsw.m_q(q + k_list[s1] - k_list[s2], g_list, lat, (3, 3, 1)))
