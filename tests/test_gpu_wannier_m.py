"""GPU parity of the real-space Wannier matrix elements (bse_wannier_m, csrc/wannier_m.cu) against
the oracle's restatement (oracle/realspace.py) of the reference's Real_space_wannier +
Dipole_Elements (bse.version13.cpp:1081-1212, 1441-1456, 1503-1650).

Tolerance: FP64 on both sides, sums in different orders: 1e-11 relative to max |M|.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import realspace  # noqa: E402


def _case(seed, cells, per_cell, nw, n_spin):
    rng = np.random.default_rng(seed)
    grid = tuple(c * p for c, p in zip(cells, per_cell))
    f = rng.normal(size=(n_spin, nw) + grid)
    axes = np.array([[cells[0] * 1.0, 0.2, 0.0], [0.1, cells[1] * 1.1, 0.0], [0.0, 0.3, cells[2] * 0.9]])
    lattice = axes / np.asarray(cells, dtype=float)[:, None]
    vol = abs(np.linalg.det(lattice))
    origin = np.array([-0.3 * cells[0], 0.2, -0.1])
    return f, axes, lattice, vol, origin


@pytest.mark.parametrize("small_q", [False, True])
@pytest.mark.parametrize("shape", [((3, 2, 1), (3, 2, 2), 2, 1), ((2, 2, 2), (4, 3, 2), 3, 2)])
def test_wannier_m_matches_oracle(gpu, shape, small_q):
    cells, per_cell, nw, n_spin = shape
    f, axes, lattice, vol, origin = _case(11, cells, per_cell, nw, n_spin)
    n_int = (3, 3, 1) if cells[2] == 1 else (3, 3, 3)
    q = np.array([0.03, -0.02, 0.01]) if not small_q else np.array([2e-5, 1e-5, 0.0])
    g_list = np.array([[0.0, 0.0, 0.0], [1.3, -0.4, 0.2], [-0.7, 0.9, 2.1]])
    ref = realspace.RealSpaceWannier(f, cells, vol, origin, axes).m_q(q, g_list, lattice, n_int, small_q=small_q)
    got = gpu.wannier_m(f, cells, vol, origin, axes, lattice, n_int, q, g_list, small_q=small_q)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_wannier_m_point_like_limit(gpu):
    """Narrow Gaussians in the middle cell of a 3 x 3 x 3 cubic supercell: M_aa(q + G) ->
    exp(i q.(1, 1, 1)) exp(i (q+G).tau_a) exp(-sigma^2 |q+G|^2 / 2) (the point-like factor of the
    kernel build times the Gaussian form factor; exp(i q.(1,1,1)) is the reference's
    origin_unitcell phase)."""
    sigma, per_cell, cells = 0.07, 16, (3, 3, 3)
    taus = np.array([[0.25, 0.25, 0.5], [0.75, 0.75, 0.5]])
    grid = tuple(c * per_cell for c in cells)
    origin = np.array([-1.0, -1.0, -1.0])
    X, Y, Z = np.meshgrid(*(np.arange(n) / per_cell for n in grid), indexing="ij")
    r = origin + np.stack([X, Y, Z], axis=-1)
    f = np.stack([np.exp(-np.sum((r - t) ** 2, axis=-1) / (4 * sigma ** 2)) for t in taus])[None]
    q = np.array([0.02, -0.01, 0.0])
    g_list = 2 * np.pi * np.array([[0, 0, 0], [1, 0, 0], [0, -1, 1]], dtype=float)
    M = gpu.wannier_m(f, cells, 1.0, origin, np.diag(np.asarray(cells, dtype=float)), np.eye(3), (3, 3, 3), q, g_list)
    for g, G in enumerate(g_list):
        k = q + G
        for a in range(2):
            expect = np.exp(1j * q.sum()) * np.exp(1j * k @ taus[a]) * np.exp(-sigma ** 2 * (k @ k) / 2)
            assert abs(M[g, a, a] - expect) < 1e-6


def test_wannier_m_rejects_bad_grid(gpu):
    f = np.zeros((1, 1, 5, 4, 4))
    with pytest.raises(gpu.BSEError) as ei:
        gpu.wannier_m(f, (2, 2, 2), 1.0, np.zeros(3), np.eye(3), np.eye(3), (1, 1, 1), np.ones(3), np.zeros((1, 3)))
    assert ei.value.status == -1
