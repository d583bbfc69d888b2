"""Seeded synthetic tight-binding models and the workloads built on them.

The reference ships no input data (its silicon hr.dat/xsf files are absent), so every
workload is synthetic and reproducible from a seed.  The models are written in the
reference's own input formats by w90io (Wannier90 *_hr.dat, *_centres.xyz, lattice
and k-list files), so the Hamiltonian_TB reader semantics stay the entry.

Workloads (sizes as named in the benchmark configurations):
  hbn_problem        2-band honeycomb, t=-2.8, onsite +-1, 12x12, 1v x 1c, N=144
  magnetic4_problem  2 sites x 2 spins, exchange splitting 0.5 eV, SOC 0.05 eV,
                     random NNN sigma=0.1, 24x24, 2v x 2c, N=2304 (spin-orbital basis)
  collinear_problem  the same lattice in the collinear two-block form (n_spin=2, SOC=0)
  orb8_problem       8 orbitals, random onsite/NN/NNN, gap ~1.5 eV, 48x48, 4v x 4c, N=36864
  cubic3d_problem    CsCl-type 3-D two-site model with the reference's own empirical
                     inverse-epsilon W and 3-D bare Coulomb (bse.version13.cpp:2697-2728)
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from .constants import (MINVAL, BSE_V_BARE_2D, BSE_V_BARE_3D, BSE_W_EMPIRICAL,
                        BSE_W_RYTOVA_KELDYSH)
from .model import BSEParams, Problem, TBModel, g_list, mp_grid

# ---------------------------------------------------------------------------- lattices


def honeycomb_lattice(a: float = 2.5, c: float = 20.0):
    """a1=(a,0,0), a2=(a/2, a sqrt3/2, 0), a3=(0,0,c); sites A=0, B=(a1+a2)/3."""
    lat = np.array([[a, 0.0, 0.0], [a / 2, a * math.sqrt(3) / 2, 0.0], [0.0, 0.0, c]]).T
    tau = np.stack([np.zeros(3), (lat[:, 0] + lat[:, 1]) / 3.0])
    return lat, tau


def _neighbour_shells(lat, sites, rmax=2, dim=2):
    """Classify (i, j, R) site pairs by distance |tau_j + R - tau_i| into shells."""
    rng = range(-rmax, rmax + 1)
    zr = rng if dim == 3 else [0]
    pairs = []
    for i, ti in enumerate(sites):
        for j, tj in enumerate(sites):
            for r1 in rng:
                for r2 in rng:
                    for r3 in zr:
                        R = np.array([r1, r2, r3])
                        d = tj + lat @ R - ti
                        pairs.append((float(np.linalg.norm(d)), i, j, (r1, r2, r3), d))
    dists = sorted({round(p[0], 8) for p in pairs})
    return pairs, dists


class _HBuilder:
    """Accumulates H(R) blocks keyed by integer R."""

    def __init__(self, nw: int, n_spin: int = 1):
        self.nw, self.n_spin = nw, n_spin
        self.blocks: Dict[Tuple[int, int, int], np.ndarray] = {}

    def add(self, R, l, m, val, spin=0):
        R = tuple(int(x) for x in R)
        if R not in self.blocks:
            self.blocks[R] = np.zeros((self.n_spin, self.nw, self.nw), np.complex128)
        self.blocks[R][spin, l, m] += val

    def add_block(self, R, blk, spin=0):
        R = tuple(int(x) for x in R)
        if R not in self.blocks:
            self.blocks[R] = np.zeros((self.n_spin, self.nw, self.nw), np.complex128)
        self.blocks[R][spin] += blk

    def finish(self):
        keys = sorted(self.blocks.keys(), key=lambda r: (abs(r[0]) + abs(r[1]) + abs(r[2]), r))
        # R = 0 first, then by distance; every R keeps its -R partner (Hermiticity)
        for r in list(keys):
            mr = tuple(-x for x in r)
            if mr not in self.blocks:
                self.blocks[mr] = np.zeros((self.n_spin, self.nw, self.nw), np.complex128)
        keys = sorted(self.blocks.keys(), key=lambda r: (abs(r[0]) + abs(r[1]) + abs(r[2]), r))
        r_cryst = np.array(keys, dtype=np.int64).reshape(-1, 3)
        h_r = np.stack([self.blocks[k] for k in keys], axis=1)   # (n_spin, nR, nw, nw)
        return r_cryst, h_r


# ---------------------------------------------------------------------------- models


def hbn_model(a=2.5, c=20.0, t=-2.8, onsite=1.0) -> TBModel:
    """Two-band hBN-like honeycomb model: onsite +onsite (A), -onsite (B), NN hopping t."""
    lat, tau = honeycomb_lattice(a, c)
    hb = _HBuilder(2)
    hb.add((0, 0, 0), 0, 0, onsite)
    hb.add((0, 0, 0), 1, 1, -onsite)
    pairs, dists = _neighbour_shells(lat, tau, rmax=1)
    dnn = dists[1]
    for d, i, j, R, _ in pairs:
        if i != j and abs(d - dnn) < 1e-6:
            hb.add(R, i, j, t)
    r_cryst, h_r = hb.finish()
    m = TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                centres=tau[None, :, :].copy(), dim=2, name="hbn")
    return m


MAGNETIC4_NOMINAL = np.array([1.0, 0.25, -2.8, 0.05] + [1.0] * 8)
MAGNETIC4_PARAM_NAMES = (["onsite", "exchange", "t_nn", "soc"] +
                         [f"nnn_{p}" for p in range(8)])


def magnetic4_basis(seed=1234, a=2.5, c=20.0, sigma=0.1):
    """Basis matrices B_p(R) of the spinful 4-orbital honeycomb model, H(R) = sum_p theta_p B_p(R).

    Orbitals (A up, B up, A down, B down).  p = 0 onsite sublattice sign, 1 exchange
    (spin sign), 2 NN hopping, 3 Kane-Mele SOC i nu_ij sigma_z on NNN, 4..11 eight
    independent random NNN patterns (complex Gaussian, std sigma/sqrt(8) each, H(-R) = H(R)^dagger).
    Returns (lattice, centres (1,4,3), list of dicts R->(4,4) block)."""
    lat, tau = honeycomb_lattice(a, c)
    site = [0, 1, 0, 1]
    spin = [1.0, 1.0, -1.0, -1.0]
    centres = np.stack([tau[s] for s in site])[None, :, :]
    pairs, dists = _neighbour_shells(lat, tau, rmax=2)
    dnn, dnnn = dists[1], dists[2]
    basis: List[Dict[Tuple[int, int, int], np.ndarray]] = [dict() for _ in range(12)]

    def put(p, R, l, m, v):
        R = tuple(int(x) for x in R)
        basis[p].setdefault(R, np.zeros((4, 4), np.complex128))
        basis[p][R][l, m] += v

    for l in range(4):
        put(0, (0, 0, 0), l, l, 1.0 if site[l] == 0 else -1.0)
        put(1, (0, 0, 0), l, l, spin[l])
    nn = [(i, j, R, d) for dd, i, j, R, d in pairs if i != j and abs(dd - dnn) < 1e-6]
    nnn = [(i, j, R, d) for dd, i, j, R, d in pairs if i == j and abs(dd - dnnn) < 1e-6]
    for i, j, R, _ in nn:
        for l in range(4):
            for m in range(4):
                if site[l] == i and site[m] == j and spin[l] == spin[m]:
                    put(2, R, l, m, 1.0)
    # Kane-Mele chirality nu = sign((d1 x d2)_z) through the intermediate NN site
    for i, j, R, dvec in nnn:
        nu = 0.0
        for i2, j2, R2, d1 in nn:
            if i2 != i:
                continue
            d2 = dvec - d1
            if abs(np.linalg.norm(d2) - dnn) < 1e-6:
                nu = float(np.sign(np.cross(d1, d2)[2]))
                break
        for l in range(4):
            for m in range(4):
                if site[l] == i and site[m] == i and spin[l] == spin[m]:
                    put(3, R, l, m, 1j * nu * spin[l])
    rng = np.random.default_rng(seed)
    pos_R = sorted({R for _, _, R, _ in nnn if R > tuple(-x for x in R)})
    sp = sigma / math.sqrt(8.0)
    for p in range(8):
        for R in pos_R:
            g = np.zeros((4, 4), np.complex128)
            for l in range(4):
                for m in range(4):
                    if site[l] == site[m]:
                        g[l, m] = sp * (rng.standard_normal() + 1j * rng.standard_normal()) / math.sqrt(2)
            mR = tuple(-x for x in R)
            basis[4 + p].setdefault(R, np.zeros((4, 4), np.complex128))
            basis[4 + p].setdefault(mR, np.zeros((4, 4), np.complex128))
            basis[4 + p][R] += g
            basis[4 + p][mR] += g.conj().T
    return lat, centres, basis


def magnetic4_model(theta=None, seed=1234, a=2.5, c=20.0, sigma=0.1) -> TBModel:
    """Spinful 4-orbital honeycomb model (exchange splitting 2*theta[1], SOC theta[3])."""
    theta = MAGNETIC4_NOMINAL if theta is None else np.asarray(theta, dtype=np.float64)
    lat, centres, basis = magnetic4_basis(seed, a, c, sigma)
    hb = _HBuilder(4)
    for p, b in enumerate(basis):
        for R, blk in b.items():
            hb.add_block(R, theta[p] * blk)
    r_cryst, h_r = hb.finish()
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                   centres=centres.copy(), dim=2, name="magnetic4")


def collinear_model(seed=1234, a=2.5, c=20.0, onsite=1.0, exch=0.25, t=-2.8, sigma=0.1) -> TBModel:
    """Collinear-magnetic form of the same lattice: two spin channels (n_spin=2), nw=2 each,
    no SOC, spin-diagonal random NNN hoppings (the reference's spinorial_calculation=1 path)."""
    lat, tau = honeycomb_lattice(a, c)
    hb = _HBuilder(2, n_spin=2)
    pairs, dists = _neighbour_shells(lat, tau, rmax=2)
    dnn, dnnn = dists[1], dists[2]
    rng = np.random.default_rng(seed)
    for s, sg in enumerate((1.0, -1.0)):
        hb.add((0, 0, 0), 0, 0, onsite + sg * exch, spin=s)
        hb.add((0, 0, 0), 1, 1, -onsite + sg * exch, spin=s)
        for d, i, j, R, _ in pairs:
            if i != j and abs(d - dnn) < 1e-6:
                hb.add(R, i, j, t, spin=s)
        for d, i, j, R, _ in pairs:
            if i == j and abs(d - dnnn) < 1e-6 and R > tuple(-x for x in R):
                g = sigma * (rng.standard_normal() + 1j * rng.standard_normal()) / math.sqrt(2)
                hb.add(R, i, i, g, spin=s)
                hb.add(tuple(-x for x in R), i, i, np.conj(g), spin=s)
    r_cryst, h_r = hb.finish()
    centres = np.stack([tau, tau])
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                   centres=centres, dim=2, name="collinear")


def _rand_herm(rng, n, sigma):
    x = sigma * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    return (x + x.conj().T) / 2


def orb8_model(seed=2024, e0=2.0, a=2.5, c=20.0, sig_on=0.3, sig_nn=0.6, sig_nnn=0.1) -> TBModel:
    """8-orbital honeycomb model: orbitals 0-3 on A around -e0, 4-7 on B around +e0,
    random Hermitian onsite blocks, random complex NN (A-B) and NNN (A-A, B-B) hoppings."""
    lat, tau = honeycomb_lattice(a, c)
    rng = np.random.default_rng(seed)
    hb = _HBuilder(8)
    hb.add_block((0, 0, 0), np.zeros((8, 8)))
    onA = _rand_herm(rng, 4, sig_on) - e0 * np.eye(4)
    onB = _rand_herm(rng, 4, sig_on) + e0 * np.eye(4)
    blk = np.zeros((8, 8), np.complex128)
    blk[:4, :4] = onA
    blk[4:, 4:] = onB
    hb.add_block((0, 0, 0), blk)
    pairs, dists = _neighbour_shells(lat, tau, rmax=2)
    dnn, dnnn = dists[1], dists[2]
    for d, i, j, R, _ in pairs:
        if i == 0 and j == 1 and abs(d - dnn) < 1e-6:
            g = sig_nn * (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
            b1 = np.zeros((8, 8), np.complex128)
            b1[:4, 4:] = g
            hb.add_block(R, b1)
            hb.add_block(tuple(-x for x in R), b1.conj().T)
    for d, i, j, R, _ in pairs:
        if i == j and abs(d - dnnn) < 1e-6 and R > tuple(-x for x in R):
            g = sig_nnn * (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
            b1 = np.zeros((8, 8), np.complex128)
            o = 4 * i
            b1[o:o + 4, o:o + 4] = g
            hb.add_block(R, b1)
            hb.add_block(tuple(-x for x in R), b1.conj().T)
    r_cryst, h_r = hb.finish()
    centres = np.stack([tau[0]] * 4 + [tau[1]] * 4)[None, :, :]
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                   centres=centres, dim=2, name="orb8")


def cubic3d_model(a=3.0, onsite=1.5, t=-1.0) -> TBModel:
    """CsCl-type two-site cubic model (A at 0, B at body centre), one orbital per site."""
    lat = np.eye(3) * a
    tau = np.stack([np.zeros(3), np.full(3, a / 2)])
    hb = _HBuilder(2)
    hb.add((0, 0, 0), 0, 0, onsite)
    hb.add((0, 0, 0), 1, 1, -onsite)
    pairs, dists = _neighbour_shells(lat, tau, rmax=1, dim=3)
    dnn = dists[1]
    for d, i, j, R, _ in pairs:
        if i != j and abs(d - dnn) < 1e-6:
            hb.add(R, i, j, t)
    r_cryst, h_r = hb.finish()
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                   centres=tau[None, :, :].copy(), dim=3, name="cubic3d")


# ---------------------------------------------------------------------------- gaps


def band_edges(model: TBModel, k_cart: np.ndarray, n_val: int):
    """(max valence, min conduction) over the k list, counting n_val bands per spin channel."""
    e = np.linalg.eigvalsh(model.hk(k_cart))            # (n_spin, nk, nw)
    return float(e[..., :n_val].max()), float(e[..., n_val:].min())


def _tune_orb8(seed, grid, gap):
    lat, _ = honeycomb_lattice()
    k, _ = mp_grid(lat, (grid, grid, 1))

    def g_of(e0):
        m = orb8_model(seed=seed, e0=e0)
        vb, cb = band_edges(m, k, 4)
        return cb - vb, m, vb, cb

    lo, hi = 0.5, 6.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        g, _, _, _ = g_of(mid)
        if g < gap:
            lo = mid
        else:
            hi = mid
    g, m, vb, cb = g_of(hi)
    return m, 0.5 * (vb + cb), g


# ---------------------------------------------------------------------------- problems

G_CUTOFF_2D = 6.0      # -> n = 2 shells along b1, b2 for a = 2.5 A: NG = 25


def _problem2d(model, grid, nv, nc, ef, cutoff=G_CUTOFF_2D, shift=(0, 0, 0), **kw):
    k, kc = mp_grid(model.lattice, (grid, grid, 1), shift)
    g = g_list(model.lattice, cutoff, dim=2)
    p = BSEParams(nv=nv, nc=nc, fermi_energy=ef, coulomb_kind=BSE_V_BARE_2D,
                  w_kind=BSE_W_RYTOVA_KELDYSH, rk_r0=10.0, rk_eps=1.0, **kw)
    return Problem(model=model, k_cart=k, g_cart=g, params=p, k_cryst=kc, grid=(grid, grid, 1))


def hbn_problem(grid=12, **kw) -> Problem:
    """2-band hBN-like model, 12x12, 1v x 1c, RK W (r0=10 A, eps=1) + bare 2-D V (N=144)."""
    return _problem2d(hbn_model(), grid, 1, 1, 0.0, **kw)


def magnetic4_problem(grid=24, theta=None, seed=1234, **kw) -> Problem:
    """Spinful 4-orbital model in the spin-orbital basis, 24x24, 2v x 2c (N=2304); exchange
    spin factor 1 (spin-orbital basis)."""
    kw.setdefault("spin_factor", 1.0)
    return _problem2d(magnetic4_model(theta=theta, seed=seed), grid, 2, 2, 0.0, **kw)


def collinear_problem(grid=12, seed=1234, **kw) -> Problem:
    """Collinear two-channel model (n_spin=2), 1v x 1c per channel pair."""
    return _problem2d(collinear_model(seed=seed), grid, 1, 1, 0.0, **kw)


def orb8_problem(grid=48, seed=2024, gap=1.5, nv=4, nc=4, **kw) -> Problem:
    """8-orbital model tuned to a ~1.5 eV gap on the 48x48 grid, 4v x 4c (N=36864 at 48x48)."""
    m, ef, _ = _tune_orb8(seed, 48, gap)
    kw.setdefault("n_refine", 256)
    return _problem2d(m, grid, nv, nc, ef, **kw)


def cubic3d_problem(grid=4, cutoff=2.2, **kw) -> Problem:
    """3-D two-site cubic model with the reference's own insulator mode: 3-D bare v,
    empirical inverse epsilon W, G cutoff in the 3-D branch."""
    m = cubic3d_model()
    k, kc = mp_grid(m.lattice, (grid, grid, grid))
    g = g_list(m.lattice, cutoff, dim=3)
    p = BSEParams(nv=1, nc=1, fermi_energy=0.0, coulomb_kind=BSE_V_BARE_3D,
                  w_kind=BSE_W_EMPIRICAL, **kw)
    return Problem(model=m, k_cart=k, g_cart=g, params=p, k_cryst=kc, grid=(grid, grid, grid))


def random_batch_problems(n_models=64, seed=77, grid_range=(12, 30)):
    """Batched workload: seeded 2- to 4-band honeycomb models with uneven grids."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_models):
        nw = int(rng.integers(2, 5))
        grid = int(rng.integers(grid_range[0], grid_range[1] + 1))
        nv = int(rng.integers(1, 3)) if nw >= 3 else 1
        nc = int(rng.integers(1, 3)) if nw - nv >= 2 else 1
        if nw == 2:
            nv = nc = 1
        m = _random_honeycomb(rng, nw)
        out.append((m, grid, nv, nc))
    probs = []
    for m, grid, nv, nc in out:
        lat = m.lattice
        k, _ = mp_grid(lat, (grid, grid, 1))
        e = np.linalg.eigvalsh(m.hk(k))[0]
        nval = m.nw // 2
        ef = 0.5 * (e[:, nval - 1].max() + e[:, nval:].min())
        nv = min(nv, nval)
        nc = min(nc, m.nw - nval)
        probs.append(_problem2d(m, grid, nv, nc, ef))
    return probs


def _random_honeycomb(rng, nw):
    lat, tau = honeycomb_lattice()
    nA = (nw + 1) // 2
    site = [0] * nA + [1] * (nw - nA)
    hb = _HBuilder(nw)
    on = np.zeros((nw, nw), np.complex128)
    for l in range(nw):
        on[l, l] = (-1.5 if l < nw // 2 else 1.5) + 0.2 * rng.standard_normal()
    hb.add_block((0, 0, 0), on)
    pairs, dists = _neighbour_shells(lat, tau, rmax=1)
    dnn = dists[1]
    for d, i, j, R, _ in pairs:
        if i == 0 and j == 1 and abs(d - dnn) < 1e-6:
            blk = np.zeros((nw, nw), np.complex128)
            for l in range(nw):
                for m in range(nw):
                    if site[l] == 0 and site[m] == 1:
                        blk[l, m] = 0.8 * (rng.standard_normal() + 1j * rng.standard_normal()) / math.sqrt(2)
            hb.add_block(R, blk)
            hb.add_block(tuple(-x for x in R), blk.conj().T)
    r_cryst, h_r = hb.finish()
    centres = np.stack([tau[s] for s in site])[None, :, :]
    return TBModel(lattice=lat, r_cryst=r_cryst, weights=np.ones(len(r_cryst)), h_r=h_r,
                   centres=centres, dim=2, name=f"rand{nw}")
