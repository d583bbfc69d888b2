"""ctypes mirror of the structs in include/bse_gpu.h and marshalling from a Problem."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .model import Problem

_dp = C.POINTER(C.c_double)


class BseModel(C.Structure):
    _fields_ = [
        ("nw", C.c_int32), ("n_spin", C.c_int32), ("n_r", C.c_int32),
        ("r_cart", _dp), ("weights", _dp), ("h_r", _dp), ("centres", _dp), ("lattice", _dp),
        ("n_k", C.c_int32), ("k_cart", _dp),
        ("n_g", C.c_int32), ("g_cart", _dp),
    ]


class BseParams(C.Structure):
    _fields_ = [
        ("nv", C.c_int32), ("nc", C.c_int32),
        ("fermi_energy", C.c_double), ("scissor", C.c_double),
        ("q", C.c_double * 3),
        ("tamm_dancoff", C.c_int32), ("ipa", C.c_int32), ("small_momentum", C.c_int32),
        ("coulomb_kind", C.c_int32), ("coulomb_radius", C.c_double), ("coulomb_min_k2", C.c_double),
        ("w_kind", C.c_int32), ("inv_eps", C.c_double), ("rk_r0", C.c_double), ("rk_eps", C.c_double),
        ("spin_factor", C.c_double),
        ("precision", C.c_int32), ("eig_solver", C.c_int32), ("n_refine", C.c_int32),
        ("rpa_eta", C.c_double), ("rpa_order", C.c_int32), ("rpa_points", C.c_int32), ("rpa_seed", C.c_uint64),
    ]


def ptr(a: np.ndarray):
    """double* view of a C-contiguous float64/complex128 array (or NULL for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    assert a.dtype in (np.float64, np.complex128), a.dtype
    return a.ctypes.data_as(_dp)


class Marshalled:
    """Owns the contiguous arrays behind a BseModel/BseParams pair (keeps them alive)."""

    def __init__(self, prob: Problem, **overrides):
        m = prob.model
        self.r_cart = np.ascontiguousarray(m.r_cart, dtype=np.float64)            # (nR,3) == 3 x nR col-major
        self.weights = np.ascontiguousarray(m.weights, dtype=np.float64)
        # h_r[s, R, l, m] -> memory order [s][R][m][l] (column-major nw x nw per R)
        self.h_r = np.ascontiguousarray(np.swapaxes(m.h_r, -1, -2), dtype=np.complex128)
        self.centres = np.ascontiguousarray(m.centres, dtype=np.float64)         # [s][l][3]
        self.lattice = np.ascontiguousarray(m.lattice.T, dtype=np.float64)       # column-major
        self.k_cart = np.ascontiguousarray(prob.k_cart, dtype=np.float64)
        self.g_cart = np.ascontiguousarray(prob.g_cart, dtype=np.float64)
        self.model = BseModel(
            nw=m.nw, n_spin=m.n_spin, n_r=m.n_r,
            r_cart=ptr(self.r_cart), weights=ptr(self.weights), h_r=ptr(self.h_r),
            centres=ptr(self.centres), lattice=ptr(self.lattice),
            n_k=prob.nk, k_cart=ptr(self.k_cart), n_g=prob.ng, g_cart=ptr(self.g_cart))
        p = prob.params.replace(**overrides) if overrides else prob.params
        self.params = BseParams(
            nv=p.nv, nc=p.nc, fermi_energy=p.fermi_energy, scissor=p.scissor,
            q=(C.c_double * 3)(*p.q), tamm_dancoff=p.tamm_dancoff, ipa=p.ipa,
            small_momentum=p.small_momentum, coulomb_kind=p.coulomb_kind,
            coulomb_radius=p.coulomb_radius, coulomb_min_k2=p.coulomb_min_k2,
            w_kind=p.w_kind, inv_eps=p.inv_eps, rk_r0=p.rk_r0, rk_eps=p.rk_eps,
            spin_factor=p.spin_factor, precision=p.precision, eig_solver=p.eig_solver,
            n_refine=p.n_refine, rpa_eta=p.rpa_eta, rpa_order=p.rpa_order, rpa_points=p.rpa_points,
            rpa_seed=p.rpa_seed)
        self.p = p
        S = m.n_spin - 1
        self.nk, self.nc, self.nv, self.ng = prob.nk, p.nc, p.nv, prob.ng
        self.nb = m.nw * m.n_spin
        self.N = prob.nk * p.nc * p.nv
        self.coupled = p.tamm_dancoff == 0 and not p.ipa
        self.n_h = (3 * S + 1) * self.N
        self.n_rho = (S + 1) * self.N
        self.n_exc = (3 * S + 1) * self.N
        self.n_opt = (S + 1) * self.N     # optically active block (spinless N, collinear 2N)
        if self.coupled:                  # full BSE: resonant + anti-resonant exciton rows, every size doubles
            self.n_h, self.n_rho, self.n_exc, self.n_opt = 2 * self.n_h, 2 * self.n_rho, 2 * self.n_exc, 2 * self.n_opt

    def band_buffers(self):
        return (np.zeros((2, self.nk, self.nc)), np.zeros((2, self.nk, self.nv)),
                np.zeros((self.nk, self.nc, self.nb), np.complex128),
                np.zeros((self.nk, self.nv, self.nb), np.complex128))
