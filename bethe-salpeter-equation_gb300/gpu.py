"""ctypes binding of libbse_gb300.so (the C ABI of include/bse_gpu.h).

There is no CPU fallback: if the CUDA library is missing or no GPU is present, the
calls raise.  ``BSEContext`` owns one bse_ctx and exposes every entry point of the
header with numpy buffers.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build
from .capi import BseModel, BseParams, Marshalled, ptr
from .constants import STATUS
from .model import Problem

_LIB = None
_dp = C.POINTER(C.c_double)

EXPORTS = [
    "bse_status_string", "bse_last_error", "bse_version", "bse_sizes", "bse_set_device",
    "bse_create", "bse_destroy", "bse_compute_bands", "bse_get_bands", "bse_set_bands",
    "bse_build_kernel", "bse_diagonalize", "bse_oscillators", "bse_eps", "bse_solve",
    "bse_stage_times", "bse_kernel_launches", "bse_reset_kernel_launches", "bse_eps_noalloc",
    "bse_solve_many", "bse_diagnostics", "bse_build_kernel_rows", "bse_set_kernel", "bse_wannier_m",
]


class BSEError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it with nvcc when absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} not built")
        _build.build()
    L = C.CDLL(path)
    L.bse_status_string.restype = C.c_char_p
    L.bse_status_string.argtypes = [C.c_int]
    L.bse_last_error.restype = C.c_char_p
    L.bse_last_error.argtypes = [C.c_void_p]
    L.bse_sizes.argtypes = [C.POINTER(BseModel), C.POINTER(BseParams)] + [C.POINTER(C.c_int64)] * 4
    L.bse_set_device.argtypes = [C.c_int]
    L.bse_create.argtypes = [C.POINTER(BseModel), C.POINTER(BseParams), C.POINTER(C.c_void_p)]
    L.bse_destroy.argtypes = [C.c_void_p]
    L.bse_destroy.restype = None
    L.bse_compute_bands.argtypes = [C.c_void_p]
    L.bse_get_bands.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
    L.bse_set_bands.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
    L.bse_build_kernel.argtypes = [C.c_void_p, _dp, _dp]
    L.bse_build_kernel_rows.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _dp]
    L.bse_set_kernel.argtypes = [C.c_void_p, _dp]
    L.bse_diagonalize.argtypes = [C.c_void_p, _dp, _dp]
    L.bse_oscillators.argtypes = [C.c_void_p, _dp]
    L.bse_eps.argtypes = [C.c_void_p, _dp, C.c_int32, C.c_double, _dp, _dp]
    L.bse_solve.argtypes = [C.c_void_p, _dp, C.c_int32, C.c_double, _dp, _dp, _dp]
    L.bse_stage_times.argtypes = [C.c_void_p, _dp, C.c_int32]
    L.bse_kernel_launches.argtypes = [C.c_void_p]
    L.bse_kernel_launches.restype = C.c_int64
    L.bse_reset_kernel_launches.argtypes = [C.c_void_p]
    L.bse_reset_kernel_launches.restype = None
    L.bse_eps_noalloc.argtypes = [C.c_int64, _dp, _dp, C.c_double, _dp, C.c_int32, C.c_double, _dp, _dp, C.c_void_p]
    L.bse_diagnostics.argtypes = [C.c_void_p, _dp, C.c_int32]
    L.bse_solve_many.argtypes = [C.POINTER(C.c_void_p), C.c_int32, _dp, C.c_int32, C.c_double, _dp, _dp, C.c_int32]
    _ip = C.POINTER(C.c_int32)
    L.bse_wannier_m.argtypes = [C.c_int32, C.c_int32, _ip, _ip, _dp, C.c_double, _dp, _dp, _dp, _ip, _dp, C.c_int32,
                                _dp, C.c_int32, _dp]
    _LIB = L
    return L


STAGES = ("bands", "tables", "build", "eig", "refine", "oscillators", "eps", "solve",
          "eig_tridiag", "eig_bisect", "eig_invit", "eig_backtransform", "eig_clusters",
          "eig_band", "eig_chase")


class BSEContext:
    """One bse_ctx: the model uploaded once, then the stages of the reference path."""

    def __init__(self, prob: Problem, **overrides):
        self.lib = load()
        self.m = Marshalled(prob, **overrides)
        self.prob = prob
        h = C.c_void_p()
        st = self.lib.bse_create(C.byref(self.m.model), C.byref(self.m.params), C.byref(h))
        if st != 0:
            raise BSEError(st, self.lib.bse_last_error(None).decode())
        self.h = h

    def _check(self, st):
        if st != 0:
            raise BSEError(st, self.lib.bse_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.bse_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- stages ---------------------------------------------------------------
    def compute_bands(self):
        self._check(self.lib.bse_compute_bands(self.h))

    def get_bands(self):
        ec, ev, cc, cv = self.m.band_buffers()
        self._check(self.lib.bse_get_bands(self.h, ptr(ec), ptr(ev), ptr(cc), ptr(cv)))
        return ec, ev, cc, cv

    def set_bands(self, ec, ev, cc, cv):
        arrs = [np.ascontiguousarray(x, dtype=t) for x, t in
                ((ec, np.float64), (ev, np.float64), (cc, np.complex128), (cv, np.complex128))]
        self._check(self.lib.bse_set_bands(self.h, *[ptr(a) for a in arrs]))

    def build_kernel(self, want_h: bool = False, want_rho: bool = False):
        """extract_hbse_and_rcv: returns (H or None, rho_cv or None) as numpy (row, col) arrays."""
        Hc = np.zeros((self.m.n_h, self.m.n_h), np.complex128) if want_h else None
        rho = np.zeros((self.m.ng, self.m.n_rho), np.complex128) if want_rho else None
        self._check(self.lib.bse_build_kernel(self.h, ptr(Hc), ptr(rho)))
        return (Hc.T if want_h else None), (rho.T if want_rho else None)

    def build_kernel_rows(self, k_lo: int, k_hi: int):
        """Rows of H with k in [k_lo, k_hi) (ascending r = g nk + k), shape (rows, n_h)."""
        nrows = (self.m.n_h // self.m.nk) * (k_hi - k_lo)
        out = np.zeros((self.m.n_h, max(nrows, 0)), np.complex128)   # column-major rows x n_h
        self._check(self.lib.bse_build_kernel_rows(self.h, int(k_lo), int(k_hi), ptr(out)))
        return out.T

    def set_kernel(self, H):
        """Upload the whole n_h x n_h H (numpy (row, col)) as if this context had built it."""
        Hc = np.ascontiguousarray(np.asarray(H, dtype=np.complex128).T)   # column-major bytes
        self._check(self.lib.bse_set_kernel(self.h, ptr(Hc)))

    def diagonalize(self, want_vectors: bool = False):
        E = np.zeros(self.m.n_exc)
        A = np.zeros((self.m.n_opt, self.m.n_opt), np.complex128) if want_vectors else None
        self._check(self.lib.bse_diagonalize(self.h, ptr(E), ptr(A)))
        return E, (A.T if want_vectors else None)

    def oscillators(self):
        f = np.zeros(self.m.n_opt, np.complex128)
        self._check(self.lib.bse_oscillators(self.h, ptr(f)))
        return f

    def eps(self, omega, gamma):
        om = np.ascontiguousarray(omega, dtype=np.float64)
        e2 = np.zeros(len(om))
        e1 = np.zeros(len(om))
        self._check(self.lib.bse_eps(self.h, ptr(om), len(om), float(gamma), ptr(e2), ptr(e1)))
        return e2, e1

    def solve(self, omega, gamma):
        om = np.ascontiguousarray(omega, dtype=np.float64)
        E = np.zeros(self.m.n_exc)
        e2 = np.zeros(len(om))
        e1 = np.zeros(len(om))
        self._check(self.lib.bse_solve(self.h, ptr(om), len(om), float(gamma), ptr(E), ptr(e2), ptr(e1)))
        return E, e2, e1

    def stage_times(self):
        ms = np.zeros(len(STAGES))
        self._check(self.lib.bse_stage_times(self.h, ptr(ms), len(STAGES)))
        return dict(zip(STAGES, ms.tolist()))

    def diagnostics(self):
        out = np.zeros(4)
        self._check(self.lib.bse_diagnostics(self.h, ptr(out), 4))
        return {"max_refined_residual": out[0], "clusters": int(out[1]), "n_refined": int(out[2]),
                "n_vectors": int(out[3])}

    def kernel_launches(self) -> int:
        return int(self.lib.bse_kernel_launches(self.h))

    def reset_kernel_launches(self):
        self.lib.bse_reset_kernel_launches(self.h)


def eps_noalloc(E, f, F, omega, gamma):
    """bse_eps_noalloc on host arrays: eps2, eps1 of the Lorentzian sum over the excitons (E, f)."""
    lib = load()
    E = np.ascontiguousarray(E, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.complex128)
    om = np.ascontiguousarray(omega, dtype=np.float64)
    e2 = np.zeros(len(om))
    e1 = np.zeros(len(om))
    st = lib.bse_eps_noalloc(len(E), ptr(E), ptr(f), float(F), ptr(om), len(om), float(gamma), ptr(e2), ptr(e1), None)
    if st != 0:
        raise BSEError(st, lib.bse_last_error(None).decode())
    return e2, e1


def wannier_m(functions, cells, cell_volume, origin, axes, lattice, n_int, q, g_list=None, small_q=False):
    """bse_wannier_m: real-space Wannier M [n_g, n_spin nw, n_spin nw] (complex128) from the
    functions [n_spin, nw, NX, NY, NZ] on the supercell grid r = origin + sum_p (X_p / N_p) axes[p]
    (axes, lattice: rows), for q + G over g_list (rows), or the small-q form."""
    lib = load()
    f = np.ascontiguousarray(functions, dtype=np.float64)
    if f.ndim != 5:
        raise ValueError("functions: [n_spin, nw, NX, NY, NZ]")
    n_spin, nw = f.shape[0], f.shape[1]
    i32 = lambda v: np.ascontiguousarray(v, dtype=np.int32)
    grid, cl, ni = i32(f.shape[2:]), i32(cells), i32(n_int)
    org = np.ascontiguousarray(origin, dtype=np.float64)
    ax = np.ascontiguousarray(axes, dtype=np.float64).reshape(3, 3)
    lat = np.ascontiguousarray(lattice, dtype=np.float64).reshape(3, 3)
    qq = np.ascontiguousarray(q, dtype=np.float64)
    g = None if g_list is None else np.ascontiguousarray(g_list, dtype=np.float64).reshape(-1, 3)
    n_g = 1 if g is None else len(g)
    out = np.zeros((n_g, n_spin * nw, n_spin * nw), dtype=np.complex128)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    st = lib.bse_wannier_m(n_spin, nw, ip(grid), ip(cl), ptr(f), float(cell_volume), ptr(org), ptr(ax), ptr(lat), ip(ni),
                           ptr(qq), n_g, None if g is None else ptr(g), 1 if small_q else 0, ptr(out))
    if st != 0:
        raise BSEError(st, lib.bse_last_error(None).decode())
    return out


def solve_many(contexts, omega, gamma, n_workers=8):
    """bse_solve_many over BSEContext objects: returns eps2, eps1 (n_ctx x n_omega)."""
    lib = load()
    om = np.ascontiguousarray(omega, dtype=np.float64)
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    e2 = np.zeros((len(contexts), len(om)))
    e1 = np.zeros((len(contexts), len(om)))
    st = lib.bse_solve_many(arr, len(contexts), ptr(om), len(om), float(gamma), ptr(e2), ptr(e1), int(n_workers))
    if st != 0:
        raise BSEError(st, lib.bse_last_error(None).decode())
    return e2, e1
