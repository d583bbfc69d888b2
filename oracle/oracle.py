"""Python driver of the CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use
this module, as the checker.  It calls the C++ restatement in bse_oracle.cpp for the
band states, pair densities and kernel build, and LAPACK zheevd through
scipy.linalg.eigh(driver="evd") for the dense solve -- the routine Armadillo's
eig_sym dispatches to in Excitonic_Hamiltonian::common_diagonalization
(bse.version13.cpp:3330); for the full BSE (tamm_dancoff = 0) numpy's zgeev, as the
reference's eig_gen (3326), with the spectrum through the inverse overlap matrix of the
eigenvectors (solve_coupled); rpa_w builds the RPA screened interaction table that build() can
use in place of the model W.  Parity against the reference binary is UNPINNED (the
reference cannot be built here); see the header of bse_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import sys
import time

import numpy as np
import scipy.linalg

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402


def _pkg():
    if "bse_gb300" in sys.modules:
        return sys.modules["bse_gb300"]
    pdir = os.path.join(ROOT, "bethe-salpeter-equation_gb300")
    spec = importlib.util.spec_from_file_location("bse_gb300", os.path.join(pdir, "__init__.py"),
                                                  submodule_search_locations=[pdir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["bse_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        capi = _pkg().capi
        L.oracle_bands.argtypes = [C.POINTER(capi.BseModel), C.POINTER(capi.BseParams), dp, dp, dp, dp]
        L.oracle_build.argtypes = [C.POINTER(capi.BseModel), C.POINTER(capi.BseParams), dp, dp, dp, dp, dp, dp, dp]
        L.oracle_rpa_eps_inv.argtypes = [C.POINTER(capi.BseModel), C.POINTER(capi.BseParams), dp, C.c_double, C.c_int,
                                         dp, dp]
        L.oracle_rpa_w.argtypes = [C.POINTER(capi.BseModel), C.POINTER(capi.BseParams), C.c_double, C.c_int, C.c_int,
                                   C.c_uint64, dp]
        L.oracle_prefactor.argtypes = [C.POINTER(capi.BseModel), C.POINTER(capi.BseParams)]
        L.oracle_prefactor.restype = C.c_double
        L.oracle_oscillators.argtypes = [C.c_int64, C.c_int64, dp, dp, dp]
        L.oracle_eps.argtypes = [C.c_int64, dp, dp, C.c_double, dp, C.c_int32, C.c_double, dp, dp]
        L.oracle_num_threads.restype = C.c_int
        _LIB = L
    return _LIB


class OracleError(RuntimeError):
    pass


def _check(st):
    if st != 0:
        raise OracleError(f"oracle status {st}")


def bands(prob, **overrides):
    """(e_c [2,nk,nc], e_v [2,nk,nv], c_c [nk,nc,nb], c_v [nk,nv,nb]); c at k, v at k-q."""
    M = _pkg().capi.Marshalled(prob, **overrides)
    ec, ev, cc, cv = M.band_buffers()
    p = _pkg().capi.ptr
    _check(lib().oracle_bands(C.byref(M.model), C.byref(M.params), p(ec), p(ev), p(cc), p(cv)))
    return ec, ev, cc, cv


def rpa_eps_inv(prob, q, eta=0.0, order=1, **overrides):
    """chi0 and eps^-1 (ng x ng) at momentum q (Dielectric_Function::pull_values 2214-2315)."""
    M = _pkg().capi.Marshalled(prob, **overrides)
    chi0 = np.zeros((prob.ng, prob.ng), np.complex128)      # C order (col, row) == column-major (row, col)
    einv = np.zeros((prob.ng, prob.ng), np.complex128)
    qq = np.ascontiguousarray(q, dtype=np.float64)
    p = _pkg().capi.ptr
    _check(lib().oracle_rpa_eps_inv(C.byref(M.model), C.byref(M.params), p(qq), eta, order, p(chi0), p(einv)))
    return chi0.T, einv.T


def rpa_w(prob, eta=0.0, order=1, n_points=64, seed=1, **overrides):
    """RPA screened interaction for every k pair: array [nk, nk, ng, ng] (numpy (row, col) per pair),
    W[i, j] = W(k_i - k_j) (pull_coulomb_potentials 2597-2690, decisions Q28/Q29)."""
    M = _pkg().capi.Marshalled(prob, **overrides)
    nk, ng = prob.nk, prob.ng
    w = np.zeros((nk, nk, ng, ng), np.complex128)            # per pair: C order (s, g) == column-major (g, s)
    p = _pkg().capi.ptr
    _check(lib().oracle_rpa_w(C.byref(M.model), C.byref(M.params), eta, order, n_points, seed, p(w)))
    return np.swapaxes(w, -1, -2)


def build(prob, band_states=None, w_table=None, **overrides):
    """Full BSE matrix (n_h x n_h, spin-rotated for collinear models) and rho_cv (n_rho x ng).
    w_table: an RPA W from rpa_w() replacing the model W of the direct terms."""
    M = _pkg().capi.Marshalled(prob, **overrides)
    if band_states is None:
        band_states = bands(prob, **overrides)
    if w_table is None and M.p.w_kind == 3 and not M.p.ipa:       # BSE_W_RPA
        w_table = rpa_w(prob, M.p.rpa_eta, M.p.rpa_order, M.p.rpa_points, M.p.rpa_seed, **overrides)
    ec, ev, cc, cv = [np.ascontiguousarray(x) for x in band_states]
    H = np.zeros((M.n_h, M.n_h), np.complex128, order="F")
    rho = np.zeros((M.ng, M.n_rho), np.complex128)      # C order (ng, n_rho) == column-major n_rho x ng
    p = _pkg().capi.ptr
    Hc = np.zeros((M.n_h, M.n_h), np.complex128)         # C buffer, filled column-major
    wt = None if w_table is None else np.ascontiguousarray(np.swapaxes(w_table, -1, -2), dtype=np.complex128)
    _check(lib().oracle_build(C.byref(M.model), C.byref(M.params), p(ec), p(ev), p(cc), p(cv),
                              p(Hc), p(rho), p(wt)))
    H = Hc.T                                             # column-major -> numpy (row, col)
    return H, rho.T


def prefactor(prob, **overrides):
    M = _pkg().capi.Marshalled(prob, **overrides)
    return float(lib().oracle_prefactor(C.byref(M.model), C.byref(M.params)))


def split_blocks(H, n_bse):
    """Collinear models: H0 = rotated spin-flip blocks {1,2}, H1 = spin-conserving {0,3}
    (common_diagonalization, bse.version13.cpp:3143-3149)."""
    N = n_bse
    idx0 = np.r_[N:3 * N]
    idx1 = np.r_[0:N, 3 * N:4 * N]
    return H[np.ix_(idx0, idx0)], H[np.ix_(idx1, idx1)]


def split_blocks_coupled(H, n_bse):
    """Collinear full BSE (8N x 8N): H0 = blocks {1,2} and H1 = blocks {0,3} of every quadrant,
    each 4N x 4N with its own coupling part (common_diagonalization, bse.version13.cpp:3151-3172)."""
    N = n_bse
    b0 = np.r_[N:3 * N]
    b1 = np.r_[0:N, 3 * N:4 * N]
    idx0 = np.r_[b0, 4 * N + b0]
    idx1 = np.r_[b1, 4 * N + b1]
    return H[np.ix_(idx0, idx0)], H[np.ix_(idx1, idx1)]


def eigh(H, eigvals_only=False):
    """LAPACK zheevd (or cheevd for complex64), ascending."""
    if eigvals_only:
        return scipy.linalg.eigh(H, eigvals_only=True, driver="evd", check_finite=False)
    return scipy.linalg.eigh(H, driver="evd", check_finite=False)


def oscillators(rho_g0, A):
    A = np.asfortranarray(A, dtype=np.complex128)
    r = np.ascontiguousarray(rho_g0, dtype=np.complex128)
    f = np.zeros(A.shape[1], np.complex128)
    p = _pkg().capi.ptr
    # column-major A has the same bytes as the C-ordered transpose
    At = np.ascontiguousarray(A.T)
    _check(lib().oracle_oscillators(A.shape[0], A.shape[1], p(r), p(At), p(f)))
    return f


def eps(E, f, F, omega, gamma):
    E = np.ascontiguousarray(E, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.complex128)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    e2 = np.zeros(len(omega))
    e1 = np.zeros(len(omega))
    p = _pkg().capi.ptr
    _check(lib().oracle_eps(len(E), p(E), p(f), F, p(omega), len(omega), gamma, p(e2), p(e1)))
    return e2, e1


def solve_coupled(H, rho_g0, F, omega, gamma):
    """Full (non-Tamm-Dancoff) BSE on the CPU, the reference's route: eig_gen of the 2N x 2N
    matrix (LAPACK zgeev, common_diagonalization 3326), eigenpairs sorted by real part (3335),
    and the spectrum through the inverse overlap ("augmentation") matrix of the eigenvectors
    (pull_augmentation_matrix 3504-3522, omega loop 3607-3620), here over all 2N eigenpairs:
      eps(w) = 1 - F rho^H V diag(1 / (w - E + i gamma)) S^{-1} V^H J rho,  S = V^H V,
    i.e. 1 - F rho^H (w - H + i gamma)^{-1} J rho with J = diag(1, -1) over the two exciton
    blocks (the reference's N x N truncation of S and its pairing of rows are not reproduced).
    Also returns the J-normalised eigenvectors (x^H J x = sign(E)) and f = rho^H x."""
    n = H.shape[0]
    N = n // 2
    w, V = np.linalg.eig(H)
    order = np.argsort(w.real, kind="stable")
    w, V = w[order], V[:, order]
    V = V / np.linalg.norm(V, axis=0)                         # unit columns (3337-3343)
    J = np.r_[np.ones(N), -np.ones(N)]
    rho = np.asarray(rho_g0, dtype=np.complex128)
    S = V.conj().T @ V
    b = np.linalg.solve(S, V.conj().T @ (J * rho))            # S^{-1} V^H J rho
    a = V.conj().T @ rho                                      # V^H rho
    om = np.asarray(omega, dtype=np.float64)
    chi = (np.conj(a)[None, :] * b[None, :] / (om[:, None] - w[None, :] + 1j * gamma)).sum(axis=1)
    eps = 1.0 - F * chi
    jn = np.einsum("il,i,il->l", V.conj(), J, V).real         # x^H J x of the unit vectors
    X = V / np.sqrt(np.abs(jn))
    f = X.T @ np.conj(rho)
    return {"E": w.real, "E_imag": w.imag, "X": X, "f": f, "jnorm_sign": np.sign(jn),
            "eps2": eps.imag, "eps1": eps.real}


def solve(prob, omega, gamma, band_states=None, want_vectors=True, timings=None, w_table=None, **overrides):
    """Whole reference path on the CPU: bands -> build -> zheevd -> oscillators -> eps."""
    t0 = time.perf_counter()
    if band_states is None:
        band_states = bands(prob, **overrides)
    t1 = time.perf_counter()
    H, rho = build(prob, band_states, w_table=w_table, **overrides)
    t2 = time.perf_counter()
    N = prob.n_bse
    ng0 = prob.ng // 2
    out = {"bands": band_states, "H": H, "rho": rho}
    p = prob.params.replace(**overrides) if overrides else prob.params
    if p.tamm_dancoff == 0 and not p.ipa:
        F = prefactor(prob, **overrides)
        if prob.model.n_spin == 2:
            # both spin blocks diagonalised (3195, 3204); the spectrum from the spin-conserving H1 (Q17)
            H0, H1 = split_blocks_coupled(H, N)
            w0 = np.linalg.eigvals(H0)
            E0 = np.sort_complex(w0[np.lexsort((w0.imag, w0.real))]).real
            res = solve_coupled(H1, rho[:, ng0], F, omega, gamma)
            E_all = np.concatenate([E0, res["E"]])
        else:
            res = solve_coupled(H, rho[:, ng0], F, omega, gamma)
            E_all = res["E"]
        t3 = time.perf_counter()
        out.update(E=E_all, E_opt=res["E"], A=res["X"], f=res["f"], F=F, eps2=res["eps2"], eps1=res["eps1"],
                   E_imag=res["E_imag"])
        if timings is not None:
            timings.update(bands=t1 - t0, build=t2 - t1, eig=t3 - t2, eps=0.0)
        return out
    if prob.model.n_spin == 2:
        H0, H1 = split_blocks(H, N)
        E0 = eigh(H0, eigvals_only=True)
        E1, A1 = eigh(H1)
        E_all = np.concatenate([E0, E1])
        E_opt, A = E1, A1
    else:
        E_opt, A = eigh(H)
        E_all = E_opt
    t3 = time.perf_counter()
    f = oscillators(rho[:, ng0], A)
    F = prefactor(prob, **overrides)
    e2, e1 = eps(E_opt, f, F, omega, gamma)
    t4 = time.perf_counter()
    out.update(E=E_all, E_opt=E_opt, A=A, f=f, F=F, eps2=e2, eps1=e1)
    if timings is not None:
        timings.update(bands=t1 - t0, build=t2 - t1, eig=t3 - t2, eps=t4 - t3)
    return out
