"""CPU tests of the C ABI: the library loads, exports every function include/bse_gpu.h
declares, and rejects bad inputs before touching a device (no compute without a GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "bse_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bse_\w+)\s*\(", src)))


def test_library_exports_header(gpu):
    lib = gpu.load()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(gpu.EXPORTS) == set(names)


def test_status_strings(gpu):
    lib = gpu.load()
    assert lib.bse_status_string(0) == b"BSE_OK"
    assert lib.bse_status_string(-4) == b"BSE_ERR_NOT_CONVERGED"


def _create(gpu, prob, **kw):
    lib = gpu.load()
    from bse_gb300.capi import Marshalled
    m = Marshalled(prob, **kw)
    h = C.c_void_p()
    st = lib.bse_create(C.byref(m.model), C.byref(m.params), C.byref(h))
    if st == 0:
        lib.bse_destroy(h)
    return st, lib.bse_last_error(None).decode()


def test_rejects_too_many_bands(synth, gpu):
    st, msg = _create(gpu, synth.hbn_problem(grid=2), nv=2)
    assert st == -1 and "nv + nc" in msg


def test_rejects_non_hermitian(synth, gpu):
    prob = synth.hbn_problem(grid=2)
    prob.model.h_r = prob.model.h_r.copy()
    prob.model.h_r[0, 1, 0, 1] += 0.3j
    st, msg = _create(gpu, prob)
    assert st == -1 and "Hermitian" in msg


def test_rejects_nan(synth, gpu):
    prob = synth.hbn_problem(grid=2)
    prob.k_cart = prob.k_cart.copy()
    prob.k_cart[1, 0] = np.nan
    st, msg = _create(gpu, prob)
    assert st == -1 and "NaN" in msg


def test_full_bse_validation(synth, gpu):
    """tamm_dancoff = 0 (coupling block): FP64, or mixed with the own solver."""
    st, msg = _create(gpu, synth.hbn_problem(grid=2), tamm_dancoff=2)
    assert st == -1 and "tamm_dancoff" in msg
    st, _ = _create(gpu, synth.hbn_problem(grid=2), tamm_dancoff=0, precision=1)
    assert st in (0, -2)
    st, msg = _create(gpu, synth.hbn_problem(grid=2), tamm_dancoff=0, precision=1, eig_solver=1)
    assert st == -1 and "own eigensolver" in msg
    st, _ = _create(gpu, synth.collinear_problem(grid=2), tamm_dancoff=0, precision=1)
    assert st in (0, -2)
    st, _ = _create(gpu, synth.collinear_problem(grid=2), tamm_dancoff=0)
    assert st in (0, -2)
    st, _ = _create(gpu, synth.hbn_problem(grid=2), tamm_dancoff=0)
    assert st in (0, -2)
    st, _ = _create(gpu, synth.collinear_problem(grid=2), tamm_dancoff=0, ipa=1, precision=1)
    assert st in (0, -2)                      # no kernel: the coupling flag has no effect


def test_full_bse_sizes(synth, gpu):
    from bse_gb300.capi import Marshalled
    lib = gpu.load()
    prob = synth.hbn_problem(grid=3)
    out = [C.c_int64() for _ in range(4)]
    for tda, factor in ((1, 1), (0, 2)):
        m = Marshalled(prob, tamm_dancoff=tda)
        assert lib.bse_sizes(C.byref(m.model), C.byref(m.params), *[C.byref(x) for x in out]) == 0
        N = prob.n_bse
        assert [x.value for x in out] == [N, factor * N, factor * N, factor * N]
        assert (m.n_exc, m.n_rho, m.n_h, m.n_opt) == (factor * N,) * 4
    prob = synth.collinear_problem(grid=3)
    N = prob.n_bse
    m = Marshalled(prob, tamm_dancoff=0)
    assert lib.bse_sizes(C.byref(m.model), C.byref(m.params), *[C.byref(x) for x in out]) == 0
    assert [x.value for x in out] == [N, 8 * N, 4 * N, 8 * N]
    assert (m.n_exc, m.n_rho, m.n_h, m.n_opt) == (8 * N, 4 * N, 8 * N, 4 * N)


def test_rejects_zero_q(synth, gpu):
    st, msg = _create(gpu, synth.hbn_problem(grid=2), q=(0.0, 0.0, 0.0))
    assert st == -1


def test_no_device_is_an_error_not_a_crash(synth, gpu):
    """Here (no GPU) a valid problem yields BSE_ERR_NO_DEVICE; on a GPU machine it succeeds."""
    st, msg = _create(gpu, synth.hbn_problem(grid=2))
    assert st in (0, -2)


def test_sizes(synth, gpu):
    lib = gpu.load()
    from bse_gb300.capi import Marshalled
    m = Marshalled(synth.collinear_problem(grid=3))
    vals = [C.c_int64() for _ in range(4)]
    assert lib.bse_sizes(C.byref(m.model), C.byref(m.params), *[C.byref(v) for v in vals]) == 0
    N = 9
    assert [v.value for v in vals] == [N, 4 * N, 2 * N, 4 * N]


def test_null_context_is_an_error_not_a_crash(gpu):
    """Every entry point taking a context returns BSE_ERR_BAD_INPUT for NULL (checked before any
    device call), the destructors accept NULL, and the allocation-free spectrum validates its
    sizes first."""
    lib = gpu.load()
    null = C.c_void_p()
    dp = C.POINTER(C.c_double)()
    assert lib.bse_compute_bands(null) == -1
    assert lib.bse_get_bands(null, dp, dp, dp, dp) == -1
    assert lib.bse_set_bands(null, dp, dp, dp, dp) == -1
    assert lib.bse_build_kernel(null, dp, dp) == -1
    assert lib.bse_diagonalize(null, dp, dp) == -1
    assert lib.bse_oscillators(null, dp) == -1
    assert lib.bse_eps(null, dp, 0, 0.05, dp, dp) == -1
    assert lib.bse_solve(null, dp, 0, 0.05, dp, dp, dp) == -1
    assert lib.bse_stage_times(null, dp, 0) == -1
    assert lib.bse_diagnostics(null, dp, 0) == -1
    assert lib.bse_kernel_launches(null) == 0
    lib.bse_reset_kernel_launches(null)
    lib.bse_destroy(null)
    assert lib.bse_solve_many(C.POINTER(C.c_void_p)(), 1, dp, 0, 0.05, dp, dp, 1) == -1
    assert lib.bse_sizes(None, None, None, None, None, None) == -1
    assert isinstance(lib.bse_last_error(None), bytes)
    one = np.ones(4)
    assert lib.bse_eps_noalloc(0, one.ctypes.data_as(C.POINTER(C.c_double)), one.ctypes.data_as(C.POINTER(C.c_double)),
                               1.0, one.ctypes.data_as(C.POINTER(C.c_double)), 4, 0.05,
                               one.ctypes.data_as(C.POINTER(C.c_double)), dp, None) == -1
    assert b"n_exc" in lib.bse_last_error(None)
    assert lib.bse_eps_noalloc(4, dp, dp, 1.0, dp, 4, 0.05, dp, dp, None) == -1


def test_rejects_out_of_range_inputs(synth, gpu):
    """Empty lists, more than 16 orbitals or 8 bands, unknown enum values, a missing -R partner:
    BSE_ERR_BAD_INPUT before any device work."""
    import dataclasses
    base = synth.hbn_problem(grid=2)
    cases = []
    cases.append((dataclasses.replace(base, k_cart=base.k_cart[:0]), {}, "empty"))
    cases.append((dataclasses.replace(base, g_cart=base.g_cart[:0]), {}, "empty"))
    cases.append((base, {"nv": 9}, None))
    cases.append((base, {"precision": 2}, "precision"))
    cases.append((base, {"eig_solver": 5}, "eig_solver"))
    cases.append((base, {"coulomb_kind": 7}, "coulomb_kind"))
    cases.append((base, {"w_kind": 9}, "w_kind"))
    cases.append((base, {"scissor": float("inf")}, "NaN"))
    for prob, kw, word in cases:
        st, msg = _create(gpu, prob, **kw)
        assert st == -1, (kw, msg)
        if word:
            assert word in msg, (kw, msg)
    # H(R) without its -R partner: drop the first non-zero R
    m = base.model
    drop = next(i for i in range(m.n_r) if np.abs(m.r_cryst[i]).sum() > 0)
    keep = [i for i in range(m.n_r) if i != drop]
    m2 = dataclasses.replace(m, r_cryst=m.r_cryst[keep], weights=m.weights[keep], h_r=m.h_r[:, keep])
    st, msg = _create(gpu, dataclasses.replace(base, model=m2))
    assert st == -1 and "-R" in msg


def test_rpa_validation(synth, gpu):
    """BSE_W_RPA: even rpa_points >= 2, rpa_order 0 or 1, a complete periodic k grid."""
    prob = synth.hbn_problem(grid=3)
    st, msg = _create(gpu, prob, w_kind=3, rpa_points=3)
    assert st == -1 and "rpa_points" in msg
    st, msg = _create(gpu, prob, w_kind=3, rpa_order=2)
    assert st == -1 and "rpa_order" in msg
    st, _ = _create(gpu, prob, w_kind=3, tamm_dancoff=0)
    assert st in (0, -2)
    part = prob.__class__(prob.model, prob.k_cart[:-1], prob.g_cart, prob.params)
    st, msg = _create(gpu, part, w_kind=3)
    assert st in (-1, -2)          # the grid check needs the context: NO_DEVICE here, BAD_INPUT on a GPU
    st, _ = _create(gpu, prob, w_kind=3)
    assert st in (0, -2)
