"""The tensor-core (tcgen05 + TMA, FP32 operands split into three BF16 parts) products of the
two-stage reduction, each on its own against an FP64 numpy evaluation of the same complex64
inputs:

  hemm    Y = A^H V                      (A m x m, V m x kk; A^H = A in the reduction)
  update  A -= V W^H + W V^H             (in place)

at square and ragged orders, full and partial panels (kk < 32), and an even leading dimension
larger than m.  The error of every element is bounded relative to its own condition scale
sum_j |a||v| (the split products carry about 2^-27 relative error, the FP32 accumulation of up to
6 * 2m / 16 partial sums a few 2^-24), plus one FP32 rounding of the stored A for the update.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib(gpu):
    L = gpu.load()
    L.bse_test_tc_hemm.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    L.bse_test_tc_rank2k.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    return L


def _rand(rng, *shape):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)


def _store(A, lda):
    """Column-major complex64 buffer with leading dimension lda holding A (m x m)."""
    m = A.shape[0]
    buf = np.zeros((m, lda), np.complex64)   # row c of buf = column c of A
    buf[:, :m] = A.T
    return buf


@pytest.mark.parametrize("m,kk,pad", [(128, 32, 0), (70, 32, 2), (300, 7, 4), (2048, 32, 0), (1000, 32, 6)])
def test_tc_hemm_matches_fp64(gpu, m, kk, pad):
    L = _lib(gpu)
    rng = np.random.default_rng(m + kk)
    A = _rand(rng, m, m)
    V = _rand(rng, m, kk)
    lda = m + pad
    Abuf = _store(A, lda)
    Vbuf = np.ascontiguousarray(V.T)           # column-major m x kk
    Y = np.zeros((kk, m), np.complex64)
    st = L.bse_test_tc_hemm(m, kk, Abuf.ctypes.data, lda, Vbuf.ctypes.data, Y.ctypes.data)
    assert st == 0, st
    A64, V64 = A.astype(np.complex128), V.astype(np.complex128)
    ref = A64.conj().T @ V64
    scale = np.abs(A64).T @ np.abs(V64)
    err = np.abs(Y.T - ref) / scale
    assert err.max() < 1e-6, err.max()


@pytest.mark.parametrize("m,kk,pad", [(128, 32, 0), (70, 32, 2), (300, 5, 4), (1000, 32, 0), (514, 31, 2)])
def test_tc_update_matches_fp64(gpu, m, kk, pad):
    L = _lib(gpu)
    rng = np.random.default_rng(10 * m + kk)
    A = _rand(rng, m, m)
    V = _rand(rng, m, kk)
    W = _rand(rng, m, kk)
    lda = m + pad + (m + pad) % 2
    Abuf = _store(A, lda)
    Vbuf = np.ascontiguousarray(V.T)
    Wbuf = np.ascontiguousarray(W.T)
    st = L.bse_test_tc_rank2k(m, kk, Abuf.ctypes.data, lda, Vbuf.ctypes.data, Wbuf.ctypes.data)
    assert st == 0, st
    got = Abuf[:, :m].T.astype(np.complex128)
    A64, V64, W64 = (x.astype(np.complex128) for x in (A, V, W))
    ref = A64 - V64 @ W64.conj().T - W64 @ V64.conj().T
    scale = np.abs(V64) @ np.abs(W64).T + np.abs(W64) @ np.abs(V64).T
    err = np.abs(got - ref) / (scale + np.abs(ref))
    assert err.max() < 1e-6, err.max()
    # the padding rows of every column are left as they were
    assert not np.any(Abuf[:, m:])


def test_tc_rejects_odd_sizes(gpu):
    """The TMA tiles need whole 16-byte granules of the 2m-real columns: odd orders and odd leading
    dimensions are refused before any device work (the reduction's orders are all even)."""
    L = _lib(gpu)
    A = np.zeros((10, 10), np.complex64)
    V = np.zeros((10, 2), np.complex64)
    assert L.bse_test_tc_hemm(8, 2, A.ctypes.data, 9, V.ctypes.data, V.ctypes.data) != 0
    assert L.bse_test_tc_hemm(9, 2, A.ctypes.data, 10, V.ctypes.data, V.ctypes.data) != 0
    assert L.bse_test_tc_rank2k(9, 2, A.ctypes.data, 10, V.ctypes.data, V.ctypes.data) != 0


@pytest.mark.parametrize("m", [512, 2048, 4096])
def test_tc_hemm_no_accumulation_bias(gpu, m):
    """All-positive operands (no cancellation): the tensor pipe's FP32 accumulation truncates, so
    one long accumulation chain per output drifts low (about -2.3e-6 relative after K = 4096,
    growing with K); the kernel's chains of K = 128, added in FP32 registers, bound the drift to a
    few units of 2^-24 whatever K."""
    L = _lib(gpu)
    rng = np.random.default_rng(m)
    A = rng.uniform(0, 1, (m, m)).astype(np.complex64)
    V = rng.uniform(0, 1, (m, 32)).astype(np.complex64)
    Y = np.zeros((32, m), np.complex64)
    Abuf = np.ascontiguousarray(A.T)           # kept alive across the call: ctypes takes a raw address
    Vbuf = np.ascontiguousarray(V.T)
    st = L.bse_test_tc_hemm(m, 32, Abuf.ctypes.data, m, Vbuf.ctypes.data, Y.ctypes.data)
    assert st == 0, st
    ref = (A.astype(np.complex128).conj().T @ V.astype(np.complex128)).real
    rel = (Y.T.real - ref) / ref
    assert abs(rel.mean()) < 5e-7, rel.mean()
    assert np.abs(rel).max() < 1e-6, np.abs(rel).max()


@pytest.mark.parametrize("tc", ["both", "hemm", "update", "cublas"])
def test_two_stage_with_tensor_core_products(synth, oracle, gpu, monkeypatch, tc):
    """The two-stage reduction with its trailing-update products on the tensor cores (the
    default; BSE_TC selects both or one of them) or on cuBLAS (BSE_BAND_UPDATE=cublas), mixed
    precision, orb8 12x12 (N_BSE = 2304): every eigenvalue within the FP32 class 1e-6 * ||H||_2
    of the FP64 oracle, the refined lowest 64 within 1e-6 eV, eps2 within 1e-4."""
    monkeypatch.setenv("BSE_TRIDIAG_MODE", "twostage")
    if tc == "cublas":
        monkeypatch.setenv("BSE_BAND_UPDATE", "cublas")
    else:
        monkeypatch.setenv("BSE_BAND_UPDATE", "tc")
        monkeypatch.setenv("BSE_TC", tc)
    omega = np.arange(2000) * 8.0 / 2000
    prob = synth.orb8_problem(grid=12)
    ref = oracle.solve(prob, omega, 0.05)
    with gpu.BSEContext(prob, precision=1, n_refine=64) as ctx:
        E, e2, _ = ctx.solve(omega, 0.05)
    assert np.abs(E[:64] - ref["E"][:64]).max() < 1e-6
    assert np.abs(E - ref["E"]).max() < 1e-6 * np.abs(ref["E"]).max()
    assert np.linalg.norm(e2 - ref["eps2"]) < 1e-4 * np.linalg.norm(ref["eps2"])
