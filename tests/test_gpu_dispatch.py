"""The build's row tiles on the GPU (bse_build_kernel_rows) and the host-assembled matrix fed back
(bse_set_kernel): the tiles equal the rows of the whole build, and a solve from the assembled
matrix equals the solve from the context's own build (FP64 exactly, mixed within its precision),
for the spin-orbital and the collinear layouts.  Plus the batch dispatcher on one rank against
bse_solve_many."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = np.arange(400) * 8.0 / 400
GAMMA = 0.05


def _dispatch():
    from importlib import import_module
    return import_module("bse_gb300.dispatch")


@pytest.mark.parametrize("name,precision", [("mag6", 0), ("mag6", 1), ("coll4", 0), ("coll4", 1)])
def test_row_tiles_and_set_kernel(synth, gpu, name, precision):
    d = _dispatch()
    prob = {"mag6": lambda: synth.magnetic4_problem(grid=6), "coll4": lambda: synth.collinear_problem(grid=4)}[name]()
    with gpu.BSEContext(prob, precision=precision) as ctx:
        H, _ = ctx.build_kernel(want_h=True)
    parts = []
    for lo, hi in d.ranges(prob.nk, 3):
        with gpu.BSEContext(prob, precision=precision) as ctx:
            rows = ctx.build_kernel_rows(lo, hi)
        assert np.array_equal(rows, H[d.tile_rows(H.shape[0], prob.nk, lo, hi)])
        parts.append((lo, hi, rows))
    Hs = d.assemble_rows(parts, prob.nk, H.shape[0])
    assert np.array_equal(Hs, H)
    with gpu.BSEContext(prob, precision=precision, n_refine=32) as ctx:
        E0, e20, _ = ctx.solve(OMEGA, GAMMA)
    with gpu.BSEContext(prob, precision=precision, n_refine=32) as ctx:
        ctx.set_kernel(Hs)
        E1, _ = ctx.diagonalize()
        ctx.oscillators()
        e21, _ = ctx.eps(OMEGA, GAMMA)
    tol = 1e-12 if precision == 0 else 1e-6
    assert np.abs(E1 - E0).max() <= tol * np.abs(E0).max()
    assert np.linalg.norm(e21 - e20) <= (1e-10 if precision == 0 else 1e-4) * np.linalg.norm(e20)


def test_row_tiles_reject_bad_ranges(synth, gpu):
    prob = synth.hbn_problem(grid=4)
    with gpu.BSEContext(prob) as ctx:
        for lo, hi in ((-1, 2), (3, 3), (0, prob.nk + 1)):
            with pytest.raises(gpu.BSEError):
                ctx.build_kernel_rows(lo, hi)
    with gpu.BSEContext(prob, tamm_dancoff=0) as ctx:
        with pytest.raises(gpu.BSEError):
            ctx.build_kernel_rows(0, 2)


def test_batch_dispatch_one_rank(synth, gpu):
    d = _dispatch()
    probs = [synth.hbn_problem(grid=g) for g in (4, 6, 5)] + [synth.magnetic4_problem(grid=4)]
    e2 = d.solve_batch(probs, OMEGA, GAMMA, 0, 1, precision=1, n_refine=16)
    ctxs = [gpu.BSEContext(p, precision=1, n_refine=16) for p in probs]
    try:
        ref, _ = gpu.solve_many(ctxs, OMEGA, GAMMA)
    finally:
        for c in ctxs:
            c.close()
    assert np.allclose(e2, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
