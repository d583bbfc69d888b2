"""Band structure along a k path on the GPU (Hamiltonian_TB::pull_bands, bse.version13.cpp:823-875).

The path's k points go through the library's batched band kernel (bse_compute_bands on a context
whose k list is the path, with q = 0 so the valence and conduction states share each k), and
come back in the reference's bands-file layout (w90io.write_bands)."""
from __future__ import annotations

import numpy as np

from . import w90io
from .model import Problem


def band_structure(prob: Problem, segments, out_path=None):
    """Selected band energies e_v [2, nk, nv], e_c [2, nk, nc] (spin rows; valence top-down from
    E_F, conduction bottom-up with the scissor) at the points of `segments` ((k0, k1, n) tuples,
    cartesian), computed on the GPU; written to out_path in the reference's layout when given."""
    from . import gpu
    kpts = w90io.band_path_points(segments)
    path_prob = Problem(model=prob.model, k_cart=kpts, g_cart=prob.g_cart,
                        params=prob.params.replace(q=(0.0, 0.0, 0.0), small_momentum=0, ipa=1),
                        k_cryst=None, grid=None)
    with gpu.BSEContext(path_prob) as ctx:
        ctx.compute_bands()
        ec, ev, _, _ = ctx.get_bands()
    if out_path is not None:
        w90io.write_bands(out_path, ev, ec, prob.model.n_spin)
    return ev, ec
