"""Independent numpy evaluation of the BSE kernel in factorised (lattice-sum) form.

Test helper: the CPU oracle keeps the reference's loop nests (stored pair densities,
G-sums per element, bse.version13.cpp:2796-2884); this module evaluates the same matrix
through the factorisation the CUDA kernels use,
  H_d[r1,r2] = -1/(V nk) sum_ab P[r1,(ab)] Phi_ab(k2-k1) conj(P[r2,(ab)])
  H_x[r1,r2] =  sf/(V nk) sum_{G != G0} v_G rho_r1(G) conj(rho_r2(G)),
so agreement checks the algebra that turns the reference's pair-density contractions into
per-Delta-k tables.
"""
import math

import numpy as np

CONV = (1.602176634 * 1000) / 8.8541878176
MINVAL = 1e-5


def _geometry(lat):
    c12 = np.cross(lat[:, 0], lat[:, 1])
    vol = abs(np.linalg.det(lat))
    area = np.linalg.norm(c12)
    return vol, area, c12 / area, vol / area


def _coulomb(p, x, normal, lz):
    if p.coulomb_kind == 0:
        k2 = np.sum(x * x, axis=-1)
        with np.errstate(divide="ignore"):
            v = CONV / (k2 + p.coulomb_radius)
        return np.where(k2 < p.coulomb_min_k2, 0.0, v)
    qn = x @ normal
    xp = x - qn[..., None] * normal
    k2 = np.sum(xp * xp, axis=-1)
    with np.errstate(divide="ignore"):
        v = CONV * lz / (2 * np.sqrt(k2))
    return np.where((k2 < p.coulomb_min_k2) | (k2 == 0), 0.0, v)


def _rk(p, x, normal, lz):
    qn = x @ normal
    xp = x - qn[..., None] * normal
    k2 = np.sum(xp * xp, axis=-1)
    a = np.sqrt(k2)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = CONV * lz / (2 * a * (p.rk_eps + p.rk_r0 * a))
    return np.where((k2 < p.coulomb_min_k2) | (k2 == 0), 0.0, v)


def _cell_avg(p, vol, area, lz, nk):
    if p.w_kind == 1 or p.coulomb_kind == 1:
        abz = (2 * math.pi) ** 2 / area
        qc = math.sqrt(abz / (math.pi * nk))
        if p.w_kind == 1:
            return CONV * lz * math.log(1 + p.rk_r0 * qc / p.rk_eps) / (p.rk_r0 * qc * qc)
        return CONV * lz / qc
    rs = 2 * math.pi * (3 / (4 * math.pi * nk * vol)) ** (1 / 3)
    return CONV * 4 * math.pi * rs * nk * vol / (2 * math.pi) ** 3


def build_factorised(prob, bands):
    ec, ev, cc, cv = bands
    m, p = prob.model, prob.params
    nk, nc, nv, nw, ns, ng = prob.nk, p.nc, p.nv, m.nw, m.n_spin, prob.ng
    S, N = ns - 1, nk * nc * nv
    vol, area, normal, lz = _geometry(m.lattice)
    q = np.asarray(p.q, dtype=float)
    G = prob.g_cart
    K = prob.k_cart
    g0 = ng // 2
    tau = m.centres                                           # (ns, nw, 3)
    # pair densities rho[s, c, v, k, g]
    rho = np.zeros((ns, nc, nv, nk, ng), np.complex128)
    for s in range(ns):
        P = np.conj(cc[:, :, None, s * nw:(s + 1) * nw]) * cv[:, None, :, s * nw:(s + 1) * nw]   # [k,c,v,a]
        ph = np.exp(1j * (G + q) @ tau[s].T)                                                   # [g,a]
        if p.small_momentum:
            ph[g0] = 1j * (tau[s] @ (q / np.linalg.norm(q)))
        rho[s] = np.einsum("kcva,ga->cvkg", P, ph)
    rho_rows = rho.reshape(ns * N, ng)
    NH = (3 * S + 1) * N
    H = np.zeros((NH, NH), np.complex128)
    if not p.ipa:
        sf = p.spin_factor if p.spin_factor >= 0 else 2 - S
        vg = _coulomb(p, G + q, normal, lz)
        vg[g0] = 0.0
        fx = sf / (nk * vol)
        for i in range(S + 1):
            for j in range(S + 1):
                Ri, Rj = rho_rows[i * N:(i + 1) * N], rho_rows[j * N:(j + 1) * N]
                H[i * 3 * N:i * 3 * N + N, j * 3 * N:j * 3 * N + N] += fx * (Ri * vg) @ Rj.conj().T
        # direct
        fw = -1.0 / (vol * nk)
        dk = K[None, :, :] - K[:, None, :]                                  # [k1,k2] = k2 - k1
        ndk = np.linalg.norm(dk, axis=-1)
        x = dk[:, :, None, :] + G[None, None, :, :]                         # [k1,k2,g,3]
        if p.w_kind == 2:
            W = _coulomb(p, x, normal, lz)
        else:
            W = (p.inv_eps * _coulomb(p, x, normal, lz)) if p.w_kind == 0 else _rk(p, x, normal, lz)
            avg = _cell_avg(p, vol, area, lz, nk)
            avg = p.inv_eps * avg if p.w_kind == 0 else avg
            W[:, :, g0] = np.where(ndk > MINVAL, W[:, :, g0], avg)
        exc = [(0, 0), (0, 1), (1, 0), (1, 1)]
        for sp in range(3 * S + 1):
            sv, sc = exc[sp]
            d = tau[sc][:, None, :] - tau[sv][None, :, :]                    # [a,b,3]
            phase = np.exp(-1j * np.einsum("xygi,abi->xygab", x, d))        # [k1,k2,g,a,b]
            Phi = np.einsum("xyg,xygab->xyab", W, phase)
            A1 = np.conj(cc[:, :, None, sc * nw:(sc + 1) * nw, None]) * cv[:, None, :, None, sv * nw:(sv + 1) * nw]
            Hd = fw * np.einsum("xcvab,xyab,yCVab->cvxCVy", A1, Phi, np.conj(A1))
            H[sp * N:(sp + 1) * N, sp * N:(sp + 1) * N] += Hd.reshape(N, N)
    # diagonal
    for i in range(S + 1):
        tr = (ec[i][:, :, None] - ev[i][:, None, :]).transpose(1, 2, 0).reshape(N)   # [c,v,k]
        H[np.arange(N) + i * 3 * N, np.arange(N) + i * 3 * N] += tr
        if S:
            trf = (ec[1 - i][:, :, None] - ev[i][:, None, :]).transpose(1, 2, 0).reshape(N)
            H[np.arange(N) + (i + 1) * N, np.arange(N) + (i + 1) * N] += trf
    if S:
        h = 1 / math.sqrt(2)
        U = np.array([[1, 0, 0, 0], [0, h, h, 0], [0, h, -h, 0], [0, 0, 0, 1]])
        B = H.reshape(4, N, 4, N)
        H = np.einsum("il,lakb,kj->iajb", U, B, U).reshape(NH, NH)
    return H, rho_rows


def coupling_factorised(prob, bands):
    """Coupling block B (NA x NA, NA = N spinless or 4N collinear) of the full BSE in factorised
    form, against the oracle's loops over stored densities (add_coupling_part,
    bse.version13.cpp:2929-3040):
      B_d[sp r1, sp2 r2] = -1/(V nk) sum_ab Q[r1,(ab)] conj(Phi^{sv1 sc1}_ab(k2-k1)) R[r2,(ab)],
          Q[r1,(ab)] = c_v1a(k1)^{sv1} conj(c_c1b(k1))^{sc1},  R[r2,(ab)] = conj(c_c2a(k2))^{sv1} c_v2b(k2)^{sc1},
          Phi^{st}_ab = sum_G W_G e^{-i(G+dk).(tau^s_a - tau^t_b)}, (sv1, sc1) the spins of block sp,
          sp2 = sp for blocks 0 and 3, 3 - sp for the spin-flip blocks;
      B_x[i*3N + r, j*3N + s] = sf/(V nk) sum_ab P_i[r,(aa)] X^{ij}_ab P_j[s,(bb)],
          X^{ij}_ab = sum_{G != G0} v(q+G) e^{i(G+q).(tau^i_a - tau^j_b)};
    collinear models then rotate U B U over the four exciton spin blocks."""
    ec, ev, cc, cv = bands
    m, p = prob.model, prob.params
    nk, nc, nv, nw, ng = prob.nk, p.nc, p.nv, m.nw, prob.ng
    ns = m.n_spin
    S = ns - 1
    N = nk * nc * nv
    NA = (3 * S + 1) * N
    vol, area, normal, lz = _geometry(m.lattice)
    q = np.asarray(p.q, dtype=float)
    G = prob.g_cart
    K = prob.k_cart
    g0 = ng // 2
    tau = m.centres                                                        # (ns, nw, 3)
    blk = lambda x, s: x[..., s * nw:(s + 1) * nw]
    B = np.zeros((NA, NA), np.complex128)
    # exchange
    sf = p.spin_factor if p.spin_factor >= 0 else 2 - S
    vg = _coulomb(p, G + q, normal, lz)
    vg[g0] = 0.0
    Pd = [np.einsum("kca,kva->cvka", np.conj(blk(cc, s)), blk(cv, s)).reshape(N, nw) for s in range(ns)]
    for i in range(ns):
        for j in range(ns):
            d = tau[i][:, None, :] - tau[j][None, :, :]
            X = np.einsum("g,gab->ab", vg, np.exp(1j * np.einsum("gi,abi->gab", G + q, d)))
            B[i * 3 * N:i * 3 * N + N, j * 3 * N:j * 3 * N + N] += sf / (nk * vol) * (Pd[i] @ X @ Pd[j].T)
    # direct
    fw = -1.0 / (vol * nk)
    dk = K[None, :, :] - K[:, None, :]
    ndk = np.linalg.norm(dk, axis=-1)
    x = dk[:, :, None, :] + G[None, None, :, :]
    if p.w_kind == 2:
        W = _coulomb(p, x, normal, lz)
    else:
        W = (p.inv_eps * _coulomb(p, x, normal, lz)) if p.w_kind == 0 else _rk(p, x, normal, lz)
        avg = _cell_avg(p, vol, area, lz, nk)
        avg = p.inv_eps * avg if p.w_kind == 0 else avg
        W[:, :, g0] = np.where(ndk > MINVAL, W[:, :, g0], avg)
    exc = [(0, 0), (0, 1), (1, 0), (1, 1)]
    for sp in range(3 * S + 1):
        sv1, sc1 = exc[sp]
        sp2 = sp if sp in (0, 3 * S) else 3 - sp
        d = tau[sv1][:, None, :] - tau[sc1][None, :, :]
        Phi = np.einsum("xyg,xygab->xyab", W, np.exp(-1j * np.einsum("xygi,abi->xygab", x, d)))
        Q = blk(cv, sv1)[:, None, :, :, None] * np.conj(blk(cc, sc1))[:, :, None, None, :]   # [k,c1,v1,a,b]
        R = np.conj(blk(cc, sv1))[:, :, None, :, None] * blk(cv, sc1)[:, None, :, None, :]   # [k,c2,v2,a,b]
        Bd = fw * np.einsum("xcvab,xyab,yCVab->cvxCVy", Q, np.conj(Phi), R)
        B[sp * N:(sp + 1) * N, sp2 * N:(sp2 + 1) * N] += Bd.reshape(N, N)
    if S:
        h = 1 / math.sqrt(2)
        U = np.array([[1, 0, 0, 0], [0, h, h, 0], [0, h, -h, 0], [0, 0, 0, 1]])
        B = np.einsum("il,lakb,kj->iajb", U, B.reshape(4, N, 4, N), U).reshape(NA, NA)
    return B
