"""Hand-written adjoint of eps2 with respect to tight-binding and screening parameters.

The reference has no derivatives; this is the differentiation extension of its path:
    theta, r0 -> H(R) -> H(k) -> band eigenpairs -> pair densities P -> kernel (V, W(r0))
    -> BSE eigenpairs (E, A) -> oscillators f = A^T conj(rho) -> eps2(w) -> L = sum_s w_s eps2(w_s)
The forward pass is the CUDA library (FP64, own eigensolver) through its C ABI; the backward
pass below is written by hand (torch tensors for the dense algebra, no autograd):

  eps2 level   g(E) = F sum_s w_s gamma / ((w_s - E)^2 + gamma^2),  Ebar_l = |f_l|^2 g'(E_l)
               C'[m,l] = conj(f_l) f_m (g(E_l) - g(E_m)) / (E_l - E_m)  (m != l; the limit g'
               for (near-)degenerate pairs -- the degenerate-safe eigenvector adjoint)
               C'[l,l] = Ebar_l,  K = A C'^T A^H  so that dL = Re tr(K dH)  (Hellmann-Feynman on
               the diagonal), rhobar = 2 A (g o conj(f))
  kernel level exchange H_x = R V R^H: Rbar = (K + K^H) R V;  direct H_d = fw sum_ab P_ab Phi_ab P_ab^H:
               Pbar from two Phi-weighted contractions of K; dL/dr0 from dPhi/dr0 -- the
               pair densities are recomputed from P, never stored
  band level   cbar from Pbar; per-k eigenvector adjoint K_k = sum_n [Ebar_n c_n c_n^H +
               sum_{m != n} c_n (cbar_n^H c_m) / (E_n - E_m) c_m^H]; H(R)bar = sum_k K_k e^{ik.R};
               dL/dtheta_p = Re sum_R w_R tr(Hbar(R) B_p(R))
An FP64 torch reference of the same forward (reference_loss) is differentiated with torch
autograd in the tests, next to central finite differences of the CUDA forward.

Scope: spinless / spin-orbital models (n_spin = 1), Tamm-Dancoff, Rytova-Keldysh W on a k-grid.
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Sequence

import numpy as np
import torch

from .constants import CONV, MINVAL
from .model import BSEParams, Problem, TBModel, reciprocal_vectors

# ---------------------------------------------------------------------------- parameterised model


class ParamModel:
    """H(R; theta) = sum_p theta_p B_p(R) on a fixed R list, plus the screening length r0."""

    def __init__(self, lattice, r_cryst, basis, centres, dim=2, name="param"):
        self.lattice = np.asarray(lattice, dtype=np.float64)
        self.r_cryst = np.asarray(r_cryst, dtype=np.int64)
        self.B = np.asarray(basis, dtype=np.complex128)     # (P, nR, nw, nw)
        self.centres = np.asarray(centres, dtype=np.float64)  # (1, nw, 3)
        self.dim = dim
        self.name = name

    @classmethod
    def magnetic4(cls, seed=1234):
        from .synth import magnetic4_basis
        lat, centres, basis = magnetic4_basis(seed)
        keys = sorted({R for b in basis for R in b}, key=lambda r: (abs(r[0]) + abs(r[1]) + abs(r[2]), r))
        nw = centres.shape[1]
        B = np.zeros((len(basis), len(keys), nw, nw), np.complex128)
        for p, b in enumerate(basis):
            for i, R in enumerate(keys):
                if R in b:
                    B[p, i] = b[R]
        return cls(lat, np.array(keys), B, centres, dim=2, name="magnetic4")

    @property
    def n_params(self):
        return self.B.shape[0]

    def model(self, theta) -> TBModel:
        h = np.einsum("p,prlm->rlm", np.asarray(theta, dtype=np.float64), self.B)[None]
        return TBModel(lattice=self.lattice, r_cryst=self.r_cryst, weights=np.ones(len(self.r_cryst)), h_r=h,
                       centres=self.centres, dim=self.dim, name=self.name)


# ---------------------------------------------------------------------------- shared geometry


def _geometry(lat):
    c12 = np.cross(lat[:, 0], lat[:, 1])
    vol = abs(np.linalg.det(lat))
    area = np.linalg.norm(c12)
    return vol, area, c12 / area, vol / area


def _inplane_norm(x, normal):
    qn = x @ normal
    xp = x - qn[..., None] * normal
    return torch.sqrt(torch.sum(xp * xp, dim=-1))


def phi_tables(prob: Problem, r0, need_grad: bool, device, dtype=torch.float64):
    """Phi_ab(k1,k2) = sum_G W_G(k2-k1) e^{-i(G + k2 - k1).(tau_a - tau_b)} for the Rytova-Keldysh
    W, and dPhi/dr0 (both [k1, k2, a, b]).  Mirrors phi_table_kernel / the oracle's w_diag."""
    p = prob.params
    r0 = torch.as_tensor(r0, device=device).to(dtype)
    vol, area, normal, lz = _geometry(prob.model.lattice)
    nk, ng = prob.nk, prob.ng
    g0 = ng // 2
    K = torch.tensor(prob.k_cart, dtype=dtype, device=device)
    G = torch.tensor(prob.g_cart, dtype=dtype, device=device)
    nrm = torch.tensor(normal, dtype=dtype, device=device)
    tau = torch.tensor(prob.model.centres[0], dtype=dtype, device=device)
    dk = K[None, :, :] - K[:, None, :]                               # [k1,k2] = k2 - k1
    x = dk[:, :, None, :] + G[None, None, :, :]
    a = _inplane_norm(x, nrm)
    C = CONV * lz / 2.0
    eps = p.rk_eps
    with torch.no_grad():
        mask = (a * a >= p.coulomb_min_k2) & (a > 0)
    a_safe = torch.where(mask, a, torch.ones_like(a))
    W = torch.where(mask, C / (a_safe * (eps + r0 * a_safe)), torch.zeros_like(a))
    dW = torch.where(mask, -C / (eps + r0 * a_safe) ** 2, torch.zeros_like(a))
    # Delta k = 0, G = G0: disk average (conv Lz ln(1 + r0 qc/eps) / (r0 qc^2))
    abz = (2 * math.pi) ** 2 / area
    qc = math.sqrt(abz / (math.pi * nk))
    u = r0 * qc / eps
    avg = CONV * lz * torch.log1p(u) / (r0 * qc * qc)
    davg = CONV * lz / (qc * qc) * ((qc / eps) / (1 + u) / r0 - torch.log1p(u) / r0 ** 2)
    zero = torch.linalg.norm(dk, dim=-1) <= MINVAL
    W[:, :, g0] = torch.where(zero, avg * torch.ones_like(W[:, :, g0]), W[:, :, g0])
    dW[:, :, g0] = torch.where(zero, davg * torch.ones_like(dW[:, :, g0]), dW[:, :, g0])
    d = tau[:, None, :] - tau[None, :, :]                            # [a,b,3]
    ph = torch.einsum("xygi,abi->xygab", x, d)
    E = torch.exp(-1j * ph.to(torch.complex128))
    Phi = torch.einsum("xyg,xygab->xyab", W.to(torch.complex128), E)
    dPhi = torch.einsum("xyg,xygab->xyab", dW.to(torch.complex128), E) if need_grad else None
    return Phi, dPhi


def exchange_table(prob: Problem, device):
    """e^{i(G+q).tau_a} [G, a] and fx v(q+G) with G0 removed (2-D bare Coulomb)."""
    p = prob.params
    vol, area, normal, lz = _geometry(prob.model.lattice)
    q = np.asarray(p.q)
    x = prob.g_cart + q
    qn = x @ normal
    xp = x - qn[:, None] * normal
    a = np.sqrt(np.sum(xp * xp, axis=1))
    with np.errstate(divide="ignore"):
        v = np.where(a > 0, CONV * lz / (2 * a), 0.0)
    v[prob.ng // 2] = 0.0
    sf = p.spin_factor if p.spin_factor >= 0 else 2.0
    fx = sf / (prob.nk * vol)
    e = np.exp(1j * (x @ prob.model.centres[0].T))
    return (torch.tensor(e, device=device), torch.tensor(fx * v, dtype=torch.float64, device=device))


# ---------------------------------------------------------------------------- loss pieces


def lorentz_g(E, omega, weights, gamma, F):
    """g(E) = F sum_s w_s gamma / ((w_s - E)^2 + gamma^2) and g'(E)."""
    d = omega[None, :] - E[:, None]
    den = d * d + gamma * gamma
    g = F * torch.sum(weights[None, :] * gamma / den, dim=1)
    gp = F * torch.sum(weights[None, :] * 2.0 * gamma * d / (den * den), dim=1)
    return g, gp


def eps2_from(E, f, omega, gamma, F):
    d = omega[None, :] - E[:, None]
    return F * torch.sum((torch.abs(f) ** 2)[:, None] * gamma / (d * d + gamma * gamma), dim=0)


# ---------------------------------------------------------------------------- torch FP64 reference


def reference_loss(pm: ParamModel, prob_template: Problem, theta, r0, omega, weights, gamma,
                   return_eps2=False, return_intermediates=False):
    """Differentiable FP64 torch forward of the same chain (used with torch.autograd as the
    FP64 reference of the hand-written adjoint).  theta, r0: torch tensors (CPU, float64)."""
    dev = theta.device
    theta = theta.to(torch.float64)
    r0 = torch.as_tensor(r0, device=dev).to(torch.float64)
    p = prob_template.params
    nv, nc = p.nv, p.nc
    B = torch.tensor(pm.B, device=dev)
    HR = torch.einsum("p,prlm->rlm", theta.to(torch.complex128), B)
    Rc = torch.tensor(pm.r_cryst.astype(np.float64) @ pm.lattice.T, device=dev)
    K = torch.tensor(prob_template.k_cart, device=dev)
    q = torch.tensor(np.asarray(p.q), device=dev)

    def hk(kk):
        ph = torch.exp(1j * (kk @ Rc.T))
        return torch.einsum("kr,rlm->klm", ph, HR)

    Ec_all, Vc_all = torch.linalg.eigh(hk(K))
    Ev_all, Vv_all = torch.linalg.eigh(hk(K - q))
    nval = int((Ec_all[0] <= p.fermi_energy).sum())
    ci = torch.arange(nval, nval + nc, device=dev)
    vi = torch.arange(nval - 1, nval - 1 - nv, -1, device=dev)
    Ec = Ec_all[:, ci] + p.scissor
    Ev = Ev_all[:, vi]
    Cc = Vc_all[:, :, ci]                  # [k, a, c]
    Cv = Vv_all[:, :, vi]                  # [k, b, v]
    Pm = torch.einsum("kac,kbv->cvkab", Cc.conj(), Cv)       # [c, v, k, a, b]
    nk = K.shape[0]
    N = nc * nv * nk
    P = Pm.reshape(N, -1)
    nw = Cc.shape[1]
    tau = torch.tensor(pm.centres[0], device=dev)
    qhat = q / torch.linalg.norm(q)
    diagP = torch.diagonal(Pm, dim1=-2, dim2=-1).reshape(N, nw)  # P[r, aa]
    rho0 = 1j * diagP @ (tau @ qhat).to(torch.complex128)
    e_tab, fxv = exchange_table(prob_template, dev)
    R = diagP @ e_tab.T                                           # [r, G]
    H = (R * fxv[None, :]) @ R.conj().T
    vol = abs(np.linalg.det(pm.lattice))
    fw = -1.0 / (vol * nk)
    Phi, _ = phi_tables(prob_template, r0, False, dev)
    Pk = Pm.reshape(nc * nv, nk, nw * nw)
    Phk = Phi.reshape(nk, nk, nw * nw)
    Hd = fw * torch.einsum("xkj,kqj,yqj->xkyq", Pk, Phk, Pk.conj()).reshape(N, N)
    H = H + Hd
    H = H + torch.diag((Ec.T[:, None, :] - Ev.T[None, :, :]).reshape(N).to(torch.complex128))
    E, A = torch.linalg.eigh(H)
    f = A.T @ rho0.conj()
    F = CONV / (vol * nk)
    eps2 = eps2_from(E, f, omega, gamma, F)
    L = torch.sum(weights * eps2)
    if return_intermediates:
        # the same quantities in the layouts of bse_get_bands / bse_diagonalize / bse_oscillators
        d = lambda x: x.detach().cpu().numpy()
        ec = np.stack([d(Ec), d(Ec)])
        ev = np.stack([d(Ev), d(Ev)])
        bands = (ec, ev, np.ascontiguousarray(d(Cc).transpose(0, 2, 1)), np.ascontiguousarray(d(Cv).transpose(0, 2, 1)))
        return L, {"E": d(E), "A": d(A), "f": d(f), "bands": bands, "eps2": d(eps2), "nval": nval,
                   "theta": d(theta), "prob": prob_template}
    return (L, eps2) if return_eps2 else L


# ---------------------------------------------------------------------------- hand-written backward


def _require_tda(prob: Problem):
    """The adjoint differentiates the Tamm-Dancoff spectrum (Hermitian H, one exciton block)."""
    p = prob.params
    if p.tamm_dancoff == 0 and not p.ipa:
        raise ValueError("the eps2 adjoint covers the Tamm-Dancoff BSE only (tamm_dancoff = 1)")


def backward(pm: ParamModel, prob: Problem, fwd: Dict[str, np.ndarray], omega, weights, gamma,
             device=None):
    """dL/dtheta (n_params) and dL/dr0 for L = sum_s weights_s eps2(omega_s), from the forward
    intermediates: E (N), A (N x N), f (N), bands (e_c, e_v, c_c, c_v as from bse_get_bands)."""
    _require_tda(prob)
    dev = device or (torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
    p = prob.params
    nv, nc, nk = p.nv, p.nc, prob.nk
    nw = pm.B.shape[2]
    N = nc * nv * nk
    vol = abs(np.linalg.det(pm.lattice))
    F = CONV / (vol * nk)
    fw = -1.0 / (vol * nk)
    c128 = torch.complex128
    om = torch.as_tensor(omega, dtype=torch.float64, device=dev)
    ws = torch.as_tensor(weights, dtype=torch.float64, device=dev)
    E = torch.as_tensor(fwd["E"], dtype=torch.float64, device=dev)
    Ah = np.asarray(fwd["A"])
    if not Ah.flags.c_contiguous and Ah.T.flags.c_contiguous:
        # column-major eigenvectors (the C ABI's layout, seen as a transposed view): move the
        # contiguous buffer and transpose on the device instead of gathering 16 N^2 bytes on the host
        A = torch.as_tensor(Ah.T, dtype=c128, device=dev).T
    else:
        A = torch.as_tensor(Ah, dtype=c128, device=dev)
    f = torch.as_tensor(fwd["f"], dtype=c128, device=dev)
    # ---- eps2 level ----
    g, gp = lorentz_g(E, om, ws, gamma, F)
    Ebar = torch.abs(f) ** 2 * gp
    dE = E[None, :] - E[:, None]                           # [m, l] = E_l - E_m
    dg = g[None, :] - g[:, None]
    close = torch.abs(dE) < 1e-9
    gmid = 0.5 * (gp[None, :] + gp[:, None])
    ratio = torch.where(close, gmid, dg / torch.where(close, torch.ones_like(dE), dE))
    Cp = f.conj()[None, :] * f[:, None] * ratio.to(c128)  # [m, l]
    Cp.diagonal().copy_(Ebar.to(c128))
    Kmat = A @ Cp.T @ A.conj().T                            # dL = Re tr(K dH)
    rhobar = 2.0 * A @ (g.to(c128) * f.conj())
    del Cp
    # ---- kernel level ----
    ec, ev, cc, cv = [torch.as_tensor(x, device=dev) for x in fwd["bands"]]
    Cc = cc.permute(0, 2, 1)                               # [k, a, c]
    Cv = cv.permute(0, 2, 1)                               # [k, b, v]
    Pm = torch.einsum("kac,kbv->cvkab", Cc.conj(), Cv)    # [c, v, k, a, b]
    P = Pm.reshape(N, nw * nw)
    diagP = torch.diagonal(Pm, dim1=-2, dim2=-1).reshape(N, nw)
    Pbar = torch.zeros_like(P)
    # diagonal energies
    dK = torch.real(torch.diagonal(Kmat)).reshape(nc, nv, nk)
    Ec_bar = dK.sum(dim=1).T                               # [k, c]
    Ev_bar = -dK.sum(dim=0).T                              # [k, v]
    # exchange
    e_tab, fxv = exchange_table(prob, dev)
    R = diagP @ e_tab.T
    Rbar = (Kmat + Kmat.conj().T) @ (R * fxv[None, :])
    Pbar_diag = Rbar @ e_tab.conj()                         # [r, a]
    # dipole (rho(G0) = i sum_a (qhat.tau_a) P[r,aa])
    tau = torch.as_tensor(pm.centres[0], device=dev)
    q = torch.as_tensor(np.asarray(p.q), device=dev)
    qt = (tau @ (q / torch.linalg.norm(q))).to(c128)
    Pbar_diag = Pbar_diag + (-1j) * rhobar[:, None] * qt[None, :]
    idx = torch.arange(nw, device=dev) * (nw + 1)
    Pbar[:, idx] += Pbar_diag
    # direct: Pbar[r1] += fw sum_r2 conj(K[r2,r1]) conj(Phi(k1,k2)) P[r2]; Pbar[r2] += fw sum_r1 K[r2,r1] P[r1] Phi
    r0 = torch.tensor(p.rk_r0, dtype=torch.float64, device=dev)
    Phi, dPhi = phi_tables(prob, r0, True, dev)
    K4 = Kmat.reshape(nc * nv, nk, nc * nv, nk)             # [cv2, k2, cv1, k1]  (rows r2, columns r1)
    Pk = P.reshape(nc * nv, nk, nw * nw)
    Phk = Phi.reshape(nk, nk, nw * nw)                     # [k1, k2, ab]
    dPhk = dPhi.reshape(nk, nk, nw * nw)
    Pb = Pbar.reshape(nc * nv, nk, nw * nw)
    # U1[cv1,k1,k2,ab] = sum_cv2 conj(K4[cv2,k2,cv1,k1]) P[cv2,k2,ab]
    U1 = torch.einsum("yqxk,yqj->xkqj", K4.conj(), Pk)
    Pb += fw * torch.einsum("xkqj,kqj->xkj", U1, Phk.conj())
    # dL/dr0 = fw Re sum K[r2,r1] P[r1,ab] dPhi(k1,k2) conj(P[r2,ab]) = fw Re sum conj(U1) P[r1] dPhi
    dr0 = fw * torch.real(torch.einsum("xkqj,xkj,kqj->", U1.conj(), Pk, dPhk))
    del U1
    U2 = torch.einsum("yqxk,xkj->yqkj", K4, Pk)            # sum_cv1 K[r2,r1] P[r1]
    Pb += fw * torch.einsum("yqkj,kqj->yqj", U2, Phk)
    del U2
    Pbar = Pb.reshape(nc, nv, nk, nw, nw)
    # ---- band level ----
    cc_bar = torch.einsum("cvkab,kbv->kac", Pbar.conj(), Cv)   # cbar_c[k, a, c]
    cv_bar = torch.einsum("cvkab,kac->kbv", Pbar, Cc)          # cbar_v[k, b, v]
    B = torch.as_tensor(pm.B, device=dev)
    Rc = torch.as_tensor(pm.r_cryst.astype(np.float64) @ pm.lattice.T, device=dev)
    Kc = torch.as_tensor(prob.k_cart, device=dev)

    def band_adjoint(kk, C_sel, cbar, Ebar_sel, sel_idx):
        # full eigenpairs of H(k) (phases of the unselected ones drop out)
        HR = torch.einsum("p,prlm->rlm", torch.as_tensor(fwd["theta"], device=dev).to(c128), B)
        Hk = torch.einsum("kr,rlm->klm", torch.exp(1j * (kk @ Rc.T)), HR)
        Eall, Vall = torch.linalg.eigh(Hk)
        Km = torch.zeros_like(Hk)
        for j, n in enumerate(sel_idx):
            cn = C_sel[:, :, j]                                   # [k, a]
            Km += Ebar_sel[:, j, None, None].to(c128) * cn[:, :, None] * cn.conj()[:, None, :]
            for m in range(nw):
                if m == n:
                    continue
                cm = Vall[:, :, m]
                coef = torch.einsum("ka,ka->k", cbar[:, :, j].conj(), cm) / (Eall[:, n] - Eall[:, m]).to(c128)
                Km += coef[:, None, None] * cn[:, :, None] * cm.conj()[:, None, :]
        # dL = Re sum_k tr(Km dH(k)) -> Hbar(R) = sum_k Km e^{ik.R}
        return torch.einsum("klm,kr->rlm", Km, torch.exp(1j * (kk @ Rc.T)))

    nval = int(fwd["nval"])
    sel_c = list(range(nval, nval + nc))
    sel_v = list(range(nval - 1, nval - 1 - nv, -1))
    qv = torch.as_tensor(np.asarray(p.q), device=dev)
    MR = band_adjoint(Kc, Cc, cc_bar, Ec_bar, sel_c) + band_adjoint(Kc - qv, Cv, cv_bar, Ev_bar, sel_v)
    # dL/dtheta_p = Re sum_R tr(MR(R) B_p(R)) (weights 1)
    dtheta = torch.real(torch.einsum("rlm,prml->p", MR, B))
    return dtheta.cpu().numpy(), float(dr0.cpu())


# ---------------------------------------------------------------------------- forward on the GPU


def gpu_forward(pm: ParamModel, prob_template: Problem, theta, r0, omega, gamma, want_vectors=True):
    """FP64 forward through the CUDA library: E, A, f, bands, eps2."""
    from . import gpu
    _require_tda(prob_template)
    prob = Problem(model=pm.model(theta), k_cart=prob_template.k_cart, g_cart=prob_template.g_cart,
                   params=prob_template.params.replace(rk_r0=float(r0)), k_cryst=prob_template.k_cryst,
                   grid=prob_template.grid)
    with gpu.BSEContext(prob, precision=0, eig_solver=0) as ctx:
        ctx.compute_bands()
        bands = ctx.get_bands()
        ctx.build_kernel()
        E, A = ctx.diagonalize(want_vectors=want_vectors)
        f = ctx.oscillators()
        e2, _ = ctx.eps(omega, gamma)
    e_all = np.linalg.eigvalsh(prob.model.hk(prob.k_cart[:1]))[0, 0]
    nval = int((e_all <= prob.params.fermi_energy).sum())
    return {"E": E, "A": A, "f": f, "bands": bands, "eps2": e2, "theta": np.asarray(theta, dtype=np.float64),
            "nval": nval, "prob": prob}


class EPS2Function(torch.autograd.Function):
    """eps2(omega; theta, r0) with the CUDA forward and the hand-written backward.

    forward(theta (P,), r0 ()) -> eps2 (n_omega,).  The backward contracts the incoming
    d/d eps2 vector with the hand-written adjoint (one adjoint per call: L = <grad, eps2>)."""

    @staticmethod
    def forward(ctx, theta, r0, pm, prob_template, omega, gamma):
        fwd = gpu_forward(pm, prob_template, theta.detach().cpu().numpy(), float(r0), omega, gamma)
        ctx.fwd = fwd
        ctx.pm, ctx.prob_template, ctx.omega, ctx.gamma = pm, prob_template, omega, gamma
        return torch.as_tensor(fwd["eps2"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        fwd = ctx.fwd
        dth, dr0 = backward(ctx.pm, fwd["prob"], fwd, ctx.omega, grad.detach().cpu().numpy(), ctx.gamma)
        return (torch.as_tensor(dth, dtype=torch.float64), torch.tensor(dr0, dtype=torch.float64),
                None, None, None, None)
