"""The hand-written adjoint of eps2 against torch autograd of an FP64 reference forward
(CPU) and, on the GPU, against central finite differences of the CUDA forward."""
import numpy as np
import pytest
import torch

OMEGA = np.arange(400) * 8.0 / 400
GAMMA = 0.05


def _setup(synth, grid):
    from bse_gb300.adjoint import ParamModel
    from bse_gb300.synth import MAGNETIC4_NOMINAL
    pm = ParamModel.magnetic4()
    prob = synth.magnetic4_problem(grid=grid)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.0, 1.0, size=len(OMEGA))
    return pm, prob, MAGNETIC4_NOMINAL.copy(), 10.0, w


def _autograd(pm, prob, theta, r0, w):
    from bse_gb300.adjoint import reference_loss
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    rr = torch.tensor(r0, dtype=torch.float64, requires_grad=True)
    L, inter = reference_loss(pm, prob, th, rr, torch.tensor(OMEGA), torch.tensor(w), GAMMA,
                              return_intermediates=True)
    L.backward()
    return float(L.detach()), th.grad.numpy().copy(), float(rr.grad), inter


def test_parameterised_model_is_the_synthetic_model(synth):
    from bse_gb300.adjoint import ParamModel
    from bse_gb300.synth import MAGNETIC4_NOMINAL
    pm = ParamModel.magnetic4()
    m0 = synth.magnetic4_model()
    k = np.random.default_rng(0).normal(size=(5, 3))
    assert np.abs(pm.model(MAGNETIC4_NOMINAL).hk(k) - m0.hk(k)).max() < 1e-12


def test_reference_forward_matches_oracle(synth, oracle):
    from bse_gb300.adjoint import reference_loss
    pm, prob, theta, r0, w = _setup(synth, 4)
    L, eps2 = reference_loss(pm, prob, torch.tensor(theta), torch.tensor(r0, dtype=torch.float64), torch.tensor(OMEGA),
                             torch.tensor(w), GAMMA, return_eps2=True)
    ref = oracle.solve(prob, OMEGA, GAMMA)
    assert np.abs(eps2.numpy() - ref["eps2"]).max() < 1e-10 * np.abs(ref["eps2"]).max()


def test_handwritten_adjoint_matches_autograd_cpu(synth):
    from bse_gb300.adjoint import backward
    pm, prob, theta, r0, w = _setup(synth, 4)
    L, g_th, g_r0, inter = _autograd(pm, prob, theta, r0, w)
    dth, dr0 = backward(pm, prob, inter, OMEGA, w, GAMMA, device=torch.device("cpu"))
    assert np.abs(dth - g_th).max() <= 1e-8 * np.abs(g_th).max()
    assert abs(dr0 - g_r0) <= 1e-8 * abs(g_r0)


def test_autograd_matches_finite_differences_cpu(synth):
    from bse_gb300.adjoint import reference_loss
    pm, prob, theta, r0, w = _setup(synth, 3)
    L, g_th, g_r0, _ = _autograd(pm, prob, theta, r0, w)
    h = 1e-5

    def loss(th, rr):
        return float(reference_loss(pm, prob, torch.tensor(th, dtype=torch.float64),
                                    torch.tensor(rr, dtype=torch.float64), torch.tensor(OMEGA),
                                    torch.tensor(w), GAMMA))

    for p_ in (0, 2, 3, 7):
        e = np.zeros_like(theta)
        e[p_] = h
        fd = (loss(theta + e, r0) - loss(theta - e, r0)) / (2 * h)
        assert abs(fd - g_th[p_]) <= 1e-4 * max(abs(g_th).max(), 1e-12)
    fd = (loss(theta, r0 + h) - loss(theta, r0 - h)) / (2 * h)
    assert abs(fd - g_r0) <= 1e-4 * abs(g_r0)


@pytest.mark.gpu
def test_adjoint_of_cuda_forward_vs_autograd_and_fd(synth):
    from bse_gb300.adjoint import backward, gpu_forward
    pm, prob, theta, r0, w = _setup(synth, 6)
    L, g_th, g_r0, _ = _autograd(pm, prob, theta, r0, w)
    fwd = gpu_forward(pm, prob, theta, r0, OMEGA, GAMMA)
    dth, dr0 = backward(pm, fwd["prob"], fwd, OMEGA, w, GAMMA)
    scale = np.abs(g_th).max()
    assert np.abs(dth - g_th).max() <= 1e-6 * scale
    assert abs(dr0 - g_r0) <= 1e-6 * abs(g_r0)
    h = 1e-5

    def loss(th, rr):
        return float(np.dot(w, gpu_forward(pm, prob, th, rr, OMEGA, GAMMA, want_vectors=False)["eps2"]))

    for p_ in range(pm.n_params):
        e = np.zeros_like(theta)
        e[p_] = h
        fd = (loss(theta + e, r0) - loss(theta - e, r0)) / (2 * h)
        assert abs(fd - dth[p_]) <= 1e-4 * scale
    fd = (loss(theta, r0 + h) - loss(theta, r0 - h)) / (2 * h)
    assert abs(fd - dr0) <= 1e-4 * abs(dr0)


@pytest.mark.gpu
def test_autograd_function_wrapper(synth):
    from bse_gb300.adjoint import EPS2Function
    pm, prob, theta, r0, w = _setup(synth, 6)
    L_ref, g_th, g_r0, _ = _autograd(pm, prob, theta, r0, w)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    rr = torch.tensor(r0, dtype=torch.float64, requires_grad=True)
    eps2 = EPS2Function.apply(th, rr, pm, prob, OMEGA, GAMMA)
    L = torch.sum(torch.tensor(w) * eps2)
    L.backward()
    assert abs(float(L) - L_ref) <= 1e-9 * abs(L_ref)
    assert np.abs(th.grad.numpy() - g_th).max() <= 1e-6 * np.abs(g_th).max()
    assert abs(float(rr.grad) - g_r0) <= 1e-6 * abs(g_r0)


def test_adjoint_rejects_full_bse(synth):
    """The adjoint differentiates the Tamm-Dancoff spectrum; a full-BSE problem is refused
    before any device work."""
    from bse_gb300.adjoint import backward, gpu_forward
    pm, prob, theta, r0, w = _setup(synth, 3)
    full = prob.__class__(model=prob.model, k_cart=prob.k_cart, g_cart=prob.g_cart,
                          params=prob.params.replace(tamm_dancoff=0), k_cryst=prob.k_cryst, grid=prob.grid)
    with pytest.raises(ValueError, match="Tamm-Dancoff"):
        gpu_forward(pm, full, theta, r0, OMEGA, GAMMA)
    with pytest.raises(ValueError, match="Tamm-Dancoff"):
        backward(pm, full, {}, OMEGA, w, GAMMA, device=torch.device("cpu"))
