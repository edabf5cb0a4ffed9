"""torch.autograd.Function over the GPU log-likelihood: backward equals the adjoint gradient (times grad_output)
and matches central finite differences of the forward."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autograd_backward_is_adjoint_gradient(gpu_lib):
    import torch
    from libkriging_gb300.autograd import loglik
    rng = np.random.default_rng(3)
    X = rng.uniform(size=(150, 3))
    y = np.sin(2 * np.pi * X).sum(axis=1)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.full((1, 3), 0.5)})
    th = torch.tensor([0.4, 0.5, 0.6], dtype=torch.float64, requires_grad=True)
    ll = loglik(k, th)
    (2.5 * ll).backward()
    _, g, _ = k.logLikelihoodFun(th.detach().numpy(), True)
    assert np.allclose(th.grad.numpy(), 2.5 * g, rtol=1e-14, atol=0)
    h = 1e-4
    for j in range(3):
        e = np.zeros(3)
        e[j] = h * th[j].item()
        fd = (k.logLikelihoodFun(th.detach().numpy() + e)[0] - k.logLikelihoodFun(th.detach().numpy() - e)[0]) / (2 * e[j])
        assert abs(g[j] - fd) < 1e-5 * max(1.0, abs(fd))
