"""torch.autograd.Function over the GPU log-likelihood (binding layer only).

``loglik(model, gamma)`` returns LL(gamma) as a 0-d tensor; its backward multiplies grad_output by the one-pass
adjoint gradient dLL/dgamma computed by the same GPU evaluation (KrigingImpl::compute_ll_grad_theta_vecs and the
Nugget alpha-gradient of Kriging::_logLikelihood in the reference).  The forward always requests the gradient, so
backward costs nothing extra.  ``vecchia_loglik`` does the same for the Vecchia approximation.
"""
from __future__ import annotations

import numpy as np
import torch


class _LogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, gamma, model):
        g = gamma.detach().to("cpu", torch.float64).numpy()
        ll, grad, _ = model.logLikelihoodFun(g, True, False)
        ctx.save_for_backward(torch.as_tensor(np.asarray(grad), dtype=gamma.dtype, device=gamma.device))
        return torch.as_tensor(ll, dtype=gamma.dtype, device=gamma.device)

    @staticmethod
    def backward(ctx, grad_output):
        (grad,) = ctx.saved_tensors
        return grad_output * grad, None


def loglik(model, gamma: torch.Tensor) -> torch.Tensor:
    """Differentiable LL(gamma) of a fitted ``libkriging_gb300.Kriging`` (gamma = theta, or [theta, alpha])."""
    return _LogLikelihood.apply(gamma, model)


class _VecchiaLogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, model):
        t = theta.detach().to("cpu", torch.float64).numpy()
        vll, grad = model.logLikelihoodVecchiaFun(t, True)
        ctx.save_for_backward(torch.as_tensor(np.asarray(grad), dtype=theta.dtype, device=theta.device))
        return torch.as_tensor(vll, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_output):
        (grad,) = ctx.saved_tensors
        return grad_output * grad, None


def vecchia_loglik(model, theta: torch.Tensor) -> torch.Tensor:
    """Differentiable Vecchia log-likelihood VLL(theta) of a model prepared for LLVecchia(m)."""
    return _VecchiaLogLikelihood.apply(theta, model)
