"""Test-only torch binding of the likelihood adjoint, and detector-resolution
recalibration on top of it.

``StripNLL.apply(rho, sigma, rec)`` returns the Poisson list-mode negative
log-likelihood L(rho, sigma) of the events held by ``rec`` (a
``capi.StripReconstruction``); its backward pass returns dL/drho (FP32 image,
from the adjoint kernel) and dL/dsigma (FP64).  The 3-sigma support of every
event is the one of ``rec``'s own sigmas and is held fixed.

``recalibrate_sigma`` alternates MLEM iterations at the current widths (on one
half of the events) with Newton steps on (sigma_z, sigma_dl) of the likelihood
of the other half, computed from the adjoint gradient, and re-derives the
supports at the new widths after every step.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi


class StripNLL(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho: torch.Tensor, sigma: torch.Tensor, rec: "capi.StripReconstruction",
                sens: torch.Tensor | None = None):
        assert rho.is_cuda and rho.dtype == torch.float32 and rho.is_contiguous()
        rec.set_stream(torch.cuda.current_stream().cuda_stream)
        grad = torch.empty_like(rho)
        s = [float(v) for v in sigma.detach().cpu().tolist()]
        loss, gs, _ = rec.nll_grad(s[0], s[1], rho.data_ptr(),
                                   None if sens is None else sens.data_ptr(), grad.data_ptr())
        ctx.save_for_backward(grad, torch.tensor(gs, dtype=torch.float64))
        ctx.sigma_device = sigma.device
        return torch.tensor(loss, dtype=torch.float64, device=rho.device)

    @staticmethod
    def backward(ctx, g):
        grad, gs = ctx.saved_tensors
        g64 = g.detach().to(torch.float64)
        return ((g64.to(grad.device) * grad.to(torch.float64)).to(torch.float32),
                (g64.cpu() * gs).to(ctx.sigma_device), None, None)


def nll(rec, rho_dev: torch.Tensor, sigma):
    """Loss and dL/dsigma at kernel widths sigma (support fixed by rec)."""
    loss, gs, _ = rec.nll_grad(float(sigma[0]), float(sigma[1]), rho_dev.data_ptr())
    return loss, np.array(gs)


def recalibrate_sigma(geom: "capi.Geometry", events: np.ndarray, sigma0, outer: int = 12,
                      mlem_iterations: int = 5, delta: float = 0.05, max_step: float = 2.0,
                      tol: float = 2e-3, device: int = 0, log=None):
    """Estimates (sigma_z, sigma_dl) by maximising the list-mode likelihood.

    The events are split in two halves.  MLEM reconstructs the image from the
    first half at the current widths; the widths are then fitted to the second,
    held-out half with the image fixed (diagonal Newton steps from the adjoint
    gradient, backtracking on the loss).  Fitting the widths to the events the
    image was reconstructed from would reward narrower kernels, because MLEM's
    image sharpens towards those very events.  Returns (sigma, history)."""
    sigma = np.array(sigma0, dtype=np.float64)
    ev_a = np.ascontiguousarray(events[0::2])
    ev_b = np.ascontiguousarray(events[1::2])
    rho = np.ones((geom.n_y, geom.n_z), np.float32)
    history = []
    for k in range(outer):
        g = capi.Geometry(geom.radius, geom.length, geom.n_y, geom.n_z, geom.pixel,
                          float(sigma[0]), float(sigma[1]))
        with capi.StripReconstruction(g, device=device) as rec:
            rec.set_events(ev_a)
            rec.rho = rho
            rec.iterate(mlem_iterations)
            rho = rec.rho
        with capi.StripReconstruction(g, device=device) as held:
            held.set_events(ev_b)
            rho_dev = torch.from_numpy(rho).cuda(device)
            torch.cuda.synchronize(device)
            loss, grad = nll(held, rho_dev, sigma)
            # diagonal Newton step from central differences of the gradient
            hess = np.zeros(2)
            for i in range(2):
                sp, sm = sigma.copy(), sigma.copy()
                sp[i] += delta
                sm[i] -= delta
                hess[i] = (nll(held, rho_dev, sp)[1][i] - nll(held, rho_dev, sm)[1][i]) / (2 * delta)
            step = np.where(hess > 0, -grad / np.where(hess > 0, hess, 1.0),
                            -np.sign(grad) * max_step)
            step = np.clip(step, -max_step, max_step)
            t = 1.0
            for _ in range(6):
                trial = sigma + t * step
                if np.all(trial > 0.5) and nll(held, rho_dev, trial)[0] <= loss:
                    break
                t *= 0.5
            sigma = sigma + t * step
        history.append(dict(iteration=k, loss=loss, sigma=sigma.tolist(), grad=grad.tolist()))
        if log:
            log(history[-1])
        if np.all(np.abs(t * step) < tol):
            break
    return sigma, history
