"""Test-only torch binding of the likelihood adjoint, and detector-resolution
recalibration on top of it.

``StripNLL.apply(rho, sigma, rec)`` returns the Poisson list-mode negative
log-likelihood L(rho, sigma) of the events held by ``rec`` (a
``capi.StripReconstruction``); its backward pass returns dL/drho (FP32 image,
from the adjoint kernel) and dL/dsigma (FP64).  The 3-sigma support of every
event is the one of ``rec``'s own sigmas and is held fixed.

``calibrate_sigma`` fits (sigma_z, sigma_dl) to the events of a calibration
source whose activity image is known (a point source at the centre of the field
of view, say): Newton-preconditioned gradient descent on the likelihood, with the
gradient from the adjoint kernel.  ``recalibrate_sigma`` is the blind form: it
alternates MLEM iterations at the current widths (on one half of the events)
with the same steps on the likelihood of the other half.  The blind form is not
identifiable: an image blurred by b under widths s predicts the same events as
the sharp image under widths sqrt(s^2 + b^2), so every width below the true one
has an image that explains the events equally well, and an MLEM image that is
still blurred pulls the fit below the true widths.
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


def _newton_step(held, rho_dev, sigma, delta, max_step, floor=0.5):
    """One diagonal Newton step on the widths with backtracking on the loss.
    Returns (loss at sigma, gradient, accepted step)."""
    loss, grad = nll(held, rho_dev, sigma)
    hess = np.zeros(2)
    for i in range(2):
        sp, sm = sigma.copy(), sigma.copy()
        sp[i] += delta
        sm[i] -= delta
        hess[i] = (nll(held, rho_dev, sp)[1][i] - nll(held, rho_dev, sm)[1][i]) / (2 * delta)
    step = np.where(hess > 0, -grad / np.where(hess > 0, hess, 1.0), -np.sign(grad) * max_step)
    step = np.clip(step, -max_step, max_step)
    t = 1.0
    for _ in range(8):
        trial = sigma + t * step
        if np.all(trial > floor) and nll(held, rho_dev, trial)[0] <= loss:
            break
        t *= 0.5
    else:
        t = 0.0
    return loss, grad, t * step


def calibrate_sigma(geom: "capi.Geometry", events: np.ndarray, source_image: np.ndarray, sigma0,
                    max_steps: int = 20, delta: float = 0.05, max_step: float = 2.0,
                    tol: float = 1e-3, device: int = 0, log=None):
    """Estimates (sigma_z, sigma_dl) from the events of a calibration source with
    a known activity image (float32[n_y, n_z], any scale).

    The likelihood's 3-sigma event supports are those of the widest widths seen
    so far (sigma0 to start with): they are re-derived only when a width grows
    past them, so the loss stays one smooth function of sigma between steps.
    Returns (sigma, history)."""
    sigma = np.array(sigma0, dtype=np.float64)
    support = sigma.copy()
    img = np.ascontiguousarray(source_image, np.float32)
    if img.shape != (geom.n_y, geom.n_z):
        raise ValueError("source image must be float32[n_y, n_z]")
    rho_dev = torch.from_numpy(img * np.float32(len(events) / max(float(img.sum()), 1e-30))).cuda(device)
    torch.cuda.synchronize(device)
    history = []
    held = None
    try:
        for k in range(max_steps):
            if held is None or np.any(sigma > support):
                support = np.maximum(support, sigma)
                if held is not None:
                    held.close()
                held = capi.StripReconstruction(
                    capi.Geometry(geom.radius, geom.length, geom.n_y, geom.n_z, geom.pixel,
                                  float(support[0]), float(support[1])), device=device)
                held.set_events(events)
            loss, grad, step = _newton_step(held, rho_dev, sigma, delta, max_step)
            sigma = sigma + step
            history.append(dict(iteration=k, loss=loss, sigma=sigma.tolist(), grad=grad.tolist()))
            if log:
                log(history[-1])
            if np.all(np.abs(step) < tol):
                break
    finally:
        if held is not None:
            held.close()
    return sigma, history


def recalibrate_sigma(geom: "capi.Geometry", events: np.ndarray, sigma0, outer: int = 12,
                      mlem_iterations: int = 5, delta: float = 0.05, max_step: float = 2.0,
                      tol: float = 2e-3, device: int = 0, log=None):
    """Blind estimate of (sigma_z, sigma_dl) with the image reconstructed at the
    current widths.

    The events are split in two halves.  MLEM reconstructs the image from the
    first half at the current widths; the widths are then fitted to the second,
    held-out half with the image fixed.  Fitting the widths to the events the
    image was reconstructed from would reward narrower kernels, because MLEM's
    image sharpens towards those very events.  The result is biased low by the
    blur left in the MLEM image (see the module docstring).  Returns
    (sigma, history)."""
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
            loss, grad, step = _newton_step(held, rho_dev, sigma, delta, max_step)
            sigma = sigma + step
        history.append(dict(iteration=k, loss=loss, sigma=sigma.tolist(), grad=grad.tolist()))
        if log:
            log(history[-1])
        if np.all(np.abs(step) < tol):
            break
    return sigma, history
