"""The SVI ELBO and its hand-written adjoint gradient as a
``torch.autograd.Function``.

``SviElbo.apply(var_params, band, model, prior_init, eps)`` returns the
Monte-Carlo ELBO estimate of one SVI step (src/parametric.rs:2262-2393) at
each row of ``var_params`` = [mu, log_sigma]; its backward pass returns the
gradient the SVI kernel computes (``lcf_svi_elbo_grad``: FP32 likelihood and
adjoint through the analytic model gradient, FP64 prior / entropy
bookkeeping), scaled by the incoming gradient.  Both passes run on the GPU
through the C ABI; PyTorch only carries the tensors, so the kernel's gradient
can be compared with autograd-driven checks (finite differences of the FP64
ELBO, ``torch.autograd.grad``) in tests.
"""
from __future__ import annotations

import numpy as np
import torch

from .lib import Context, default_context


class BandArrays:
    """A peak-normalised band as the fitter holds it (BandFitData,
    src/parametric.rs:3014-3025, built at :3581-3632)."""

    def __init__(self, times, flux, flux_err):
        times = np.asarray(times, np.float64)
        flux = np.asarray(flux, np.float64)
        err = np.asarray(flux_err, np.float64)
        peak = float(np.max(flux))
        self.times = np.ascontiguousarray(times)
        self.flux = np.ascontiguousarray(flux / peak)
        self.obs_var = np.ascontiguousarray((err / peak) ** 2 + 1e-10)
        self.is_upper = np.ascontiguousarray(((err > 0) & (flux / err < 3.0)).astype(np.uint8))
        self.upper_flux = np.ascontiguousarray(3.0 * err / peak)

    def args(self):
        return self.times, self.flux, self.obs_var, self.is_upper, self.upper_flux


class SviElbo(torch.autograd.Function):
    """(ELBO, flags) of var_params, with the SVI kernel's adjoint as the
    ELBO's gradient; flags (lcf_svi_elbo_grad's) are not differentiable."""

    @staticmethod
    def forward(ctx, var_params: torch.Tensor, band: BandArrays, model: int, prior_init, eps,
                lcf: Context | None = None):
        lcf = lcf or default_context()
        vp = var_params.detach().to("cpu", torch.float64).numpy()
        elbo, grad, flags = lcf.svi_elbo_grad(model, *band.args(), prior_init, vp, eps)
        ctx.save_for_backward(torch.from_numpy(grad).to(var_params.device, var_params.dtype))
        flags_t = torch.from_numpy(flags).to(var_params.device)
        ctx.mark_non_differentiable(flags_t)
        return torch.from_numpy(elbo).to(var_params.device, var_params.dtype), flags_t

    @staticmethod
    def backward(ctx, g_elbo: torch.Tensor, g_flags):
        (grad,) = ctx.saved_tensors
        return g_elbo.unsqueeze(-1) * grad, None, None, None, None, None


def svi_elbo(var_params: torch.Tensor, band: BandArrays, model: int, prior_init, eps, lcf: Context | None = None):
    """ELBO estimate per row of ``var_params`` (n_points, 2 np), differentiable
    through the SVI kernel's adjoint, and the flags of lcf_svi_elbo_grad."""
    return SviElbo.apply(var_params, band, int(model), prior_init, eps, lcf)
