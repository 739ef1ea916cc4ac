"""``torch.autograd`` binding of the adjoint likelihood gradient.

``LogLikelihood.apply(rows, image_model, data, psf_kernels)`` returns the (B,)
FP64 log-likelihoods of the (B, param_count) parameter rows and, in the
backward pass, ``grad_output[:, None] * d logL / d rows`` from the adjoint
kernel (``lensgb_loglike_grad``), computed together with the forward pass so
the ray grid is traced twice in all (forward image, adjoint), never stored.
This is what ``jax.grad`` through the reference's
``ImageModel.likelihood_data_given_model`` (``image_model.py:163-221``)
provides, for the profiles the adjoint supports (EPL, EPL_MULTIPOLE_M1M3M4,
SIE, NIE, NFW, TNFW, NFW_ELLIPSE_CSE, CONVERGENCE and SHEAR lenses; Sersic
light) and every PSF and numerics option of the image path.  Without a
gradient to compute (``torch.no_grad()`` or rows that do not require one) the
forward likelihood runs alone.
"""

import torch


class LogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rows, image_model, data=None, psf_kernels=None):
        if not ctx.needs_input_grad[0]:
            # no gradient wanted (torch.no_grad(), or rows without requires_grad):
            # the forward likelihood alone, without the adjoint pass
            ctx.save_for_backward(None)
            logl = image_model.likelihood_batch(rows=rows.detach(), data=data,
                                                psf_kernels=psf_kernels)
            return logl.to(rows.device)
        logl, grad = image_model.likelihood_grad_batch(rows=rows.detach(), data=data,
                                                       psf_kernels=psf_kernels)
        ctx.save_for_backward(grad)
        return logl.to(rows.device)

    @staticmethod
    def backward(ctx, grad_output):
        (grad,) = ctx.saved_tensors
        if grad is None:
            return None, None, None, None
        g = grad_output.to(grad.device, grad.dtype)[:, None] * grad
        return g, None, None, None


def log_likelihood(rows, image_model, data=None, psf_kernels=None):
    """Differentiable (B,) logL of parameter rows (a float64 CUDA tensor)."""
    return LogLikelihood.apply(rows, image_model, data, psf_kernels)
