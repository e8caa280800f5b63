"""torch.autograd.Function over one image update with the NNF held fixed.

    out = image_update(ctx, params, image, lam, sigma, dom, ext, nnf, conf, lam_d=None)

runs the CUDA update (nli_update with orig = image) forward and the
hand-written adjoint kernels (nli_update_backward) backward, giving
gradients with respect to the image, lambda (and lambda_d for NL-depth) and
the patch-weight sigma.  The NNF, masks and confidence are constants.
"""
from __future__ import annotations

import copy

import torch


class ImageUpdate(torch.autograd.Function):
    @staticmethod
    def forward(fctx, image, lam, sigma, lam_d, nli, params, dom, ext, nnf, conf):
        p = copy.copy(params)
        p.lambda_ = float(lam)
        p.sigma = float(sigma)
        if lam_d is not None:
            p.lambda_d = float(lam_d)
        img = image.detach().to(torch.float32).contiguous()
        out, _ = nli.update(p, img, img, dom, ext, nnf, conf, same_orig=False)
        fctx.nli, fctx.p = nli, p
        fctx.masks = (dom, ext, nnf, conf)
        fctx.has_lam_d = lam_d is not None
        fctx.save_for_backward(img, out)
        return out

    @staticmethod
    def backward(fctx, grad_out):
        img, out = fctx.saved_tensors
        dom, ext, nnf, conf = fctx.masks
        gi, dl, dld, ds = fctx.nli.update_backward(fctx.p, img, out, dom, ext, nnf, conf,
                                                   grad_out.to(torch.float32).contiguous())
        as_t = lambda v: torch.tensor(v, dtype=torch.float64)  # noqa: E731
        return (gi, as_t(dl), as_t(ds), as_t(dld) if fctx.has_lam_d else None, None, None, None, None, None, None)


def image_update(nli, params, image, lam, sigma, dom, ext, nnf, conf=None, lam_d=None):
    """One differentiable update step; lam, sigma (and lam_d) may be tensors
    with requires_grad."""
    return ImageUpdate.apply(image, lam, sigma, lam_d, nli, params, dom, ext, nnf, conf)


def replay_updates(nli, params, image, lam, sigma, dom, ext, nnf, conf=None, steps=1, lam_d=None):
    """`steps` update steps from `image` with one checkpointed NNF held fixed
    (for instance a level's final NNF from Context.intermediate(INTER_NNF)),
    each a differentiable image_update: gradients flow back through every
    step to the starting image, lambda and sigma.  The backward pass
    recomputes each step's weights and coefficients from the saved image;
    only the images between steps are kept.  NL-Poisson steps here use the
    step's own input as `orig`; the multiscale driver keeps the level's
    start image there, which gives the same exact solution (the known
    pixels, the only ones the solution reads outside the hole, never
    change)."""
    u = image
    for _ in range(steps):
        u = image_update(nli, params, u, lam, sigma, dom, ext, nnf, conf, lam_d)
    return u
