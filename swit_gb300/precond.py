"""Gradient preconditioning of SWIT on device (torch, float64), equal to the
reference's numpy/scipy code:

    grad_precond(grad, forw, back, ...)   toolbox/postprocess.py:20-85
    grad_taper(nx, nz, ...)               toolbox/postprocess.py:88-111
    smooth2d(Z, span)                     toolbox/tools.py:255-275 (Gaussian kernel of gauss2, 237-252)

Arrays are (nx, nz) like the reference's; vectors of length nx*nz are reshaped.
The figure the reference draws of the illuminations is not reproduced.
"""
import math

import torch


def _gauss_1d(span, dtype, device):
    """One factor of the kernel of tools.py:255-269: exp(-x^2 / (2 span^2)) on
    x = linspace(-2 span, 2 span, 2 span + 1), normalised to sum 1.  The 2-D kernel
    exp(-0.5 (X^2 + Y^2) / span^2) / (2 pi span^2), normalised to sum 1, is the outer
    product of two of these (the constant cancels in the normalisation)."""
    x = torch.linspace(-2.0 * span, 2.0 * span, 2 * span + 1, dtype=torch.float64, device=device)
    a = torch.exp(-0.5 * x ** 2 / float(span) ** 2)
    return (a / a.sum()).to(dtype)


def _conv_axis(Z, k):
    """Zero-filled 'same' convolution of every row of Z (m, n) with the
    symmetric odd-length k: one (2r+1)-tap stencil pass, O(m n r) work and no
    n x n operator."""
    r = k.numel() // 2
    out = torch.nn.functional.conv1d(Z.reshape(Z.shape[0], 1, Z.shape[1]), k.reshape(1, 1, -1), padding=r)
    return out.reshape(Z.shape)


def _conv_same(Z, k):
    """scipy.signal.convolve2d(Z, outer(k, k), 'same') with zero fill, as two
    separable passes (along z, then along x)."""
    Z = _conv_axis(Z.contiguous(), k)
    return _conv_axis(Z.t().contiguous(), k).t()


def smooth2d(Z, span=10):
    """tools.py:255-275: Gaussian smoothing, normalised by the smoothed ones array."""
    Z = torch.as_tensor(Z, dtype=torch.float64)
    k = _gauss_1d(int(span), Z.dtype, Z.device)
    num = _conv_same(Z, k)
    den = _conv_same(torch.ones_like(Z), k)
    return num / den


def _hamming(M, dtype, device):
    n = torch.arange(M, dtype=torch.float64, device=device)
    return (0.54 - 0.46 * torch.cos(2.0 * math.pi * n / (M - 1))).to(dtype)


def grad_taper(nx, nz, tapersize=20, thred=0.05, marine_or_land="Marine", device="cpu"):
    """postprocess.py:88-111 (the Marine/Offshore test is case-sensitive, as there)."""
    if marine_or_land in ["Marine", "Offshore"]:
        taper = torch.ones((nx, nz), dtype=torch.float64, device=device)
        taper[:, :tapersize] = 0.0
        return taper
    H = _hamming(tapersize * 2, torch.float64, device)[tapersize:]
    taper = torch.zeros((nx, nz), dtype=torch.float64, device=device)
    taper[:, :tapersize] = H
    taper = smooth2d(taper, span=tapersize // 2)
    taper = taper / taper.max()
    taper = taper * (1 - thred)
    taper = -taper + 1
    return taper * taper


def grad_precond(grad, forw, back, nx, nz, vpmax, marine_or_land, grad_mute, grad_thred, grad_smooth,
                 grad_mask=None):
    """postprocess.py:20-85: taper, illumination (pseudo-Hessian) preconditioning,
    optional smoothing and mask, scaling to vpmax / max|g|.  Returns a vector of nx*nz."""
    dev = grad.device if torch.is_tensor(grad) else "cpu"
    grad = torch.as_tensor(grad, dtype=torch.float64, device=dev).reshape(nx, nz).clone()
    forw = torch.as_tensor(forw, dtype=torch.float64, device=dev).reshape(nx, nz)
    back = torch.as_tensor(back, dtype=torch.float64, device=dev).reshape(nx, nz)
    if grad_mute > 0:
        grad = grad * grad_taper(nx, nz, tapersize=grad_mute, thred=grad_thred, marine_or_land=marine_or_land,
                                 device=dev)
    span = 40 if min(nx, nz) > 40 else int(min(nx, nz) / 2)
    forw = smooth2d(forw, span)
    back = smooth2d(back, span)
    epsilon = 0.0001
    forw = forw / forw.max()
    back = back / back.max()
    precond = forw + back
    precond = precond / precond.max()
    precond = torch.where(precond < epsilon, torch.full_like(precond, epsilon), precond)
    grad = grad / precond
    if grad_smooth > 0:
        if marine_or_land in ["Marine", "Offshore"]:
            grad[:, grad_mute:] = smooth2d(grad[:, grad_mute:], span=grad_smooth)
        else:
            grad = smooth2d(grad, span=grad_smooth)
    if grad_mask is not None:
        mask = torch.as_tensor(grad_mask, dtype=torch.float64, device=dev)
        if tuple(mask.shape) != (nx, nz):
            raise ValueError("Wrong size of grad mask: the size of the mask should be identical to the size of vp model")
        grad = grad * mask
    grad = grad * (vpmax / grad.abs().max())
    return grad.reshape(nx * nz)
