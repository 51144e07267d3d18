"""Conditioning of the chi2 gradient, for the accuracy tests of the batched
FP32 gradient (test infrastructure).

For a parameter theta_j, d chi2 / d theta_j = sum_k t_jk with one term per
visibility,

    t_jk = 2 w_k Re(conj(V_k - obs_k) dV_k/dtheta_j).

The float64 torch restatement of chi2Profile (torch_reference.py) gives V and,
by forward-mode differentiation, every dV_k/dtheta_j, hence the terms, the
reference gradient sum_k t_jk and the condition number of that sum,

    kappa_j = sum_k |t_jk| / |sum_k t_jk|.

A computation whose terms each carry a relative error e has an error of at
most e * kappa_j relative to the gradient, however the sum is ordered; FP32
terms carry e of a few units of 2^-24, so kappa_j says how many digits an FP32
bulk can keep for component j.  Near a fit's optimum the residuals are noise,
the terms cancel and kappa_j grows like the square root of the number of
visibilities.

The parameters are those of a Gaussian ring profile model: theta = (r0
[arcsec], sigma [arcsec], flux [Jy], inc, PA, dRA, dDec [rad]), the profile
I(R) = flux g(R) / (2 pi dR sum_i g(R_i) R_i), g = exp(-(R - r0)^2 / (2 sigma^2)),
in Jy/sr.
"""
import math

import numpy as np
import torch

from torch_reference import sample_image_parts_t, sweep_t

ARCSEC = 4.84813681109536e-06
NAMES = ("r0", "sigma", "flux", "inc", "PA", "dRA", "dDec")


def ring_profile_t(theta, R, dR):
    """Jy/sr samples of the ring model at the radii R (float64 tensors)."""
    r0, sig, flux = theta[0] * ARCSEC, theta[1] * ARCSEC, theta[2]
    g = torch.exp(-0.5 * ((R - r0) / sig) ** 2)
    return flux * g / (2 * math.pi * dR * torch.sum(g * R))


def model_inputs_t(theta, R, dR):
    """(profile, params) of theta as float32-rounded values in float64 tensors;
    the rounding is a constant offset (straight-through), so derivatives are
    those of the float64 model taken at the rounded point."""
    I = ring_profile_t(theta, R, dR)
    p = theta[3:7]
    I = I + (I.float().double() - I).detach()
    p = p + (p.float().double() - p).detach()
    return I, p


def vis_parts_t(theta, geo, u, v):
    I, p = model_inputs_t(theta, geo["R"], geo["dR"])
    img = sweep_t(I, p[0], geo["Rmin"], geo["dR"], geo["nxy"], geo["dxy"])
    return sample_image_parts_t(img, geo["dxy"], u, v, p[1], p[2], p[3])


def vis_t(theta, geo, u, v):
    """Model visibilities of theta (float64, torch reference semantics)."""
    return vis_parts_t(theta, geo, u, v)[0]


# Sign ambiguity.  A swept profile's spectrum is real, and the reference's
# visibility is then V = A sign(z) e^{i phi} (A the bilinear modulus, z the
# bilinear value of the cell's corners): a step in z at z = 0.  Where |z| is
# within the rounding of an FP32 spectrum (a few 1e-7 of its peak) an FP32
# evaluation cannot know the sign; about one visibility in 1e7 falls there
# near a fit's optimum.  Flipping the sign of V_k moves chi2 by
# 4 w_k |Re(V_k conj(obs_k))| and the gradient term t_jk by at most 2 |t_jk|;
# the tests allow these amounts, taken from the float64 reference at the
# visibilities with |z| < AMBIGUOUS * max|S|, beside the rounding bounds.
AMBIGUOUS = 1e-6


def reference_gradient(theta, geo, u, v, re, im, w):
    """float64 reference of one model (every tensor on one device):
    chi2, gradient (7,), kappa (7,), sum_k |t_jk| (7,), and the sign-ambiguity
    allowances of chi2 (scalar) and of the gradient (7,)."""
    theta = theta.detach().clone()
    V, z, smax = vis_parts_t(theta, geo, u, v)
    rr, ri = V.real - re, V.imag - im
    chi2 = float(torch.sum(w * (rr * rr + ri * ri)))
    amb = torch.abs(z) < AMBIGUOUS * smax
    amb_chi2 = float(torch.sum((4 * w * torch.abs(V.real * re + V.imag * im))[amb]))
    grad, kappa, absum, amb_grad = np.zeros(7), np.zeros(7), np.zeros(7), np.zeros(7)
    for j in range(7):
        e = torch.zeros_like(theta)
        e[j] = 1.0
        _, J = torch.func.jvp(lambda th: vis_t(th, geo, u, v), (theta,), (e,))
        t = 2 * w * (rr * J.real + ri * J.imag)
        s = float(torch.sum(t))
        a = float(torch.sum(torch.abs(t)))
        grad[j], absum[j] = s, a
        kappa[j] = a / abs(s) if s != 0 else math.inf
        amb_grad[j] = 2 * float(torch.sum(torch.abs(t)[amb]))
    return chi2, grad, kappa, absum, amb_chi2, amb_grad


def gpu_gradient(thetas, geo, ds):
    """chi2 (B,) and d chi2 / d theta (B, 7) of B ring models through the
    batched FP32 path and its autograd Function."""
    from galario_gb300.autograd import chi2_profile
    th = thetas.detach().clone().cuda().requires_grad_(True)
    R = geo["R"].cuda()
    I = torch.stack([ring_profile_t(th[b], R, geo["dR"]) for b in range(th.shape[0])])
    chi2 = chi2_profile(I.float(), th[:, 3:7].float(), ds, geo["Rmin"], geo["dR"], geo["dxy"], geo["nxy"])
    chi2.sum().backward()
    return chi2.detach().cpu().numpy(), th.grad.cpu().numpy()
