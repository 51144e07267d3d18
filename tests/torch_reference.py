"""float64 torch restatement of chi2Profile, differentiable by autograd.

Test infrastructure: the reference gradient for the hand-written adjoint
kernels.  Same semantics as the reference's CPU path (sweep_core
src/galario.cpp:1048-1071, central pixel :1136-1153, shifts + R2C FFT
:1310-1312, interpolate_core :749-815, apply_phase_sampled_core :877-884,
chi2 :1519-1529), with floor() treated as piecewise constant.
"""
import math

import torch


def central_pixel_t(I, Rmin, dR, dxy):
    iIN = int(math.floor((dxy / 2 - Rmin) / dR))
    flux = I.new_zeros(())
    for i in range(1, iIN):
        flux = flux + (Rmin + dR * i) * I[i]
    flux = flux * 2.
    flux = flux + Rmin * I[0] + (Rmin + iIN * dR) * I[iIN]
    flux = flux * dR
    I_interp = (I[iIN + 1] - I[iIN]) / dR * (dxy / 2. - (Rmin + dR * iIN)) + I[iIN]
    flux = flux + ((Rmin + iIN * dR) * I[iIN] + dxy / 2. * I_interp) * (dxy / 2. - (Rmin + iIN * dR))
    return dxy * dxy * flux / ((dxy / 2.) ** 2 - Rmin ** 2)


def sweep_t(I, inc, Rmin, dR, nxy, dxy):
    N, nr = nxy, I.shape[0]
    rmax = min(int(math.ceil((Rmin + nr * dR) / dxy)), N // 2)
    off = N // 2 - rmax
    k = torch.arange(2 * rmax, dtype=torch.float64, device=I.device)
    x = (rmax - k) * dxy
    y = (rmax - k) * dxy
    xs = x / torch.cos(inc)
    r2 = xs[None, :] ** 2 + y[:, None] ** 2
    pos = r2 > 0
    r = torch.where(pos, torch.sqrt(torch.where(pos, r2, torch.ones_like(r2))), torch.zeros_like(r2))
    iR = torch.clamp(torch.floor((r.detach() - Rmin) / dR), min=0).long()
    valid = iR <= nr - 2
    iRc = torch.clamp(iR, max=nr - 2)
    frac = (r - iRc.to(torch.float64) * dR - Rmin) / dR
    val = torch.where(valid, I[iRc] + frac * (I[iRc + 1] - I[iRc]), torch.zeros_like(r)) * dxy ** 2
    img = torch.nn.functional.pad(val, (off, N - off - 2 * rmax, off, N - off - 2 * rmax))
    cen = central_pixel_t(I, Rmin, dR, dxy)
    mask = torch.zeros_like(img)
    mask[N // 2, N // 2] = 1.
    return img * (1 - mask) + cen * mask


def sample_image_t(img, dxy, u, v, PA, dRA, dDec, v_origin=1.):
    return sample_image_parts_t(img, dxy, u, v, PA, dRA, dDec, v_origin)[0]


def sample_image_parts_t(img, dxy, u, v, PA, dRA, dDec, v_origin=1.):
    """(V, z, max|S|): the visibilities, the complex bilinear interpolant z
    of each (whose argument gives the phase) and the spectrum's peak modulus."""
    N = img.shape[0]
    S = torch.fft.fftshift(torch.fft.rfft2(torch.fft.fftshift(img)), dim=0)
    c, s = torch.cos(PA), torch.sin(PA)
    ur = u * c - v * s
    vr = u * s + v * c
    duv = 1. / (dxy * N)
    su = torch.where(ur.detach() < 0, -1., 1.).to(torch.float64)
    indu = ur.abs() / duv
    indv = N / 2 + v_origin * su * vr / duv
    fu = torch.floor(indu.detach()).long()
    fv = torch.floor(indv.detach()).long()
    q = indu - fu.to(torch.float64)
    t = indv - fv.to(torch.float64)
    y0, y1, y2, y3 = S[fv, fu], S[fv + 1, fu], S[fv + 1, fu + 1], S[fv, fu + 1]
    w0, w1, w2, w3 = (1 - t) * (1 - q), t * (1 - q), t * q, (1 - t) * q
    z = y0 * w0 + y1 * w1 + y2 * w2 + y3 * w3
    A = y0.abs() * w0 + y1.abs() * w1 + y2.abs() * w2 + y3.abs() * w3
    e = z / z.abs()
    U = A * torch.complex(e.real, su * e.imag)
    dra = dRA * c - dDec * s
    ddec = dRA * s + dDec * c
    phi = 2 * math.pi * (ur * dra + vr * ddec)
    return U * torch.exp(1j * phi), z, S.abs().max()


def chi2_profile_t(I, inc, PA, dRA, dDec, Rmin, dR, nxy, dxy, u, v, re, im, w):
    img = sweep_t(I, inc, Rmin, dR, nxy, dxy)
    V = sample_image_t(img, dxy, u, v, PA, dRA, dDec)
    return torch.sum(w * ((V.real - re) ** 2 + (V.imag - im) ** 2))
