"""Seeded input generators and numpy restatements used by the tests.

They restate, in this project's own code, the semantics of the reference's
test helpers (python/utils.py of galario 1.2.2), which no longer import with
numpy 2 / scipy 1.18: create_reference_image (utils.py:324-348),
create_sampling_points (:351-364), radial_profile (:161-172),
generate_random_vis (:460-469), matrix_size (:407-423), uv_idx/uv_idx_r2c
(:367-387), int_bilin_MT (:390-404), apply_phase_array (:427-457),
apply_rotation (:472-485), central_pixel (:175-206), sweep_ref (:245-321).
"""
from __future__ import annotations

import numpy as np

arcsec = 4.84813681109536e-06
deg = 0.017453292519943295

# parameter sets of the reference tests (python/test_galario.py:43-46)
par1 = {'dRA': 0., 'dDec': 0.4, 'PA': 2., 'nxy': 1024}
par2 = {'dRA': -3.5, 'dDec': 7.2, 'PA': -23., 'nxy': 2048}
par3 = {'dRA': 2.3, 'dDec': 3.2, 'PA': 88., 'nxy': 4096}
par4 = {'dRA': 0., 'dDec': 0., 'PA': 145., 'nxy': 1024}


def reference_image(size, x0=10., y0=-3., sigma_x=50., sigma_y=30., dtype='float64'):
    """Elliptical Gaussian in pixel units with the reference's axis orientation."""
    x = (np.arange(size, dtype=float) - size / 2.)
    xx, yy = np.meshgrid(-x, -x)
    return np.exp(-(xx - x0) ** 2. / sigma_x - (yy - y0) ** 2. / sigma_y).astype(dtype)


def sampling_points(nsamples, maxuv=1., dtype='float64', seed=42):
    """Uniform radius in [maxuv/100, maxuv] and uniform angle."""
    rng = np.random.RandomState(seed)
    uvdist = rng.uniform(low=maxuv / 100., high=maxuv, size=nsamples)
    phi = rng.uniform(low=0., high=2. * np.pi, size=nsamples)
    return (uvdist * np.cos(phi)).astype(dtype), (uvdist * np.sin(phi)).astype(dtype)


def radial_profile(Rmin, dR, nrad, mode='Gauss', dtype='float64', gauss_width=100.):
    R = np.linspace(Rmin, Rmin + dR * (nrad - 1), nrad).astype(dtype)
    if mode == 'Gauss':
        return np.exp(-(R / gauss_width) ** 2)
    return np.cos(2. * np.pi * R / gauss_width) ** 2. * np.exp(-(R / gauss_width) ** 2)


def random_vis(nsamples, dtype, seed=7):
    rng = np.random.RandomState(seed)
    x = 3. * rng.uniform(0., 1., nsamples).astype(dtype) + 2.8 + 1j * rng.uniform(0., 1., nsamples).astype(dtype) + 8.2
    y = 8. * rng.uniform(0.5, 3., nsamples).astype(dtype) + 5.7 + 1j * rng.uniform(0., 6., nsamples).astype(dtype) + 21.2
    w = rng.uniform(0., 1e4, nsamples).astype(dtype)
    w /= w.sum()
    return x, y, w


def matrix_size(u, v, maxuv_factor=4.8, minuv_factor=4.):
    uvdist = np.sqrt(u ** 2 + v ** 2)
    maxuv = uvdist.max() * maxuv_factor
    minuv = uvdist.min() / minuv_factor
    n = int(2 ** np.ceil(np.log2(np.uint(maxuv / minuv))))
    return n, minuv, maxuv


def uv_idx_r2c(u, v, du, half):
    indu = np.abs(u) / du
    indv = half + v / du
    neg = u < 0.
    indv[neg] = half - v[neg] / du
    return indu, indv


def bilinear(f, x, y):
    """Bilinear interpolation of the 2D array f at pixel coordinates (x: column, y: row)."""
    fx, fy = np.floor(x).astype(int), np.floor(y).astype(int)
    t, q = y - fy, x - fx
    y0, y1, y2, y3 = f[fy, fx], f[fy + 1, fx], f[fy + 1, fx + 1], f[fy, fx + 1]
    return t * q * (y0 - y1 + y2 - y3) + t * (y1 - y0) + q * (y3 - y0) + y0


def apply_phase_array(u, v, vis, x0, y0):
    theta = u * (2. * np.pi * x0) + v * (2. * np.pi * y0)
    return vis * (np.cos(theta) + 1j * np.sin(theta))


def apply_rotation(PA, dRA, dDec, u, v):
    c, s = np.cos(PA), np.sin(PA)
    return dRA * c - dDec * s, dRA * s + dDec * c, u * c - v * s, u * s + v * c


def py_sample_image(image, dxy, u, v, dRA=0., dDec=0., PA=0., origin='upper'):
    """numpy restatement of sampleImage (semantics of utils.py:38-99): rfft2 of the
    fftshifted image, half-plane bilinear amp/phase interpolation, phase shift."""
    v_origin = 1. if origin == 'upper' else -1.
    nxy = image.shape[0]
    du = 1. / (nxy * dxy)
    ft = np.fft.fftshift(np.fft.rfft2(np.fft.fftshift(image)), axes=0)
    dRArot, dDecrot, ur, vr = apply_rotation(PA, dRA, dDec, u, v)
    indu = np.abs(ur) / du
    indv = nxy / 2. + v_origin * vr / du
    neg = ur < 0.
    indv[neg] = nxy / 2. - v_origin * vr[neg] / du
    re = bilinear(ft.real, indu, indv)
    im = bilinear(ft.imag, indu, indv)
    amp = bilinear(np.abs(ft), indu, indv)
    im[neg] *= -1.
    ph = np.angle(re + 1j * im)
    theta = 2. * np.pi * (ur * dRArot + vr * dDecrot)
    return amp * (np.cos(theta + ph) + 1j * np.sin(theta + ph))


def central_pixel(I, Rmin, dR, dxy):
    iIN = int(np.floor((dxy / 2 - Rmin) // dR))
    flux = 0.
    for i in range(1, iIN):
        flux += (Rmin + dR * i) * I[i]
    flux *= 2.
    flux += Rmin * I[0] + (Rmin + iIN * dR) * I[iIN]
    flux *= dR
    I_interp = (I[iIN + 1] - I[iIN]) / dR * (dxy / 2. - (Rmin + dR * iIN)) + I[iIN]
    flux += ((Rmin + iIN * dR) * I[iIN] + dxy / 2. * I_interp) * (dxy / 2. - (Rmin + iIN * dR))
    return flux / ((dxy / 2.) ** 2 - Rmin ** 2)


def sweep_ref(I, Rmin, dR, nrow, ncol, dxy, inc, Dx=0., Dy=0., dtype='float64', origin='upper'):
    """Image of an axisymmetric profile on the pixel-centre meshgrid, linear
    interpolation in R, zero outside the profile, central pixel = mean intensity."""
    v_origin = 1. if origin == 'upper' else -1.
    nrad = len(I)
    gridrad = np.linspace(Rmin, Rmin + dR * (nrad - 1), nrad)
    x = (np.linspace(0.5, -0.5 + 1. / float(ncol), ncol)) * dxy * ncol
    y = (np.linspace(0.5, -0.5 + 1. / float(nrow), nrow)) * dxy * nrow * v_origin
    xx, yy = np.meshgrid((x - Dx) / np.cos(inc), (y - Dy))
    rr = np.sqrt(xx ** 2. + yy ** 2.)
    img = np.interp(rr, gridrad, I, left=0., right=0.)
    img[rr < gridrad[0]] = 0.
    img[int(nrow / 2 + Dy / dxy * v_origin), int(ncol / 2 - Dx / dxy)] = central_pixel(I, Rmin, dR, dxy)
    return (img * dxy ** 2.).astype(dtype)


def rel_max(a, b):
    """max|a - b| / max|b|."""
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def uv_log_uniform(nd, rmin, rmax, seed):
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), nd))
    th = rng.uniform(0, 2 * np.pi, nd)
    return r * np.cos(th), r * np.sin(th)
