"""GPU parity of the galario_gb300 CUDA path against the CPU oracle.

Tolerances (double): max|dV|/max|V| <= 1e-12 and |dchi2|/chi2 <= 1e-12.
Tolerances (single, against the double oracle): max|dV|/max|V| <= 1e-5 and
|dchi2|/chi2 <= 1e-6.  Every call goes through the C ABI of
libgalario_gb300.so.
"""
import numpy as np
import pytest

from helpers import (arcsec, deg, par1, par2, par3, par4, reference_image, sampling_points, radial_profile,
                     random_vis, matrix_size, uv_idx_r2c, bilinear, apply_phase_array, rel_max, sweep_ref,
                     py_sample_image, uv_log_uniform)

pytestmark = pytest.mark.gpu

DP_V, DP_CHI2 = 1e-12, 1e-12
SP_V, SP_CHI2 = 1e-5, 1e-6


@pytest.fixture(scope="module")
def g():
    import galario_gb300 as g
    g.double.use_gpu(0)
    return g


@pytest.fixture(scope="module")
def orc(oracle_port):
    return {"double": oracle_port.get("port", "double"), "single": oracle_port.get("port", "single")}


def _ring_image(nxy, dxy, r0=0.3, sig=0.05, flux=0.1, dtype=np.float64):
    x = (np.linspace(0.5, -0.5 + 1. / nxy, nxy)) * nxy
    xx, yy = np.meshgrid(x, x)
    r = np.hypot(xx, yy) * dxy / arcsec
    img = np.exp(-(r - r0) ** 2 / (2 * sig ** 2))
    return (img * flux / img.sum()).astype(dtype)


def _obs(nd, seed=1):
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    return rng.normal(0, sigma), rng.normal(0, sigma), 1. / sigma ** 2


# --------------------------------------------------------------------- FFT
@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 256, 1024, 2048, 10, 12, 36, 100])
@pytest.mark.parametrize("prec", ["double", "single"])
def test_fft2d_vs_numpy(g, n, prec):
    mod = getattr(g, prec)
    rng = np.random.default_rng(n)
    img = rng.standard_normal((n, n)).astype(mod.real_dtype)
    ref = np.fft.rfft2(img.astype(np.float64))
    out = mod._fft2d(img)
    assert out.shape == (n, n // 2 + 1)
    tol = 1e-14 if prec == "double" else 2e-6
    assert rel_max(out, ref) <= tol


# ---------------------------------------------------- end-to-end, double
@pytest.mark.parametrize("pars", [par1, par2, par4], ids=["par1", "par2", "par4"])
@pytest.mark.parametrize("origin", ["upper", "lower"])
def test_sample_image_double(g, orc, pars, origin):
    nxy = pars['nxy']
    u, v = sampling_points(3000, 3e3)
    _, minuv, maxuv = matrix_size(u, v)
    dxy = 1. / maxuv
    img = reference_image(nxy)
    kw = dict(dRA=pars['dRA'] * arcsec, dDec=pars['dDec'] * arcsec, PA=pars['PA'] * deg, origin=origin)
    vg = g.double.sampleImage(img, dxy, u, v, **kw)
    vo = orc["double"].sampleImage(img, dxy, u, v, **kw)
    assert rel_max(vg, vo) <= DP_V


def test_chi2_image_double_config0(g, orc):
    """The reference's CPU-runnable configuration: chi2Image in float64,
    nxy = 1024, dxy = 0.01 arcsec, a Gaussian ring (r0 = 0.3", sigma = 0.05")
    of 0.1 Jy, 1e5 uv points with radius log-uniform in [1e4, 2e6] wavelengths
    and uniform angle, observations = the reference's sampleImage plus
    Gaussian noise with sigma uniform in [0.5, 1.5] mJy and w = 1/sigma^2,
    dRA = 0.05", dDec = -0.03", origin 'upper', seed 0."""
    nxy, dxy, nd = 1024, 0.01 * arcsec, 100000
    img = _ring_image(nxy, dxy)
    u, v = uv_log_uniform(nd, 1e4, 2e6, seed=0)
    kw = dict(dRA=0.05 * arcsec, dDec=-0.03 * arcsec, PA=0., origin='upper')
    model = orc["double"].sampleImage(img, dxy, u, v, **kw)
    vg = g.double.sampleImage(img, dxy, u, v, **kw)
    assert rel_max(vg, model) <= DP_V
    rng = np.random.default_rng(0)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    n_re, n_im = rng.normal(0, sigma), rng.normal(0, sigma)
    re, im, w = model.real + n_re, model.imag + n_im, 1. / sigma ** 2
    cg = g.double.chi2Image(img, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Image(img, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2
    # the exact model leaves the noise
    noise = np.sum(w * (n_re ** 2 + n_im ** 2))
    assert abs(cg - noise) / noise <= 1e-9
    # a model shifted by 0.01" is worse than the true one
    kw2 = dict(kw, dRA=0.06 * arcsec)
    assert g.double.chi2Image(img, dxy, u, v, re, im, w, **kw2) > cg


def test_chi2_image_double_small(g, orc):
    """A small image with uv points up to 0.49 of the spectrum half-width."""
    nxy, nd = 64, 500
    dxy = 0.01 * arcsec * 1024 / nxy
    img = _ring_image(nxy, dxy)
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(nd, 1e4 * 64 / nxy, 0.49 * nxy / 2 * duv, seed=0)
    re, im, w = _obs(nd)
    kw = dict(dRA=0.05 * arcsec, dDec=-0.03 * arcsec, PA=0.)
    cg = g.double.chi2Image(img, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Image(img, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2


@pytest.mark.parametrize("inc,PA,dRA,dDec", [(0., 0., 0., 0.), (40 * deg, 70 * deg, 0.02, -0.04), (70 * deg, 3., -0.05, 0.01)])
def test_profile_double(g, orc, inc, PA, dRA, dDec):
    nxy, dxy = 1024, 3e-3 * arcsec * 4
    Rmin, dR, nr = 1e-4 * arcsec, 1e-3 * arcsec, 2048
    R = Rmin + dR * np.arange(nr)
    I = np.exp(-0.5 * ((R - 0.6 * arcsec) / (0.08 * arcsec)) ** 2) + 0.4 * np.exp(
        -0.5 * ((R - 1.4 * arcsec) / (0.2 * arcsec)) ** 2)
    I *= 1e10
    duv = 1 / (nxy * dxy)
    nd = 20000
    u, v = uv_log_uniform(nd, 1e3, 0.45 * nxy / 2 * duv, seed=3)
    re, im, w = _obs(nd, seed=4)
    kw = dict(inc=inc, PA=PA, dRA=dRA * arcsec, dDec=dDec * arcsec)
    vg = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
    vo = orc["double"].sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
    assert rel_max(vg, vo) <= DP_V
    cg = g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2


@pytest.mark.parametrize("nxy", [256, 250])
def test_profile_wider_than_image(g, orc, nxy):
    """Profile support beyond the image (rmax clamped to nxy/2: the edge row and
    column carry emission) and a non power of two size: the symmetric-profile
    shortcuts (shared mirror rows, paired real columns, real spectrum) must
    still match the oracle."""
    dxy = 0.02 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 1e-3 * arcsec, 4000  # extent 4", image half-width 2.5"
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * (R / (1.5 * arcsec)) ** 2)
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(5000, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=5)
    re, im, w = _obs(5000, seed=6)
    kw = dict(inc=35 * deg, PA=1.2, dRA=0.03 * arcsec, dDec=-0.01 * arcsec)
    vg = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
    vo = orc["double"].sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
    assert rel_max(vg, vo) <= DP_V
    cg = g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2


@pytest.mark.parametrize("n", [250, 360, 1000, 6000])
@pytest.mark.parametrize("prec", ["double", "single"])
def test_fft2d_mixed_radix_sizes(g, n, prec):
    """Even sizes that are not powers of two (250 = 2 5^3, 360 = 2^3 3^2 5,
    1000 = 2^3 5^3, 6000 = 2^4 3 5^3): the mixed-radix (2, 3, 4, 5, 7)
    shared-memory FFT of the row and column passes, against numpy's rfft2."""
    mod = getattr(g, prec)
    rng = np.random.default_rng(n + 7)
    img = rng.standard_normal((n, n)).astype(mod.real_dtype)
    ref = np.fft.rfft2(img.astype(np.float64))
    out = mod._fft2d(img)
    assert out.shape == (n, n // 2 + 1)
    tol = 1e-14 if prec == "double" else 4e-6
    assert rel_max(out, ref) <= tol, rel_max(out, ref)


@pytest.mark.parametrize("nxy", [360, 1000])
def test_chi2_image_mixed_radix_sizes(g, orc, nxy):
    """chi2Image and sampleImage end to end at non-power-of-two sizes against the oracle."""
    dxy = 0.01 * arcsec * 1024 / nxy
    img = _ring_image(nxy, dxy)
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(20000, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=nxy)
    re, im, w = _obs(20000, seed=nxy + 1)
    kw = dict(dRA=0.02 * arcsec, dDec=-0.01 * arcsec, PA=0.7)
    vg = g.double.sampleImage(img, dxy, u, v, **kw)
    vo = orc["double"].sampleImage(img, dxy, u, v, **kw)
    assert rel_max(vg, vo) <= DP_V
    cg = g.double.chi2Image(img, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Image(img, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2


def test_sweep_double(g, orc):
    Rmin, dR, nr = 1e-6 * arcsec, 0.001 * arcsec, 2000
    dxy = 0.2 * arcsec
    I = radial_profile(Rmin, dR, nr, 'Cos-Gauss', gauss_width=dxy * 6)
    for nxy, inc in [(1024, 20 * deg), (2048, 44.23 * deg), (6, 0.), (10, 0.3)]:
        a = g.double.sweep(I, Rmin, dR, nxy, 0.2 * arcsec, inc)
        b = orc["double"].sweep(I, Rmin, dR, nxy, 0.2 * arcsec, inc)
        assert a.shape == (nxy, nxy)
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


# ----------------------------------------------------- end-to-end, single
def test_single_vs_double_oracle(g, orc):
    nxy, dxy = 1024, 0.01 * arcsec
    img = _ring_image(nxy, dxy)
    duv = 1 / (nxy * dxy)
    nd = 50000
    u, v = uv_log_uniform(nd, 1e4, 0.45 * nxy / 2 * duv, seed=5)
    re, im, w = _obs(nd, seed=6)
    kw = dict(dRA=0.05 * arcsec, dDec=-0.03 * arcsec, PA=0.7)
    vo = orc["double"].sampleImage(img, dxy, u, v, **kw)
    f = np.float32
    vs = g.single.sampleImage(img.astype(f), dxy, u.astype(f), v.astype(f), **kw)
    assert vs.dtype == np.complex64
    # the single inputs are rounded to float32: compare against the double oracle on the same rounded inputs
    vo32 = orc["double"].sampleImage(img.astype(f).astype(np.float64), dxy, u.astype(f).astype(np.float64),
                                     v.astype(f).astype(np.float64), **kw)
    assert rel_max(vs, vo32) <= SP_V
    assert rel_max(vs, vo) <= 1e-4
    cs = g.single.chi2Image(img.astype(f), dxy, u.astype(f), v.astype(f), re.astype(f), im.astype(f), w.astype(f), **kw)
    co = orc["double"].chi2Image(img.astype(f).astype(np.float64), dxy, u.astype(f).astype(np.float64),
                                 v.astype(f).astype(np.float64), re.astype(f).astype(np.float64),
                                 im.astype(f).astype(np.float64), w.astype(f).astype(np.float64), **kw)
    assert abs(cs - co) / abs(co) <= SP_CHI2


# ------------------------------------------------------------ expert stages
@pytest.mark.parametrize("prec", ["double", "single"])
def test_interpolate_vs_numpy(g, prec):
    mod = getattr(g, prec)
    size, maxuv = 1024, 1000.
    img = reference_image(size)
    u, v = sampling_points(10000, maxuv / 2.2)
    du = maxuv / size
    indu, indv = uv_idx_r2c(u, v, du, size / 2.)
    ft = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(img)))
    re, im, amp = bilinear(ft.real, indu, indv), bilinear(ft.imag, indu, indv), bilinear(np.abs(ft), indu, indv)
    im[u < 0] *= -1.
    ph = np.angle(re + 1j * im)
    ref = amp * np.exp(1j * ph)
    out = mod.interpolate(ft.astype(mod.complex_dtype), du, u.astype(mod.real_dtype), v.astype(mod.real_dtype))
    tol = 1e-13 if prec == "double" else 2e-5
    assert rel_max(out, ref) <= tol


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("pars", [par1, par2, par3])
def test_apply_phase_vis(g, prec, pars):
    mod = getattr(g, prec)
    dRA, dDec = pars['dRA'] * arcsec, pars['dDec'] * arcsec
    u, v = sampling_points(10000, 3e3, dtype=mod.real_dtype)
    rng = np.random.RandomState(3)
    vis = (rng.random_sample(10000) * 10. + 1j * rng.random_sample(10000) * 30.).astype(mod.complex_dtype)
    ref = apply_phase_array(u.astype(np.float64), v.astype(np.float64), vis.astype(np.complex128), dRA, dDec)
    out = mod.apply_phase_vis(dRA, dDec, u, v, vis)
    tol = 1e-14 if prec == "double" else 1e-6
    assert rel_max(out, ref) <= tol


@pytest.mark.parametrize("prec", ["double", "single"])
def test_reduce_chi2(g, prec):
    mod = getattr(g, prec)
    x, y, w = random_vis(1000, mod.real_dtype)
    ref = np.sum(((x.real - y.real) ** 2. + (x.imag - y.imag) ** 2.) * w.astype(np.float64))
    out = mod.reduce_chi2(x.real.copy(), x.imag.copy(), w, y.astype(mod.complex_dtype))
    tol = 1e-14 if prec == "double" else 1e-6
    assert abs(out - ref) / ref <= tol


@pytest.mark.parametrize("prec", ["double", "single"])
def test_uv_rotate_and_shifts(g, prec):
    mod = getattr(g, prec)
    u, v = sampling_points(1000, 3e3, dtype=mod.real_dtype)
    a, b, ur, vr = mod.uv_rotate(0.3, 1e-6, -2e-6, u, v)
    c, s = np.cos(0.3), np.sin(0.3)
    tol = 1e-14 if prec == "double" else 1e-6
    np.testing.assert_allclose(ur, u * c - v * s, rtol=tol, atol=tol * 3e3)
    np.testing.assert_allclose(vr, u * s + v * c, rtol=tol, atol=tol * 3e3)
    np.testing.assert_allclose([a, b], [1e-6 * c + 2e-6 * s, 1e-6 * s - 2e-6 * c], rtol=1e-6 if prec == "single" else 1e-14)
    img = reference_image(64, dtype=mod.real_dtype)
    sh = mod._fftshift(img).view(mod.real_dtype)[:, :-2]
    np.testing.assert_array_equal(sh, np.fft.fftshift(img))
    m = (np.random.RandomState(1).random_sample((64, 33)) + 1j).astype(mod.complex_dtype)
    ref = np.fft.fftshift(m, axes=0)
    mod._fftshift_axis0(m)
    np.testing.assert_array_equal(m, ref)


# --------------------------------------------------------- reference tests
@pytest.mark.parametrize("pars", [par1, par2, par3, par4], ids=["0", "1", "2", "3"])
def test_all_like_reference(g, pars):
    """Restates test_all (python/test_galario.py:431-504): sampleImage,
    sampleProfile, chi2Image, chi2Profile against the numpy restatement."""
    u, v = sampling_points(1000, 3e3)
    _, minuv, maxuv = matrix_size(u, v)
    nxy = pars['nxy']
    dxy = 1. / maxuv
    Rmin, dR, nrad, inc = dxy / 100., dxy / 10.5, 10000, 20. * deg
    dRA, dDec, PA = pars['dRA'] * arcsec, pars['dDec'] * arcsec, pars['PA'] * deg
    I = radial_profile(Rmin, dR, nrad, 'Gauss', gauss_width=dxy * 10)
    img = sweep_ref(I, Rmin, dR, nxy, nxy, dxy, inc)
    vpy = py_sample_image(img, dxy, u, v, PA=PA, dRA=dRA, dDec=dDec)
    vg = g.double.sampleImage(img, dxy, u, v, PA=PA, dRA=dRA, dDec=dDec)
    rtol = 1e-6
    np.testing.assert_allclose(vg.real, vpy.real, rtol=rtol, atol=0)
    np.testing.assert_allclose(vg.imag, vpy.imag, rtol=rtol, atol=np.abs(np.mean(vg.real)) * rtol)
    vp = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, inc=inc, dRA=dRA, dDec=dDec, PA=PA)
    np.testing.assert_allclose(vp.real, vg.real, rtol=rtol, atol=0)
    np.testing.assert_allclose(vp.imag, vg.imag, rtol=rtol, atol=np.abs(np.mean(vp.real)) * rtol)
    x, _, w = random_vis(1000, 'float64')
    c_img = g.double.chi2Image(img, dxy, u, v, x.real.copy(), x.imag.copy(), w, dRA=dRA, dDec=dDec)
    c_pro = g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, x.real.copy(), x.imag.copy(), w, inc=inc, dRA=dRA,
                                 dDec=dDec)
    vpy0 = py_sample_image(img, dxy, u, v, dRA=dRA, dDec=dDec)
    c_py = np.sum(((vpy0.real - x.real) ** 2 + (vpy0.imag - x.imag) ** 2) * w)
    np.testing.assert_allclose(c_img, c_py, rtol=rtol)
    np.testing.assert_allclose(c_pro, c_img, rtol=rtol)


def test_uv_wrap_and_outside_spectrum(g, orc):
    """A corner past the last spectrum column wraps into the next row of the
    row-major N x (N/2+1) array, exactly as the reference's flat indexing does
    (src/galario.cpp:774-780); a corner past the end of the array raises."""
    nxy, dxy = 64, 1e-8
    duv = 1 / (nxy * dxy)
    img = reference_image(nxy)
    u = np.array([0.1 * duv, 40.3 * duv, -32.5 * duv])
    v = np.array([0.2 * duv, 0.1 * duv, 3.7 * duv])
    vg = g.double.sampleImage(img, dxy, u, v)
    vo = orc["double"].sampleImage(img, dxy, u, v)
    assert rel_max(vg, vo) <= DP_V
    bad_v = np.array([0.2 * duv, 40 * duv])
    with pytest.raises(ValueError, match="outside the image spectrum"):
        g.double.sampleImage(img, dxy, u[:2].copy(), bad_v)
    with pytest.raises(ValueError, match="not finite"):
        g.double.sampleImage(img, dxy, np.array([np.nan, 1.]), np.array([0., 1.]))
    # the context stays usable afterwards
    out = g.double.sampleImage(img, dxy, u[:1].copy(), v[:1].copy())
    assert np.isfinite(out).all()


def test_concurrent_host_threads(g):
    """Calls from several host threads (ctypes releases the GIL) are serialised
    per device by the library and give the same results as sequential calls."""
    from concurrent.futures import ThreadPoolExecutor
    nxy, dxy = 512, 0.01 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 5e-4 * arcsec, 2000
    R = Rmin + dR * np.arange(nr)
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(20000, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=9)
    re, im, w = _obs(20000, seed=10)
    profiles = [1e10 * np.exp(-0.5 * ((R - (0.2 + 0.05 * k) * arcsec) / (0.05 * arcsec)) ** 2) for k in range(8)]

    def run(k):
        return g.double.chi2Profile(profiles[k], Rmin, dR, nxy, dxy, u, v, re, im, w, inc=0.1 * k, PA=0.2 * k)
    seq = [run(k) for k in range(8)]
    with ThreadPoolExecutor(max_workers=4) as ex:
        par = list(ex.map(run, range(8)))
    assert par == seq  # the same launches in the same order per call: bit-identical


def test_profile_sign_near_zero_crossings(g, orc):
    """The FP64 profile path takes the sign of the interpolated real spectrum
    value z from an FP32 estimate and recomputes it in FP64 when the estimate
    is within its error bound of zero.  Points placed 1e-9, 1e-6 and 1e-3 of a
    cell beside the zero crossings of z along the u axis (v = 0, where z is
    linear in the cell fraction) exercise both branches; a wrong sign would
    flip a visibility of full amplitude.  The real parts are compared: the
    reference's value there also carries an imaginary part amp * Im z / Re z,
    the rounding-level imaginary part of its FFT over a vanishing real part,
    which the real-spectrum path does not have."""
    nxy, dxy = 512, 0.02 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 1e-3 * arcsec, 4000
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * ((R - 1.0 * arcsec) / (0.1 * arcsec)) ** 2)
    duv = 1 / (nxy * dxy)
    kmax = int(0.45 * nxy / 2)
    # at v = 0 and a whole cell index the interpolation returns the corner itself
    uk = np.arange(1, kmax + 1) * duv
    yk = orc["double"].sampleProfile(I, Rmin, dR, nxy, dxy, uk, np.zeros_like(uk)).real
    u = []
    scale = np.abs(yk).max()
    for k in range(len(yk) - 1):
        a, b = yk[k], yk[k + 1]
        if a * b < 0 and min(abs(a), abs(b)) > 1e-6 * scale:
            qs = a / (a - b)  # z = a + q (b - a) vanishes at q = a / (a - b)
            for d in (1e-9, -1e-9, 1e-6, -1e-6, 1e-3, -1e-3):
                q = qs + d
                if 0 < q < 1:
                    u.append((k + 1 + q) * duv)
    assert len(u) >= 24, len(u)
    u = np.array(u)
    v = np.zeros_like(u)
    vg = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v)
    vo = orc["double"].sampleProfile(I, Rmin, dR, nxy, dxy, u, v)
    assert np.array_equal(np.sign(vg.real), np.sign(vo.real))
    assert rel_max(vg.real, vo.real) <= DP_V
    assert np.all(vg.imag == 0)


def test_chunked_host_pointer_chi2_profile(g, orc):
    """A host-pointer chi2Profile of more than 2^19 visibilities uploads and
    evaluates them in chunks on two streams (one chi2 reduction over all
    chunks): same chi2 as the oracle, and an invalid point of a later chunk is
    reported with its index in the whole array."""
    nxy, dxy = 512, 0.02 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 1e-3 * arcsec, 4000
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * ((R - 0.8 * arcsec) / (0.15 * arcsec)) ** 2)
    duv = 1 / (nxy * dxy)
    nd = 3 * (1 << 18) + 123  # three chunks of uneven length
    u, v = uv_log_uniform(nd, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=11)
    re, im, w = _obs(nd, seed=12)
    kw = dict(inc=30 * deg, PA=0.7, dRA=0.02 * arcsec, dDec=0.01 * arcsec)
    cg = g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    co = orc["double"].chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    assert abs(cg - co) / abs(co) <= DP_CHI2
    # deterministic: the same call again gives the same bits
    assert g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw) == cg
    bad = u.copy()
    bad[700001] = np.nan
    with pytest.raises(ValueError, match="not finite.*index 700001"):
        g.double.chi2Profile(I, Rmin, dR, nxy, dxy, bad, v, re, im, w, **kw)
    # the context stays usable afterwards
    assert g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw) == cg


def test_profile_records_full_window_and_wrap(g, orc):
    """FP64 profiles at nxy >= 1024 take the even-sequence column pass, which
    also writes the real cell records; with points beyond |u| = N/2 duv the
    window spans every column (K = N/2 + 1) and the records of the last column
    take their u + 1 corners from column 0 of the next rows, as the
    reference's flat indexing does (src/galario.cpp:774-780)."""
    nxy, dxy = 1024, 0.01 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 5e-4 * arcsec, 6000  # (dxy/2 - Rmin)/dR = 9.8 > 5
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * ((R - 0.5 * arcsec) / (0.2 * arcsec)) ** 2)
    duv = 1 / (nxy * dxy)
    rng = np.random.default_rng(13)
    u = np.concatenate([rng.uniform(-0.49, 0.49, 3000) * nxy * duv,
                        np.array([512.3, -512.6, 512.9, 600.2, 0.25, 511.5]) * duv])
    v = np.concatenate([rng.uniform(-0.49, 0.49, 3000) * nxy * duv,
                        np.array([3.2, -7.7, 0.4, 11.1, 0.3, -200.2]) * duv])
    for kw in (dict(), dict(inc=0.5, dRA=0.01 * arcsec, dDec=-0.02 * arcsec)):
        vg = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
        vo = orc["double"].sampleProfile(I, Rmin, dR, nxy, dxy, u, v, **kw)
        assert rel_max(vg.real, vo.real) <= DP_V
        re, im, w = _obs(len(u), seed=14)
        cg = g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
        co = orc["double"].chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
        assert abs(cg - co) / abs(co) <= DP_CHI2
