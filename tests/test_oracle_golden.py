"""The CPU oracle (oracle/galario_oracle.c) pinned to the reference.

- against the golden fixtures produced by the reference's own CPU code
  (tests/golden/make_golden.py);
- its FFT against numpy.fft with the reference's test_FFT contract
  (python/test_galario.py:222-244: DP rtol 1e-16 / atol 1e-8, SP 1e-5 / 1e-3);
- its end-to-end path against the numpy restatement of the reference tests
  (test_all, python/test_galario.py:431-504, rtol 1e-6).
"""
import numpy as np
import pytest

import golden_cases
from helpers import (arcsec, deg, par1, par4, reference_image, sampling_points, matrix_size, radial_profile,
                     sweep_ref, py_sample_image, random_vis)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_oracle_matches_reference_golden(oracle_port, precision):
    impl = oracle_port.get("port", precision)
    d = golden_cases.load(precision)
    tol = 1e-13 if precision == "double" else 1e-5
    for name, got, exp in golden_cases.run_all(impl, d):
        assert np.shape(got) == np.shape(exp), name
        assert golden_cases.rel(got, exp) <= tol, (name, golden_cases.rel(got, exp))


@pytest.mark.parametrize("precision,rtol,atol", [("double", 1e-16, 1e-8), ("single", 1e-5, 1e-3)])
@pytest.mark.parametrize("size", [16, 1024, 10, 100])
def test_oracle_fft_vs_numpy(oracle_port, precision, rtol, atol, size):
    impl = oracle_port.get("port", precision)
    img = reference_image(size, dtype=impl.real)
    ft = np.fft.fft2(img)
    got = impl._fft2d(img)
    assert got.shape == (size, size // 2 + 1)
    np.testing.assert_allclose(got.real, ft[:, :size // 2 + 1].real, rtol=rtol, atol=atol)
    np.testing.assert_allclose(got.imag, ft[:, :size // 2 + 1].imag, rtol=rtol, atol=atol)


@pytest.mark.parametrize("pars", [par1, par4], ids=["par1", "par4"])
def test_oracle_all_like_reference(oracle_port, pars):
    impl = oracle_port.get("port", "double")
    u, v = sampling_points(1000, 3e3)
    _, minuv, maxuv = matrix_size(u, v)
    nxy = pars['nxy']
    dxy = 1. / maxuv
    Rmin, dR, nrad, inc = dxy / 100., dxy / 10.5, 10000, 20. * deg
    dRA, dDec, PA = pars['dRA'] * arcsec, pars['dDec'] * arcsec, pars['PA'] * deg
    I = radial_profile(Rmin, dR, nrad, 'Gauss', gauss_width=dxy * 10)
    img = sweep_ref(I, Rmin, dR, nxy, nxy, dxy, inc)
    vpy = py_sample_image(img, dxy, u, v, PA=PA, dRA=dRA, dDec=dDec)
    vo = impl.sampleImage(img, dxy, u, v, PA=PA, dRA=dRA, dDec=dDec)
    np.testing.assert_allclose(vo.real, vpy.real, rtol=1e-6, atol=0)
    np.testing.assert_allclose(vo.imag, vpy.imag, rtol=1e-6, atol=np.abs(np.mean(vo.real)) * 1e-6)
    vp = impl.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, inc=inc, dRA=dRA, dDec=dDec, PA=PA)
    np.testing.assert_allclose(vp.real, vo.real, rtol=1e-6, atol=0)
    x, _, w = random_vis(1000, 'float64')
    c1 = impl.chi2Image(img, dxy, u, v, x.real.copy(), x.imag.copy(), w, dRA=dRA, dDec=dDec)
    vpy0 = py_sample_image(img, dxy, u, v, dRA=dRA, dDec=dDec)
    np.testing.assert_allclose(c1, np.sum(((vpy0.real - x.real) ** 2 + (vpy0.imag - x.imag) ** 2) * w), rtol=1e-6)


def test_oracle_sweep_vs_numpy(oracle_port):
    """Restates test_intensity_sweep (python/test_galario.py:63-111) at rtol 1e-12."""
    impl = oracle_port.get("port", "double")
    Rmin, dR, nrad, nxy, dxy, inc = 1e-6 * arcsec, 0.001 * arcsec, 2000, 1024, 0.2 * arcsec, 20. * deg
    I = radial_profile(Rmin, dR, nrad, 'Gauss', gauss_width=dxy * 6)
    ref = sweep_ref(I, Rmin, dR, nxy, nxy, dxy, inc)
    got = impl.sweep(I, Rmin, dR, nxy, dxy, inc)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)


def test_oracle_errors(oracle_port):
    impl = oracle_port.get("port", "double")
    with pytest.raises(ValueError, match="dimension.*is less than 2"):
        impl._fft2d(np.ones((1, 1)))
    with pytest.raises(ValueError, match="Expect a square image"):
        impl._fft2d(np.ones((10, 12)))
    with pytest.raises(ValueError, match="dimension.*is odd"):
        impl._fft2d(np.ones((9, 9)))
    with pytest.raises(ValueError, match="Try reducing dR"):
        impl.chi2Profile(np.ones(100), 1e-4 * arcsec, 1e-3 * arcsec, 64, 3e-3 * arcsec, np.ones(3), np.ones(3),
                         np.ones(3), np.ones(3), np.ones(3))


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).have_ref(), reason="reference build absent")
@pytest.mark.parametrize("precision", ["double", "single"])
def test_oracle_port_vs_reference_build(oracle_port, precision):
    """Where the reference build exists (oracle/_ref), the port agrees with it at a larger size."""
    port, ref = oracle_port.get("port", precision), oracle_port.get("ref", precision)
    nxy, dxy = 512, 0.01 * arcsec
    duv = 1 / (nxy * dxy)
    img = reference_image(nxy, sigma_x=400., sigma_y=300., dtype=port.real)
    rng = np.random.default_rng(5)
    r = rng.uniform(0.01, 0.45, 20000) * nxy / 2 * duv
    th = rng.uniform(0, 2 * np.pi, 20000)
    u, v = (r * np.cos(th)).astype(port.real), (r * np.sin(th)).astype(port.real)
    kw = dict(dRA=0.1 * arcsec, dDec=-0.05 * arcsec, PA=1.1)
    a, b = port.sampleImage(img, dxy, u, v, **kw), ref.sampleImage(img, dxy, u, v, **kw)
    assert golden_cases.rel(a, b) <= (1e-15 if precision == "double" else 1e-6)
