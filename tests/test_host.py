"""Host-side logic of galario_gb300 that needs no GPU: argument checks with the
reference's exceptions and messages, the pure-numpy helpers, and the C ABI
library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

import galario_gb300 as g
from helpers import arcsec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "galario_gb300.h")


def test_module_surface_matches_reference():
    expected = ['arcsec', 'deg', 'cgs_to_Jy', 'pc', 'au', '_init', '_cleanup', 'set_v_origin', 'ngpus', 'use_gpu',
                'threads', 'check_obs', 'check_image_size', 'get_image_size', 'sampleImage', 'sampleProfile',
                'chi2Image', 'chi2Profile', 'get_coords_meshgrid', 'sweep', 'uv_rotate', 'interpolate',
                'apply_phase_vis', 'reduce_chi2', '_fft2d', '_fftshift', '_fftshift_axis0']
    for mod in (g.double, g.single, g.double_cuda, g.single_cuda):
        for name in expected:
            assert hasattr(mod, name), name
        assert sorted(mod.__all__) == sorted(expected)
    assert g.HAVE_CUDA is True
    assert g.arcsec == 4.84813681109536e-06 and g.deg == 0.017453292519943295


def test_library_exports_every_declared_symbol():
    from galario_gb300 import _lib
    src = open(HEADER).read()
    names = sorted(set(re.findall(r"\b(galario_\w+)\s*\(", src)))
    assert len(names) >= 30
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("mod", ["double", "single"])
def test_exception_messages_like_reference(mod):
    """test_exception (python/test_galario.py:617-628); raised before any GPU work."""
    m = getattr(g, mod)
    r = m.real_dtype
    with pytest.raises(ValueError, match="dimension.*is less than 2"):
        m._fft2d(np.ones((1, 1), dtype=r))
    with pytest.raises(ValueError, match="Expect a square image"):
        m._fft2d(np.ones((10, 12), dtype=r))
    with pytest.raises(ValueError, match="dimension.*is odd"):
        m._fft2d(np.ones((9, 9), dtype=r))


def test_buffer_checks_like_cython_memoryviews():
    d = g.double
    with pytest.raises(ValueError, match="Buffer dtype mismatch, expected 'double' but got 'float'"):
        d.sampleImage(np.ones((4, 4), np.float32), 1., np.ones(3), np.ones(3))
    with pytest.raises(ValueError, match="Buffer dtype mismatch, expected 'float' but got 'double'"):
        g.single.sampleImage(np.ones((4, 4)), 1., np.ones(3, np.float32), np.ones(3, np.float32))
    with pytest.raises(ValueError, match="ndarray is not C-contiguous"):
        d.sampleImage(np.ones((4, 8))[:, ::2], 1., np.ones(3), np.ones(3))
    with pytest.raises(ValueError, match="wrong number of dimensions"):
        d.sampleImage(np.ones(16), 1., np.ones(3), np.ones(3))
    with pytest.raises(IndexError):
        d.sampleImage(np.ones((4, 4)), 1., np.ones(0), np.ones(0))
    with pytest.raises(AssertionError, match="origin"):
        d.sampleImage(np.ones((4, 4)), 1., np.ones(3), np.ones(3), origin="left")
    with pytest.raises(AssertionError, match="Wrong array length: vis_obs_im"):
        d.chi2Image(np.ones((4, 4)), 1., np.ones(3), np.ones(3), np.ones(3), np.ones(2), np.ones(3))
    with pytest.raises(AssertionError, match="Rmin < dxy"):
        d.sampleProfile(np.ones(10), 2., 1., 8, 1., np.ones(3), np.ones(3))


def test_profile_checks_before_gpu():
    with pytest.raises(ValueError, match="Try reducing dR"):
        g.double.chi2Profile(np.ones(4096), 1e-4 * arcsec, 1e-3 * arcsec, 4096, 3e-3 * arcsec, np.ones(3),
                             np.ones(3), np.ones(3), np.ones(3), np.ones(3))
    with pytest.raises(ValueError, match="is odd"):
        g.double.sampleProfile(np.ones(100), 1e-6, 1e-7, 15, 1e-5, np.ones(3), np.ones(3))


def test_get_coords_meshgrid_like_reference():
    """test_get_coords_meshgrid (python/test_galario.py:631-656)."""
    for mod, nxy, inc, dxy, Dx, Dy, tol in [(g.single, 1000, 20., 2e-3, -2., 0., 1e-6),
                                            (g.double, 1000, 33.4, 1e-8, 0.23, -1.23, 1e-15)]:
        real = mod.real_dtype
        x = (np.linspace(0.5, -0.5 + 1. / nxy, nxy, dtype=real)) * dxy * nxy
        y = (np.linspace(0.5, -0.5 + 1. / nxy, nxy, dtype=real)) * dxy * nxy
        x_m, y_m = np.meshgrid((x - Dx) / np.cos(inc), y - Dy)
        R_m = np.sqrt(x_m ** 2. + y_m ** 2.)
        got = mod.get_coords_meshgrid(nxy, nxy, dxy, inc, Dx=Dx, Dy=Dy, origin='upper')
        for a, b in zip((x, y, x_m, y_m, R_m), got):
            np.testing.assert_allclose(b, a, atol=0, rtol=tol)


def test_image_size_helpers():
    rng = np.random.default_rng(0)
    r = rng.uniform(1e4, 2e6, 1000)
    th = rng.uniform(0, 2 * np.pi, 1000)
    u, v = r * np.cos(th), r * np.sin(th)
    nxy, dxy = g.double.get_image_size(u, v)
    assert nxy & (nxy - 1) == 0
    duv = 1 / (nxy * dxy)
    assert g.double.check_image_size(u, v, nxy, dxy, duv)
    with pytest.raises(AssertionError):
        g.double.check_image_size(u, v, 64, dxy, 1 / (64 * dxy))


def test_threads_hint():
    t0 = g.double.threads()
    assert g.double.threads(8) == 8
    g.double.threads(t0)
