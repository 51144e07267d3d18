"""Implementation of the ``galario_gb300.double`` / ``galario_gb300.single`` modules.

Each module mirrors the Python surface of the reference's ``galario.double``
/ ``galario.single`` (``python/libcommon.pyx:32-39``): same function names,
argument order, defaults, units and exceptions.  Arguments are checked the
way the reference's Cython typed memoryviews check them (exact dtype,
C-contiguity, dimensionality -> ``ValueError``), then the call goes through
the C ABI (``include/galario_gb300.h``) to the CUDA kernels.  There is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

# constants (reference libcommon.pyx:42-47)
arcsec = 4.84813681109536e-06       # radians
deg = 0.017453292519943295          # radians
cgs_to_Jy = 1e23                    # 1 Jy = 1.0e-23 erg/(s cm^2 Hz)
pc = 3.0856775815e18                # cm (IAU 2015 Resolution B2)
au = 1.49597870700e13               # cm (IAU 2012 Resolution B1)

__all__ = ['arcsec', 'deg', 'cgs_to_Jy', 'pc', 'au',
           '_init', '_cleanup', 'set_v_origin',
           'ngpus', 'use_gpu', 'threads',
           'check_obs', 'check_image_size', 'get_image_size',
           'sampleImage', 'sampleProfile', 'chi2Image', 'chi2Profile',
           'get_coords_meshgrid',
           'sweep', 'uv_rotate', 'interpolate', 'apply_phase_vis', 'reduce_chi2',
           '_fft2d', '_fftshift', '_fftshift_axis0']

_CY_NAMES = {np.dtype(np.float64): "double", np.dtype(np.float32): "float",
             np.dtype(np.complex128): "double complex", np.dtype(np.complex64): "float complex",
             np.dtype(np.int64): "long", np.dtype(np.int32): "int", np.dtype(np.float16): "half"}


def _cy(dt) -> str:
    return _CY_NAMES.get(np.dtype(dt), str(np.dtype(dt)))


def _buffer(x, dtype, ndim: int):
    """Accept exactly what a Cython ``dtype[::1]`` / ``dtype[:, ::1]`` memoryview accepts."""
    try:
        a = x if isinstance(x, np.ndarray) else np.asarray(memoryview(x))
    except TypeError:
        raise TypeError("a bytes-like object is required, not '%s'" % type(x).__name__) from None
    if a.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d)" % (ndim, a.ndim))
    if a.dtype != np.dtype(dtype):
        raise ValueError("Buffer dtype mismatch, expected '%s' but got '%s'" % (_cy(dtype), _cy(a.dtype)))
    if not a.flags.c_contiguous:
        raise ValueError("ndarray is not C-contiguous")
    return a


def _first(a):
    """The reference takes ``&a[0]``, which raises on an empty buffer."""
    if a.shape[0] == 0:
        raise IndexError("Out of bounds on buffer access (axis 0)")


def _ptr(a) -> int:
    return a.ctypes.data


def set_v_origin(origin):
    """Dec (v) axis orientation of the matrix origin (libcommon.pyx:107-116)."""
    if origin == 'upper':
        return 1.
    elif origin == 'lower':
        return -1.
    raise AssertionError("Expect origin='upper' or 'lower', got {}".format(origin))


def check_obs(vis_obs_re, vis_obs_im, vis_obs_w, vis=None, u=None, v=None):
    """Consistency of the observation arrays' lengths (libcommon.pyx:208-220)."""
    nd = len(vis_obs_re)
    assert len(vis_obs_im) == nd, "Wrong array length: vis_obs_im."
    assert len(vis_obs_w) == nd, "Wrong array length: vis_obs_w."
    if vis is not None and len(vis):
        assert len(vis) == nd, "Wrong array length: vis."
    if u is not None and len(u):
        assert len(u) == nd, "Wrong array length: u"
    if v is not None and len(v):
        assert len(v) == nd, "Wrong array length: v"
    return True


def check_image_size(u, v, nxy, dxy, duv, PB=0, verbose=False):
    """Nyquist / field-of-view checks of the image set-up (libcommon.pyx:223-288)."""
    assert len(u) == len(v), "Wrong array length: u, v must have same length."
    uvdist = np.hypot(u, v)
    MRS = 0.6 / np.min(uvdist)
    max_uv = np.max(uvdist) * 2.
    FOV = nxy * dxy
    FOV_to_MRS = FOV / MRS
    UVFOV_to_MAXUV = 1 / (max_uv * dxy)
    FOV_to_MRS_str = "Nxy * dxy / MRS = {} must be > 1 at the very least".format(FOV_to_MRS)
    UVFOV_to_MAXUV_str = "Nxy * duv / (2*max(u,v)) = {} must be > 2 for Nyquist sampling".format(UVFOV_to_MAXUV)
    if PB != 0:
        FOV_to_PB = FOV / PB
        FOV_to_PB_str = "Nxy * dxy / PB = {} must be > 1".format(FOV_to_PB)
    if verbose:
        print(FOV_to_MRS_str)
        print(UVFOV_to_MAXUV_str)
        if PB != 0:
            print(FOV_to_PB_str)
    assert FOV_to_MRS > 1, FOV_to_MRS_str
    assert UVFOV_to_MAXUV > 2, UVFOV_to_MAXUV_str
    if PB != 0:
        assert FOV_to_PB > 1, FOV_to_PB_str
    # the interpolation indices must stay inside the spectrum
    assert np.max(np.abs(u) / duv <= nxy // 2 + 1)
    assert np.max(np.abs(v) / duv <= nxy // 2)
    return True


def get_image_size(u, v, PB=0, f_min=5., f_max=2.5, verbose=False):
    """Recommended (nxy, dxy) for the given (u, v) coverage (libcommon.pyx:291-361)."""
    uvdist = np.hypot(u, v)
    MRS = 0.6 / np.min(uvdist)
    duv = 1 / MRS / f_min
    max_uv = np.max(uvdist) * 2. * f_max
    nxy = int(2 ** np.ceil(np.log2(max_uv / duv)))
    nxy_MRS = nxy
    dxy = 1 / (nxy * duv)
    if PB != 0:
        while dxy * nxy / PB < 1.:
            nxy *= 2
    if verbose:
        print("dxy:{:e}arcsec\tnxy_MRS:{}".format(dxy / arcsec, nxy_MRS))
        print("nxy_MRS: matrix size to have FOV > f_min * MRS, where f_min:{} and MRS:{:e}arcsec".format(
            f_min, MRS / arcsec))
        if PB != 0:
            print("nxy_FOV:{}".format(nxy))
            print("nxy_FOV: matrix size to have FOV > PB")
    return nxy, dxy


def _cleanup_guard():
    pass


def make(precision: str) -> dict:
    """Build the namespace of one precision module ('double' or 'single')."""
    real = np.float64 if precision == "double" else np.float32
    cplx = np.complex128 if precision == "double" else np.complex64
    R = C.c_double if precision == "double" else C.c_float

    def call(name, *args):
        _lib.check(_lib.fn(name, precision)(*args))

    def _init():
        """Create the per-device context (galario init, src/galario.cpp:392-406)."""
        _lib.check(_lib.lib().galario_init())

    def _cleanup():
        """Release device buffers (galario cleanup, src/galario.cpp:408-428)."""
        _lib.check(_lib.lib().galario_cleanup())

    def ngpus():
        """Number of CUDA devices (libcommon.pyx:124-135)."""
        n = C.c_int(0)
        _lib.check(_lib.lib().galario_ngpus(C.byref(n)))
        return n.value

    def use_gpu(device_id):
        """Select the CUDA device for this thread (libcommon.pyx:138-159)."""
        _lib.check(_lib.lib().galario_use_gpu(int(device_id)))

    def threads(num=0):
        """Get/set the threads-per-block hint (libcommon.pyx:162-199); launch shapes are tuned internally."""
        return int(_lib.lib().galario_threads(int(num)))

    def get_coords_meshgrid(nrow, ncol, dxy=1., inc=0., Dx=0., Dy=0., origin='upper'):
        """(R.A., Dec.) pixel-centre meshgrid of the image (libcommon.pyx:731-797)."""
        v_origin = set_v_origin(origin)
        x = (np.linspace(0.5, -0.5 + 1. / float(ncol), ncol, dtype=real)) * ncol * dxy
        y = (np.linspace(0.5, -0.5 + 1. / float(nrow), nrow, dtype=real)) * nrow * dxy * v_origin
        x_m, y_m = np.meshgrid((x - Dx) / np.cos(inc), (y - Dy))
        R_m = np.hypot(x_m, y_m)
        return x, y, x_m, y_m, R_m

    # ---------------------------------------------------------------- user API
    def sampleImage(image, dxy, u, v, dRA=0., dDec=0., PA=0., check=False, origin='upper'):
        """Synthetic visibilities of an image at (u, v) (libcommon.pyx:371-443).

        image: (nxy, nxy) Jy/pixel; dxy, dRA, dDec, PA in rad; u, v in wavelengths.
        Returns complex visibilities in Jy.
        """
        image = _buffer(image, real, 2)
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        nxy = image.shape[0]
        duv = 1 / (dxy * nxy)
        if check:
            check_image_size(u, v, nxy, dxy, duv)
        vis = np.zeros(len(u), dtype=cplx)
        v_origin = set_v_origin(origin)
        _first(image)
        _first(u)
        _first(v)
        assert len(v) == len(u), "Wrong array length: v"
        call("sample_image", nxy, image.shape[1], _ptr(image), R(v_origin), R(dRA), R(dDec), R(duv), R(PA),
             len(u), _ptr(u), _ptr(v), _ptr(vis))
        return vis

    def sampleProfile(intensity, Rmin, dR, nxy, dxy, u, v, dRA=0., dDec=0., PA=0., inc=0., check=False):
        """Synthetic visibilities of an axisymmetric profile (libcommon.pyx:446-530).

        intensity in Jy/sr on R = Rmin + i*dR (rad); inc in rad.
        """
        intensity = _buffer(intensity, real, 1)
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        assert Rmin < dxy, \
            "For the interpolation of the image center, expect Rmin < dxy, but got Rmin={}, dxy={}".format(Rmin, dxy)
        duv = 1 / (dxy * nxy)
        if check:
            check_image_size(u, v, nxy, dxy, duv)
        vis = np.zeros(len(u), dtype=cplx)
        _first(intensity)
        _first(u)
        _first(v)
        assert len(v) == len(u), "Wrong array length: v"
        call("sample_profile", len(intensity), _ptr(intensity), R(Rmin), R(dR), R(dxy), int(nxy), R(inc), R(dRA),
             R(dDec), R(duv), R(PA), len(u), _ptr(u), _ptr(v), _ptr(vis))
        return vis

    def chi2Image(image, dxy, u, v, vis_obs_re, vis_obs_im, vis_obs_w, dRA=0., dDec=0., PA=0., check=False,
                  origin='upper'):
        """chi2 = sum w [(Re V_obs - Re V)^2 + (Im V_obs - Im V)^2] of an image (libcommon.pyx:533-626)."""
        image = _buffer(image, real, 2)
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        vis_obs_re = _buffer(vis_obs_re, real, 1)
        vis_obs_im = _buffer(vis_obs_im, real, 1)
        vis_obs_w = _buffer(vis_obs_w, real, 1)
        check_obs(vis_obs_re, vis_obs_im, vis_obs_w, u=u, v=v)
        nxy = image.shape[0]
        duv = 1 / (dxy * nxy)
        if check:
            check_image_size(u, v, nxy, dxy, duv)
        v_origin = set_v_origin(origin)
        for a in (image, u, v, vis_obs_re, vis_obs_im, vis_obs_w):
            _first(a)
        out = R(0)
        call("chi2_image", image.shape[0], image.shape[1], _ptr(image), R(v_origin), R(dRA), R(dDec), R(duv),
             R(PA), len(u), _ptr(u), _ptr(v), _ptr(vis_obs_re), _ptr(vis_obs_im), _ptr(vis_obs_w), C.byref(out))
        return float(out.value)

    def chi2Profile(intensity, Rmin, dR, nxy, dxy, u, v, vis_obs_re, vis_obs_im, vis_obs_w, dRA=0., dDec=0., PA=0.,
                    inc=0., check=False):
        """chi2 of an axisymmetric profile model (libcommon.pyx:629-728)."""
        intensity = _buffer(intensity, real, 1)
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        vis_obs_re = _buffer(vis_obs_re, real, 1)
        vis_obs_im = _buffer(vis_obs_im, real, 1)
        vis_obs_w = _buffer(vis_obs_w, real, 1)
        check_obs(vis_obs_re, vis_obs_im, vis_obs_w, u=u, v=v)
        assert Rmin < dxy, \
            "For the interpolation of the image center, expect Rmin < dxy, but got Rmin={}, dxy={}".format(Rmin, dxy)
        duv = 1 / (dxy * nxy)
        if check:
            check_image_size(u, v, nxy, dxy, duv)
        for a in (intensity, u, v, vis_obs_re, vis_obs_im, vis_obs_w):
            _first(a)
        out = R(0)
        call("chi2_profile", len(intensity), _ptr(intensity), R(Rmin), R(dR), R(dxy), int(nxy), R(inc), R(dRA),
             R(dDec), R(duv), R(PA), len(u), _ptr(u), _ptr(v), _ptr(vis_obs_re), _ptr(vis_obs_im),
             _ptr(vis_obs_w), C.byref(out))
        return float(out.value)

    # ---------------------------------------------------------- expert stages
    def sweep(intensity, Rmin, dR, nxy, dxy, inc=0.):
        """Image (nxy, nxy) in Jy/pixel from a radial profile (libcommon.pyx:800-848)."""
        intensity = _buffer(intensity, real, 1)
        assert Rmin < dxy, "For the interpolation algorithm, Rmin must be smaller than dxy. " \
                           "Currently Rmin={}\t dxy={}".format(Rmin, dxy)
        image = np.empty((nxy, nxy // 2 + 1), dtype=cplx, order='C')
        _first(intensity)
        call("sweep", len(intensity), _ptr(intensity), R(Rmin), R(dR), int(nxy), R(dxy), R(inc), _ptr(image))
        return np.ascontiguousarray(image.view(dtype=real)[:, :-2])

    def uv_rotate(PA, dRA, dDec, u, v):
        """(dRArot, dDecrot, urot, vrot) rotated by PA (libcommon.pyx:851-899)."""
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        nd = len(u)
        assert nd == len(v)
        a, b = R(0), R(0)
        urot = np.copy(u, order='C')
        vrot = np.copy(v, order='C')
        _first(u)
        call("uv_rotate", R(PA), R(dRA), R(dDec), C.byref(a), C.byref(b), nd, _ptr(u), _ptr(v), _ptr(urot),
             _ptr(vrot))
        return float(a.value), float(b.value), urot, vrot

    def interpolate(r2cFT, duv, u, v, origin='upper'):
        """Bilinear amp/phase interpolation of an R2C spectrum at (u, v) (libcommon.pyx:902-944)."""
        r2cFT = _buffer(r2cFT, cplx, 2)
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        vis = np.empty(len(u), dtype=cplx, order='C')
        v_origin = set_v_origin(origin)
        _first(r2cFT)
        _first(u)
        _first(v)
        call("interpolate", r2cFT.shape[0], r2cFT.shape[1], _ptr(r2cFT), R(v_origin), len(u), _ptr(u), _ptr(v),
             R(duv), _ptr(vis))
        return vis

    def apply_phase_vis(dRA, dDec, u, v, vis):
        """Visibilities translated by (dRA, dDec) in the image plane (libcommon.pyx:947-985)."""
        u = _buffer(u, real, 1)
        v = _buffer(v, real, 1)
        vis = _buffer(vis, cplx, 1)
        vis_out = np.copy(vis, order='C')
        _first(u)
        _first(v)
        _first(vis)
        call("apply_phase_sampled", R(dRA), R(dDec), len(vis), _ptr(u), _ptr(v), _ptr(vis_out))
        return vis_out

    def reduce_chi2(vis_obs_re, vis_obs_im, vis_obs_w, vis):
        """chi2 of observed vs model visibilities (libcommon.pyx:988-1021)."""
        vis_obs_re = _buffer(vis_obs_re, real, 1)
        vis_obs_im = _buffer(vis_obs_im, real, 1)
        vis_obs_w = _buffer(vis_obs_w, real, 1)
        vis = _buffer(vis, cplx, 1)
        check_obs(vis_obs_re, vis_obs_im, vis_obs_w, vis)
        for a in (vis_obs_re, vis_obs_im, vis_obs_w, vis):
            _first(a)
        out = R(0)
        call("reduce_chi2", len(vis), _ptr(vis_obs_re), _ptr(vis_obs_im), _ptr(vis), _ptr(vis_obs_w),
             C.byref(out))
        return float(out.value)

    def _fft2d(image):
        """2D R2C FFT: (nx, ny) reals -> (nx, ny//2+1) complex (libcommon.pyx:1024-1034)."""
        image = _buffer(image, real, 2)
        nx, ny = image.shape
        if nx < 2 or ny < 2 or nx != ny or nx % 2:
            call("fft2d", nx, ny, None)  # raises the reference's ValueError
        res = np.zeros((nx, ny // 2 + 1), dtype=cplx)
        res.view(real)[:, :ny] = image
        call("fft2d", nx, ny, _ptr(res))
        return res

    def _fftshift(matrix):
        """Quadrant swap, returned in the padded complex layout (libcommon.pyx:1037-1064)."""
        matrix = _buffer(matrix, real, 2)
        nx, ny = matrix.shape
        assert nx % 2 == 0 and ny % 2 == 0, "Expect even matrix size but got {}".format(matrix.shape)
        if nx < 2 or ny < 2 or nx != ny:
            call("fftshift", nx, ny, None)
        res = np.zeros((nx, ny // 2 + 1), dtype=cplx)
        res.view(real)[:, :ny] = matrix
        call("fftshift", nx, ny, _ptr(res))
        return res

    def _fftshift_axis0(matrix):
        """Swap upper and lower halves of a complex matrix, in place (libcommon.pyx:1067-1082)."""
        matrix = _buffer(matrix, cplx, 2)
        assert matrix.shape[0] % 2 == 0, "Axis 0 of `matrix` has to be even "
        _first(matrix)
        call("fftshift_axis0", matrix.shape[0], matrix.shape[1], _ptr(matrix))

    ns = dict(arcsec=arcsec, deg=deg, cgs_to_Jy=cgs_to_Jy, pc=pc, au=au,
              _init=_init, _cleanup=_cleanup, set_v_origin=set_v_origin,
              ngpus=ngpus, use_gpu=use_gpu, threads=threads,
              check_obs=check_obs, check_image_size=check_image_size, get_image_size=get_image_size,
              sampleImage=sampleImage, sampleProfile=sampleProfile, chi2Image=chi2Image, chi2Profile=chi2Profile,
              get_coords_meshgrid=get_coords_meshgrid,
              sweep=sweep, uv_rotate=uv_rotate, interpolate=interpolate, apply_phase_vis=apply_phase_vis,
              reduce_chi2=reduce_chi2, _fft2d=_fft2d, _fftshift=_fftshift, _fftshift_axis0=_fftshift_axis0,
              real_dtype=real, complex_dtype=cplx, __all__=list(__all__))
    return ns
