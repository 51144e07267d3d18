"""CPU oracle for the galario synthetic-visibility / chi2 path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, as the checker or as the
timed CPU baseline.  The GPU product (``galario_gb300``) never does.

Two interchangeable back ends expose the same numpy-level API, which mirrors
the argument handling of the reference's Cython layer
(``python/libcommon.pyx:371-728``, ``:800-1082``):

* ``port``: ``oracle/_build/liboracle.so``, the plain-C restatement of the
  reference CPU path (``oracle/galario_oracle.c``), built anywhere;
* ``ref``: ``oracle/_ref/libgalario_ref_{double,single}.so``, the reference's
  own ``src/galario.cpp`` compiled unchanged against the project's FFTW-API
  shim (``oracle/shim``).  It exists only where the reference sources were
  present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = {"double": os.path.join(HERE, "_ref", "libgalario_ref_double.so"),
          "single": os.path.join(HERE, "_ref", "libgalario_ref_single.so")}

_VALUE_ERROR, _MEMORY_ERROR = 1, 2


def build_port() -> str:
    """Compile the C restatement (fast, no reference sources needed)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def have_ref() -> bool:
    return all(os.path.exists(p) for p in REF_SO.values())


class OracleError(RuntimeError):
    pass


class _Oracle:
    """numpy front end over one precision of one back end."""

    def __init__(self, kind: str, precision: str):
        assert kind in ("port", "ref") and precision in ("double", "single")
        self.kind, self.precision = kind, precision
        self.real = np.float64 if precision == "double" else np.float32
        self.cplx = np.complex128 if precision == "double" else np.complex64
        ct = C.c_double if precision == "double" else C.c_float
        self._ct = ct
        if kind == "port":
            if not os.path.exists(PORT_SO):
                build_port()
            self._lib = C.CDLL(PORT_SO)
            sfx = "_d" if precision == "double" else "_f"
            self._fn = lambda name: getattr(self._lib, "orc_" + name + sfx)
            self._err = self._lib.orc_last_error
            self._threads = self._lib.orc_threads
        else:
            self._lib = C.CDLL(REF_SO[precision])
            self._fn = lambda name: getattr(self._lib, "ref_" + name)
            self._err = self._lib.ref_last_error
            self._threads = self._lib.ref_threads
            self._lib.ref_init()
        self._err.restype = C.c_char_p
        self._threads.argtypes = [C.c_int]
        self._threads.restype = C.c_int

    # -- plumbing ---------------------------------------------------------
    def _call(self, name, *args):
        conv = []
        for a in args:
            if isinstance(a, np.ndarray):
                conv.append(C.c_void_p(a.ctypes.data))
            elif isinstance(a, bool):
                conv.append(C.c_int(int(a)))
            elif isinstance(a, (int, np.integer)):
                conv.append(C.c_int(int(a)))
            elif isinstance(a, (float, np.floating)):
                conv.append(self._ct(float(a)))
            else:
                conv.append(a)
        st = self._fn(name)(*conv)
        if st != 0:
            msg = self._err().decode()
            if st == _VALUE_ERROR:
                raise ValueError(msg)
            if st == _MEMORY_ERROR:
                raise MemoryError(msg)
            raise OracleError(msg)

    def _arr(self, x, dtype=None):
        return np.ascontiguousarray(x, dtype=dtype or self.real)

    def threads(self, num: int = 0) -> int:
        return self._threads(int(num))

    @staticmethod
    def _v_origin(origin):
        if origin == "upper":
            return 1.0
        if origin == "lower":
            return -1.0
        raise AssertionError("Expect origin='upper' or 'lower', got {}".format(origin))

    # -- the four user functions (libcommon.pyx:371-728) -------------------
    def sampleImage(self, image, dxy, u, v, dRA=0., dDec=0., PA=0., origin="upper"):
        image, u, v = self._arr(image), self._arr(u), self._arr(v)
        nxy = image.shape[0]
        duv = 1. / (dxy * nxy)
        vis = np.zeros(len(u), dtype=self.cplx)
        self._call("sample_image", nxy, nxy, image, self._v_origin(origin), dRA, dDec, duv, PA, len(u), u, v, vis)
        return vis

    def sampleProfile(self, intensity, Rmin, dR, nxy, dxy, u, v, dRA=0., dDec=0., PA=0., inc=0.):
        intensity, u, v = self._arr(intensity), self._arr(u), self._arr(v)
        duv = 1. / (dxy * nxy)
        vis = np.zeros(len(u), dtype=self.cplx)
        self._call("sample_profile", len(intensity), intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA,
                   len(u), u, v, vis)
        return vis

    def chi2Image(self, image, dxy, u, v, re, im, w, dRA=0., dDec=0., PA=0., origin="upper"):
        image, u, v = self._arr(image), self._arr(u), self._arr(v)
        re, im, w = self._arr(re), self._arr(im), self._arr(w)
        nxy = image.shape[0]
        duv = 1. / (dxy * nxy)
        out = np.zeros(1, dtype=self.real)
        self._call("chi2_image", image.shape[0], image.shape[1], image, self._v_origin(origin), dRA, dDec, duv, PA,
                   len(u), u, v, re, im, w, out)
        return float(out[0])

    def chi2Profile(self, intensity, Rmin, dR, nxy, dxy, u, v, re, im, w, dRA=0., dDec=0., PA=0., inc=0.):
        intensity, u, v = self._arr(intensity), self._arr(u), self._arr(v)
        re, im, w = self._arr(re), self._arr(im), self._arr(w)
        duv = 1. / (dxy * nxy)
        out = np.zeros(1, dtype=self.real)
        self._call("chi2_profile", len(intensity), intensity, Rmin, dR, dxy, nxy, inc, dRA, dDec, duv, PA,
                   len(u), u, v, re, im, w, out)
        return float(out[0])

    # -- expert stages (libcommon.pyx:800-1082) ----------------------------
    def sweep(self, intensity, Rmin, dR, nxy, dxy, inc=0.):
        intensity = self._arr(intensity)
        buf = np.empty((nxy, nxy // 2 + 1), dtype=self.cplx)
        self._call("sweep", len(intensity), intensity, Rmin, dR, nxy, dxy, inc, buf)
        return np.ascontiguousarray(buf.view(self.real)[:, :-2])

    def uv_rotate(self, PA, dRA, dDec, u, v):
        u, v = self._arr(u), self._arr(v)
        urot, vrot = u.copy(), v.copy()
        a, b = np.zeros(1, self.real), np.zeros(1, self.real)
        self._call("uv_rotate_api" if self.kind == "port" else "uv_rotate", PA, dRA, dDec, a, b, len(u), u, v,
                   urot, vrot)
        return float(a[0]), float(b[0]), urot, vrot

    def interpolate(self, r2cFT, duv, u, v, origin="upper"):
        ft = np.ascontiguousarray(r2cFT, dtype=self.cplx)
        u, v = self._arr(u), self._arr(v)
        vis = np.empty(len(u), dtype=self.cplx)
        self._call("interpolate_api" if self.kind == "port" else "interpolate", ft.shape[0], ft.shape[1], ft,
                   self._v_origin(origin), len(u), u, v, duv, vis)
        return vis

    def apply_phase_vis(self, dRA, dDec, u, v, vis):
        u, v = self._arr(u), self._arr(v)
        out = np.array(vis, dtype=self.cplx, copy=True, order="C")
        self._call("apply_phase_api" if self.kind == "port" else "apply_phase", dRA, dDec, len(out), u, v, out)
        return out

    def reduce_chi2(self, re, im, w, vis):
        re, im, w = self._arr(re), self._arr(im), self._arr(w)
        vis = np.ascontiguousarray(vis, dtype=self.cplx)
        out = np.zeros(1, dtype=self.real)
        self._call("reduce_chi2", len(vis), re, im, vis, w, out)
        return float(out[0])

    def _fft2d(self, image):
        image = self._arr(image)
        nx, ny = image.shape
        if self.kind == "ref":
            out = np.empty((nx, ny // 2 + 1), dtype=self.cplx)
            self._call("fft2d", nx, ny, image, out)
            return out
        buf = np.zeros((nx, ny // 2 + 1), dtype=self.cplx)
        buf.view(self.real)[:, :ny] = image
        self._call("fft2d", nx, ny, buf)
        return buf

    def _fftshift(self, image):
        image = self._arr(image)
        nx, ny = image.shape
        if self.kind == "ref":
            out = np.empty((nx, ny // 2 + 1), dtype=self.cplx)
            self._call("fftshift", nx, ny, image, out)
            return out
        buf = np.zeros((nx, ny // 2 + 1), dtype=self.cplx)
        buf.view(self.real)[:, :ny] = image
        self._call("fftshift", nx, ny, buf)
        return buf

    def _fftshift_axis0(self, matrix):
        """In place, as the reference (libcommon.pyx:1067-1082)."""
        assert matrix.dtype == self.cplx and matrix.flags.c_contiguous
        self._call("fftshift_axis0", matrix.shape[0], matrix.shape[1], matrix)


_cache: dict = {}


def get(kind: str = "port", precision: str = "double") -> _Oracle:
    key = (kind, precision)
    if key not in _cache:
        _cache[key] = _Oracle(kind, precision)
    return _cache[key]
