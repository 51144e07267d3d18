"""ctypes binding of libgalario_gb300.so (the C ABI declared in include/galario_gb300.h).

The library is loaded lazily on first use.  There is no CPU fallback: if the
library is missing or no CUDA device is usable, every compute call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgalario_gb300.so")

OK, EINVAL, ENOMEM, ERUNTIME = 0, 1, 2, 3

_lock = threading.Lock()
_lib = None

_p = C.c_void_p
_i = C.c_int
_d = C.c_double
_f = C.c_float


def _protos(R):
    """argtypes of the precision-specific entry points, R = c_double / c_float."""
    return {
        "sample_image": [_i, _i, _p, R, R, R, R, R, _i, _p, _p, _p],
        "chi2_image": [_i, _i, _p, R, R, R, R, R, _i, _p, _p, _p, _p, _p, _p],
        "sample_profile": [_i, _p, R, R, R, _i, R, R, R, R, R, _i, _p, _p, _p],
        "chi2_profile": [_i, _p, R, R, R, _i, R, R, R, R, R, _i, _p, _p, _p, _p, _p, _p],
        "chi2_profile_device": [_i, _p, _p, R, R, R, _i, R, R, R, R, R, _i, _p, _p, _p, _p, _p, _p, _p],
        "chi2_image_device": [_i, _i, _p, R, R, R, R, R, _i, _p, _p, _p, _p, _p, _p, _p],
        "sweep": [_i, _p, R, R, _i, R, R, _p],
        "uv_rotate": [R, R, R, _p, _p, _i, _p, _p, _p, _p],
        "interpolate": [_i, _i, _p, R, _i, _p, _p, R, _p],
        "apply_phase_sampled": [R, R, _i, _p, _p, _p],
        "reduce_chi2": [_i, _p, _p, _p, _p, _p],
        "fft2d": [_i, _i, _p],
        "fftshift": [_i, _i, _p],
        "fftshift_axis0": [_i, _i, _p],
    }


def lib() -> C.CDLL:
    """Load the library (once) and declare every prototype."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "galario_gb300: the CUDA library %s is not built; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` (or python -m galario_gb300._build)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for sfx, R in (("_d", _d), ("_f", _f)):
            for name, args in _protos(R).items():
                fn = getattr(L, "galario_" + name + sfx)
                fn.argtypes = args
                fn.restype = _i
        L.galario_last_error.restype = C.c_char_p
        L.galario_last_error.argtypes = []
        L.galario_version.restype = C.c_char_p
        L.galario_threads.argtypes = [_i]
        L.galario_threads.restype = _i
        L.galario_ngpus.argtypes = [C.POINTER(_i)]
        L.galario_use_gpu.argtypes = [_i]
        L.galario_init.argtypes = []
        L.galario_cleanup.argtypes = []
        L.galario_device_status.argtypes = [C.POINTER(C.c_uint)]
        L.galario_stage_timing.argtypes = [_i]
        L.galario_stage_name.argtypes = [_i]
        L.galario_stage_name.restype = C.c_char_p
        L.galario_stage_times.argtypes = [C.POINTER(C.c_double), C.POINTER(_i), _i]
        L.galario_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
        for n in ("galario_ngpus", "galario_use_gpu", "galario_init", "galario_cleanup", "galario_device_status",
                  "galario_stage_timing", "galario_stage_times", "galario_measure_fp64_peak"):
            getattr(L, n).restype = _i
        _lib = L
        return L


def check(status: int) -> None:
    """Raise the Python exception the reference's Cython layer would raise."""
    if status == OK:
        return
    msg = lib().galario_last_error().decode(errors="replace")
    if status == EINVAL:
        raise ValueError(msg)
    if status == ENOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def fn(name: str, precision: str):
    return getattr(lib(), "galario_" + name + ("_d" if precision == "double" else "_f"))
