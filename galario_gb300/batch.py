"""Batched FP32 chi2 (and its gradient) of many profile models on the GPU.

New surface beside the reference's API (the reference evaluates one model per
call and has no gradient): a device-resident ``Dataset`` and
``chi2_profile_batch``, which evaluates B radial-profile models (shared radial
grid, per-model inclination, position angle and offsets) against one dataset
in one set of launches, optionally with the gradient of every chi2 with
respect to the profile samples and to (inc, PA, dRA, dDec).

Arrays are torch CUDA tensors (float32); chi2 comes back as float64.  Units
as in galario: radians for Rmin, dR, dxy, inc, PA, dRA, dDec; wavelengths for
u, v; Jy/sr for the intensity.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_P = C.c_void_p
_F = C.c_float
_I = C.c_int


def _bind():
    L = _lib.lib()
    if not getattr(L, "_gb_batch_bound", False):
        L.galario_dataset_create_f.argtypes = [_I, _P, _P, _P, _P, _P, _I, C.POINTER(_P)]
        L.galario_dataset_free.argtypes = [_P]
        L.galario_dataset_nvis.argtypes = [_P, C.POINTER(_I)]
        L.galario_chi2_profile_batch_f.argtypes = [_P, _I, _I, _P, _F, _F, _F, _I, _P, _P, _P, _P, _P]
        for n in ("galario_dataset_create_f", "galario_dataset_free", "galario_dataset_nvis",
                  "galario_chi2_profile_batch_f"):
            getattr(L, n).restype = _I
        L._gb_batch_bound = True
    return L


class Dataset:
    """Observed visibilities resident on the current GPU (float32 copies).

    u, v [wavelengths], re, im [Jy], w [1/Jy^2]: numpy arrays or torch tensors
    (CPU or CUDA).  The maximum |uv| is computed once here, so the spectrum
    window of every later call is known without a device round trip.
    """

    def __init__(self, u, v, re, im, w):
        import torch
        arrs = []
        for a in (u, v, re, im, w):
            t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
            t = t.to(device="cuda", dtype=torch.float32).contiguous()
            arrs.append(t)
        n = arrs[0].numel()
        if any(t.numel() != n for t in arrs):
            raise AssertionError("Wrong array length: u, v, re, im, w must have the same length")
        L = _bind()
        h = _P()
        torch.cuda.synchronize()
        _lib.check(L.galario_dataset_create_f(n, *(t.data_ptr() for t in arrs), 1, C.byref(h)))
        self._h = h
        self.nd = n

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.check(_bind().galario_dataset_free(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def chi2_profile_batch(dataset: Dataset, intensity, params, Rmin, dR, dxy, nxy, grad=False):
    """chi2 of B profile models against ``dataset``.

    intensity: (B, nr) float32 CUDA tensor [Jy/sr] on R = Rmin + i dR;
    params: (B, 4) float32 CUDA tensor of (inc, PA, dRA, dDec) [rad].
    Returns chi2 (B,) float64, and with grad=True also dchi2/dintensity (B, nr)
    and dchi2/dparams (B, 4), both float32.
    """
    import torch
    intensity = intensity.to(dtype=torch.float32).contiguous()
    params = params.to(dtype=torch.float32).contiguous()
    if intensity.dim() != 2 or params.dim() != 2 or params.shape[1] != 4 or params.shape[0] != intensity.shape[0]:
        raise ValueError("intensity must be (B, nr) and params (B, 4)")
    if not (intensity.is_cuda and params.is_cuda):
        raise ValueError("intensity and params must be CUDA tensors")
    assert Rmin < dxy, \
        "For the interpolation of the image center, expect Rmin < dxy, but got Rmin={}, dxy={}".format(Rmin, dxy)
    B, nr = intensity.shape
    dev = intensity.device
    chi2 = torch.empty(B, dtype=torch.float64, device=dev)
    gI = torch.empty_like(intensity) if grad else None
    gp = torch.empty_like(params) if grad else None
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = _bind()
    _lib.check(L.galario_chi2_profile_batch_f(dataset.handle, B, nr, intensity.data_ptr(), _F(Rmin), _F(dR),
                                              _F(dxy), int(nxy), params.data_ptr(), chi2.data_ptr(),
                                              gI.data_ptr() if grad else None, gp.data_ptr() if grad else None,
                                              _P(stream)))
    return (chi2, gI, gp) if grad else chi2
