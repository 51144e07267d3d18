"""Batched FP32 chi2 (and its gradient) of many models on the GPU.

New surface beside the reference's API (the reference evaluates one model per
call and has no gradient): a device-resident ``Dataset``;
``chi2_profile_batch``, which evaluates B radial-profile models (shared radial
grid, per-model inclination, position angle and offsets) against one dataset
in one set of launches, optionally with the gradient of every chi2 with
respect to the profile samples and to (inc, PA, dRA, dDec); and
``chi2_image_batch``, the same for B free-form images with the gradient with
respect to every pixel and to (PA, dRA, dDec).

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
        L.galario_dataset_create_f.argtypes = [_I, _P, _P, _P, _P, _P, _I, _P, _I, C.POINTER(_P)]
        L.galario_dataset_free.argtypes = [_P]
        L.galario_dataset_nvis.argtypes = [_P, C.POINTER(_I)]
        L.galario_dataset_nsets.argtypes = [_P, C.POINTER(_I)]
        L.galario_batch_status.argtypes = [C.POINTER(C.c_uint)]
        L.galario_chi2_profile_batch_f.argtypes = [_P, _I, _I, _P, _F, _F, _F, _I, _P, _P, _P, _P, _P, _P]
        L.galario_chi2_image_batch_f.argtypes = [_P, _I, _I, _P, _F, _F, _P, _P, _P, _P, _P, _P]
        for n in ("galario_dataset_create_f", "galario_dataset_free", "galario_dataset_nvis",
                  "galario_dataset_nsets", "galario_chi2_profile_batch_f", "galario_chi2_image_batch_f",
                  "galario_batch_status"):
            getattr(L, n).restype = _I
        L._gb_batch_bound = True
    return L


def status() -> int:
    """Synchronise the device and return the error bits of the last batched call (0: none)."""
    e = C.c_uint(0)
    _lib.check(_bind().galario_batch_status(C.byref(e)))
    return int(e.value)


class Dataset:
    """Observed visibilities resident on the current GPU (float32 copies).

    u, v [wavelengths], re, im [Jy], w [1/Jy^2]: numpy arrays or torch tensors
    (CPU or CUDA), or lists of them, one entry per visibility set (for example
    one per spectral window or per observation; the sets may differ in
    length).  chi2 is additive over the sets: ``chi2_profile_batch`` returns
    the total, or with ``per_set=True`` one chi2 per set.  The maximum |uv|
    over all sets is computed once here, so the spectrum window of every later
    call is known without a device round trip.
    """

    def __init__(self, u, v, re, im, w):
        import torch
        cols = [u, v, re, im, w]
        if isinstance(u, (list, tuple)):
            nsets = len(u)
            if nsets == 0 or any(not isinstance(c, (list, tuple)) or len(c) != nsets for c in cols):
                raise ValueError("u, v, re, im, w must be lists of the same length (one entry per set)")
        else:
            nsets = 1
            cols = [[c] for c in cols]

        def flat(parts):
            ts = [p if isinstance(p, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(p)) for p in parts]
            ts = [t.reshape(-1).to(device="cuda", dtype=torch.float32) for t in ts]
            return ts
        per = [flat(c) for c in cols]
        lengths = [t.numel() for t in per[0]]
        for c in per:
            if [t.numel() for t in c] != lengths:
                raise AssertionError("Wrong array length: u, v, re, im, w must have the same length")
        arrs = [torch.cat(c).contiguous() for c in per]
        n = arrs[0].numel()
        offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int32)
        L = _bind()
        h = _P()
        torch.cuda.synchronize()
        _lib.check(L.galario_dataset_create_f(n, *(t.data_ptr() for t in arrs), nsets,
                                              offsets.ctypes.data_as(_P), 1, C.byref(h)))
        self._h = h
        self.nd = n
        self.nsets = nsets
        self.nvis_per_set = lengths

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


def chi2_profile_batch(dataset: Dataset, intensity, params, Rmin, dR, dxy, nxy, grad=False, per_set=False):
    """chi2 of B profile models against ``dataset``.

    intensity: (B, nr) float32 CUDA tensor [Jy/sr] on R = Rmin + i dR;
    params: (B, 4) float32 CUDA tensor of (inc, PA, dRA, dDec) [rad];
    nxy: even, in [16, 16384]; a power of two unless the spectrum passes run
    on the tensor cores (the default where the folded quadrant rmax + 1, the
    uv window and the profile fit them).
    Returns chi2 float64, (B,) summed over the dataset's sets or (B, nsets)
    with per_set=True; with grad=True also dchi2/dintensity (B, nr) and
    dchi2/dparams (B, 4) of the total chi2, both float32.
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
    sets = torch.empty((B, dataset.nsets), dtype=torch.float64, device=dev) if per_set else None
    gI = torch.empty_like(intensity) if grad else None
    gp = torch.empty_like(params) if grad else None
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = _bind()
    _lib.check(L.galario_chi2_profile_batch_f(dataset.handle, B, nr, intensity.data_ptr(), _F(Rmin), _F(dR),
                                              _F(dxy), int(nxy), params.data_ptr(), chi2.data_ptr(),
                                              sets.data_ptr() if per_set else None,
                                              gI.data_ptr() if grad else None, gp.data_ptr() if grad else None,
                                              _P(stream)))
    out = sets if per_set else chi2
    return (out, gI, gp) if grad else out


def chi2_image_batch(dataset: Dataset, images, params, dxy, origin="upper", grad=False, per_set=False):
    """chi2 of B images against ``dataset`` (chi2Image semantics per image).

    images: (B, nxy, nxy) float32 CUDA tensor [Jy/pixel], nxy a power of two;
    params: (B, 3) float32 CUDA tensor of (PA, dRA, dDec) [rad];
    origin: 'upper' or 'lower', as chi2Image.  Returns chi2 float64, (B,) or
    (B, nsets) with per_set=True; with grad=True also dchi2/dimages
    (B, nxy, nxy) and dchi2/dparams (B, 3), both float32.
    """
    import torch
    if origin == "upper":
        v_origin = 1.0
    elif origin == "lower":
        v_origin = -1.0
    else:
        raise AssertionError("origin must be 'upper' or 'lower', not {}".format(origin))
    images = images.to(dtype=torch.float32).contiguous()
    params = params.to(dtype=torch.float32).contiguous()
    if images.dim() != 3 or images.shape[1] != images.shape[2]:
        raise ValueError("images must be (B, nxy, nxy)")
    if params.dim() != 2 or params.shape != (images.shape[0], 3):
        raise ValueError("params must be (B, 3): PA, dRA, dDec")
    if not (images.is_cuda and params.is_cuda):
        raise ValueError("images and params must be CUDA tensors")
    B, nxy = images.shape[0], images.shape[1]
    dev = images.device
    chi2 = torch.empty(B, dtype=torch.float64, device=dev)
    sets = torch.empty((B, dataset.nsets), dtype=torch.float64, device=dev) if per_set else None
    gI = torch.empty_like(images) if grad else None
    gp = torch.empty_like(params) if grad else None
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = _bind()
    _lib.check(L.galario_chi2_image_batch_f(dataset.handle, B, nxy, images.data_ptr(), _F(dxy), _F(v_origin),
                                            params.data_ptr(), chi2.data_ptr(),
                                            sets.data_ptr() if per_set else None,
                                            gI.data_ptr() if grad else None, gp.data_ptr() if grad else None,
                                            _P(stream)))
    out = sets if per_set else chi2
    return (out, gI, gp) if grad else out
