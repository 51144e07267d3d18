"""Host-pointer chi2Profile schedules against the oracle.

A host-pointer call (the reference's calling convention: plain numpy arrays,
re-uploaded every call, src/galario.cpp:1615-1656) runs one of three
schedules on the GPU:

- device reads host memory (GALARIO_ZERO_COPY unset, the device reports
  coherent pageable access) and every array is page-locked: the copy engines
  upload (u, v) and the first visibilities' observations, the visibility pass
  reads the rest of the observations in place;
- the same with a pageable array: the extent pass reads (u, v) from the
  caller's arrays and writes their device copies, a staging kernel copies
  the first observations;
- GALARIO_ZERO_COPY=0: chunked copy-engine uploads.

Each is compared with the FP64 oracle (double: relative 1e-12; single: 1e-6
against the oracle on the float32-rounded inputs) for sizes with and without
a staged head, odd lengths, and arrays that start 8 (4) bytes past a 16-byte
boundary (the staging kernels' scalar paths).
"""
import numpy as np
import pytest

from helpers import arcsec, deg, uv_log_uniform

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "single": 1e-6}


def _case(nd, seed):
    nxy, dxy, nr = 1024, 0.01 * arcsec, 2000
    Rmin, dR = 1e-4 * arcsec, 5e-4 * arcsec
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(nd, 1e4, 0.45 * nxy / 2 * duv, seed=seed)
    rng = np.random.default_rng(seed + 1)
    R = Rmin + dR * np.arange(nr)
    I = np.exp(-0.5 * ((R - 0.3 * arcsec) / (0.05 * arcsec)) ** 2) * 1e10
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    re, im = rng.normal(0, sigma), rng.normal(0, sigma)
    geo = dict(Rmin=Rmin, dR=dR, nxy=nxy, dxy=dxy)
    kw = dict(inc=30 * deg, PA=70 * deg, dRA=0.02 * arcsec, dDec=-0.01 * arcsec)
    return I, u, v, re, im, 1 / sigma ** 2, geo, kw


def _misaligned(a):
    """a copy of `a` whose data starts one element past a 64-byte boundary"""
    buf = np.empty(len(a) + 16, dtype=a.dtype)
    off = (-buf.ctypes.data % 64) // a.itemsize + 1
    out = buf[off:off + len(a)]
    out[:] = a
    assert out.ctypes.data % 16 != 0
    return out


def _pinned(torch, a):
    t = torch.empty(len(a), dtype=torch.float64 if a.dtype == np.float64 else torch.float32, pin_memory=True)
    arr = t.numpy()
    arr[:] = a
    return t, arr


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("nd", [1, 777, 4096, 300_001])
def test_chi2_profile_host_schedules(prec, nd, oracle_port, monkeypatch):
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    mod = g.double if prec == "double" else g.single
    np_t = np.float64 if prec == "double" else np.float32
    I, u, v, re, im, w, geo, kw = _case(nd, seed=nd % 97)
    arrs = [np.asarray(a, dtype=np_t) for a in (I, u, v, re, im, w)]
    f64 = [np.asarray(a, dtype=np.float64) for a in arrs]
    gf = {k: float(np_t(x)) for k, x in geo.items() if k != "nxy"}
    kwf = {k: float(np_t(x)) for k, x in kw.items()}
    orc = oracle_port.get("port", "double")
    ref = orc.chi2Profile(f64[0], gf["Rmin"], gf["dR"], geo["nxy"], gf["dxy"], *f64[1:], **kwf)
    keep = []
    pinned = []
    for a in arrs:
        t, arr = _pinned(torch, a)
        keep.append(t)
        pinned.append(arr)
    inputs = {"pageable": arrs, "pinned": pinned, "misaligned": [arrs[0]] + [_misaligned(a) for a in arrs[1:]],
              "mixed": [arrs[0], pinned[1], arrs[2], pinned[3], arrs[4], pinned[5]]}
    got = {}
    for zc in ("1", "0"):
        monkeypatch.setenv("GALARIO_ZERO_COPY", zc)
        for name, h in inputs.items():
            c = mod.chi2Profile(h[0], gf["Rmin"], gf["dR"], geo["nxy"], gf["dxy"], *h[1:], **kwf)
            got[(zc, name)] = c
            assert abs(c - ref) / ref <= TOL[prec], (zc, name, c, ref)
    # every schedule sums the same terms: they agree far below the tolerance
    vals = np.array(list(got.values()))
    assert (vals.max() - vals.min()) / ref <= (1e-13 if prec == "double" else 2e-7)
