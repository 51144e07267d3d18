"""The single-model device-resident entry points against the oracle.

galario_chi2_profile_device_{d,f} and galario_chi2_image_device_{d,f} take
inputs already in device memory (the reference re-uploads every input on
every call, src/galario.cpp:1279-1280,1584-1589), enqueue the work on the
caller's stream and write chi2 (double) to device memory.  Each is called
through the C ABI on torch-owned buffers and compared with the CPU oracle:
double within relative 1e-12, single within 1e-6 against the double oracle on
the same float32-rounded inputs.  Two calls in a row on one stream (the
second with other parameters) check that nothing of the first leaks into the
second; galario_device_status reports no device-side error.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import arcsec, deg, uv_log_uniform

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "single": 1e-6}


def _obs(nd, seed):
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    return rng.normal(0, sigma), rng.normal(0, sigma), 1. / sigma ** 2


def _ring(nr, Rmin, dR, r0, sig):
    R = Rmin + dR * np.arange(nr)
    return np.exp(-0.5 * ((R - r0 * arcsec) / (sig * arcsec)) ** 2) * 1e10


def _dev(torch, a, dt):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype=dt)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_chi2_profile_device(prec, oracle_port):
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    from galario_gb300 import _lib
    g.double.use_gpu(0)
    np_t = np.float64 if prec == "double" else np.float32
    t_t = torch.float64 if prec == "double" else torch.float32
    R = C.c_double if prec == "double" else C.c_float
    nxy, dxy, nd, nr = 1024, 0.01 * arcsec, 200_000, 2000
    Rmin, dR = 1e-4 * arcsec, 5e-4 * arcsec
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(nd, 1e4, 0.45 * nxy / 2 * duv, seed=11)
    nre, nim, w = _obs(nd, 12)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    fn = _lib.fn("chi2_profile_device", prec)
    orc = oracle_port.get("port", "double")
    f64 = lambda a: np.asarray(a, dtype=np.float64)  # noqa: E731
    for it, (r0, sig, inc, PA, dRA, dDec) in enumerate(((0.3, 0.05, 30 * deg, 70 * deg, 0.02, -0.01),
                                                        (0.6, 0.1, 55 * deg, 10 * deg, -0.03, 0.04))):
        I = np.asarray(_ring(nr, Rmin, dR, r0, sig), dtype=np_t)
        I_d = _dev(torch, I, t_t)
        geo = [np_t(x) for x in (Rmin, dR, dxy, inc, dRA * arcsec, dDec * arcsec, duv, PA)]
        # observations: the oracle's model of the same parameters plus noise
        # (chi2 near the noise level, as in a fit)
        model = orc.sampleProfile(f64(I), float(geo[0]), float(geo[1]), nxy, float(geo[2]), f64(np_t(u)),
                                  f64(np_t(v)), inc=float(geo[3]), dRA=float(geo[4]), dDec=float(geo[5]),
                                  PA=float(geo[7]))
        r = {k: np.asarray(x, dtype=np_t) for k, x in dict(u=u, v=v, re=model.real + nre, im=model.imag + nim,
                                                             w=w).items()}
        d = {k: _dev(torch, x, t_t) for k, x in r.items()}
        st = fn(nr, I.ctypes.data, I_d.data_ptr(), R(geo[0]), R(geo[1]), R(geo[2]), nxy, R(geo[3]), R(geo[4]),
                R(geo[5]), R(geo[6]), R(geo[7]), nd, d["u"].data_ptr(), d["v"].data_ptr(), d["re"].data_ptr(),
                d["im"].data_ptr(), d["w"].data_ptr(), out.data_ptr(), C.c_void_p(stream.cuda_stream))
        _lib.check(st)
        err = C.c_uint(99)
        _lib.check(_lib.lib().galario_device_status(C.byref(err)))
        assert err.value == 0
        got = float(out.item())
        ref = orc.chi2Profile(f64(I), float(geo[0]), float(geo[1]), nxy, float(geo[2]), f64(r["u"]), f64(r["v"]),
                              f64(r["re"]), f64(r["im"]), f64(r["w"]), inc=float(geo[3]), dRA=float(geo[4]),
                              dDec=float(geo[5]), PA=float(geo[7]))
        assert abs(got - ref) / ref <= TOL[prec], (prec, it, got, ref)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_chi2_image_device(prec, oracle_port):
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    from galario_gb300 import _lib
    g.double.use_gpu(0)
    np_t = np.float64 if prec == "double" else np.float32
    t_t = torch.float64 if prec == "double" else torch.float32
    R = C.c_double if prec == "double" else C.c_float
    nxy, dxy, nd = 1024, 0.01 * arcsec, 150_000
    duv = 1 / (nxy * dxy)
    x = (np.arange(nxy) - nxy / 2) * dxy
    rad = np.hypot(x[None, :], x[:, None])
    u, v = uv_log_uniform(nd, 1e4, 0.45 * nxy / 2 * duv, seed=21)
    nre, nim, w = _obs(nd, 22)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    fn = _lib.fn("chi2_image_device", prec)
    orc = oracle_port.get("port", "double")
    f64 = lambda a: np.asarray(a, dtype=np.float64)  # noqa: E731
    for it, (r0, sig, vo, PA, dRA, dDec) in enumerate(((0.3, 0.05, 1.0, 25 * deg, 0.02, -0.01),
                                                       (0.8, 0.1, -1.0, 140 * deg, -0.03, 0.04))):
        img = np.exp(-0.5 * ((rad - r0 * arcsec) / (sig * arcsec)) ** 2)
        img = np.asarray(img * (0.1 / img.sum()), dtype=np_t)
        img_d = _dev(torch, img, t_t)
        geo = [np_t(x) for x in (dRA * arcsec, dDec * arcsec, duv, PA)]
        origin = "upper" if vo > 0 else "lower"
        model = orc.sampleImage(f64(img), float(np_t(dxy)), f64(np_t(u)), f64(np_t(v)), dRA=float(geo[0]),
                                dDec=float(geo[1]), PA=float(geo[3]), origin=origin)
        r = {k: np.asarray(a, dtype=np_t) for k, a in dict(u=u, v=v, re=model.real + nre, im=model.imag + nim,
                                                             w=w).items()}
        d = {k: _dev(torch, a, t_t) for k, a in r.items()}
        st = fn(nxy, nxy, img_d.data_ptr(), R(vo), R(geo[0]), R(geo[1]), R(geo[2]), R(geo[3]), nd,
                d["u"].data_ptr(), d["v"].data_ptr(), d["re"].data_ptr(), d["im"].data_ptr(), d["w"].data_ptr(),
                out.data_ptr(), C.c_void_p(stream.cuda_stream))
        _lib.check(st)
        err = C.c_uint(99)
        _lib.check(_lib.lib().galario_device_status(C.byref(err)))
        assert err.value == 0
        got = float(out.item())
        ref = orc.chi2Image(f64(img), float(np_t(dxy)), f64(r["u"]), f64(r["v"]), f64(r["re"]), f64(r["im"]),
                            f64(r["w"]), dRA=float(geo[0]), dDec=float(geo[1]), PA=float(geo[3]),
                            origin=origin)
        assert abs(got - ref) / ref <= TOL[prec], (prec, it, got, ref)
