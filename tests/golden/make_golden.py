"""Generate the golden fixtures in tests/golden/ from the reference itself.

The outputs come from the reference's own CPU code (galario 1.2.2
src/galario.cpp, compiled unchanged into oracle/_ref/ against the project's
FFTW-API shim: ``make -C oracle ref``).  Inputs are seeded and small so the
fixtures stay a few hundred KB.  Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from helpers import arcsec, deg, reference_image, uv_log_uniform  # noqa: E402


def gen(precision: str) -> dict:
    ref = O.get("ref", precision)
    real = ref.real
    out = {}
    rng = np.random.default_rng(2024)

    # --- FFT (reference _copy_input + _fft2d) ---
    for n in (8, 12, 64):
        img = rng.standard_normal((n, n)).astype(real)
        out["fft%d_in" % n] = img
        out["fft%d_out" % n] = ref._fft2d(img)

    # --- sampleImage / chi2Image ---
    nxy, dxy = 64, 0.05 * arcsec
    duv = 1. / (nxy * dxy)
    img = reference_image(nxy, x0=3., y0=-2., sigma_x=40., sigma_y=25.).astype(real)
    nd = 300
    u, v = uv_log_uniform(nd, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=11)
    u, v = u.astype(real), v.astype(real)
    sig = rng.uniform(0.5, 1.5, nd)
    re = rng.normal(0, sig).astype(real)
    im = rng.normal(0, sig).astype(real)
    w = (1. / sig ** 2).astype(real)
    out.update(img_image=img, img_u=u, img_v=v, img_re=re, img_im=im, img_w=w,
               img_dxy=np.array(dxy))
    cases = [dict(dRA=0., dDec=0., PA=0., origin="upper"),
             dict(dRA=0.3 * arcsec, dDec=-0.2 * arcsec, PA=0.6, origin="upper"),
             dict(dRA=-0.1 * arcsec, dDec=0.4 * arcsec, PA=2.2, origin="lower")]
    for i, kw in enumerate(cases):
        out["img_case%d_params" % i] = np.array([kw["dRA"], kw["dDec"], kw["PA"], 1. if kw["origin"] == "upper" else -1.])
        out["img_case%d_vis" % i] = ref.sampleImage(img, dxy, u, v, **kw)
        out["img_case%d_chi2" % i] = np.array(ref.chi2Image(img, dxy, u, v, re, im, w, **kw))

    # --- sampleProfile / chi2Profile / sweep ---
    nxy_p, dxy_p = 128, 0.02 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 1.5e-3 * arcsec, 600
    R = Rmin + dR * np.arange(nr)
    I = (np.exp(-0.5 * ((R - 0.3 * arcsec) / (0.05 * arcsec)) ** 2) +
         0.4 * np.exp(-0.5 * ((R - 0.6 * arcsec) / (0.08 * arcsec)) ** 2)) * 1e10
    I = I.astype(real)
    duv_p = 1. / (nxy_p * dxy_p)
    up, vp = uv_log_uniform(nd, 0.5 * duv_p, 0.45 * nxy_p / 2 * duv_p, seed=12)
    up, vp = up.astype(real), vp.astype(real)
    out.update(pro_I=I, pro_u=up, pro_v=vp, pro_scalars=np.array([Rmin, dR, dxy_p, nxy_p]))
    pcases = [dict(inc=0., PA=0., dRA=0., dDec=0.),
              dict(inc=40 * deg, PA=70 * deg, dRA=0.02 * arcsec, dDec=-0.04 * arcsec)]
    for i, kw in enumerate(pcases):
        out["pro_case%d_params" % i] = np.array([kw["inc"], kw["PA"], kw["dRA"], kw["dDec"]])
        out["pro_case%d_vis" % i] = ref.sampleProfile(I, Rmin, dR, nxy_p, dxy_p, up, vp, **kw)
        out["pro_case%d_chi2" % i] = np.array(ref.chi2Profile(I, Rmin, dR, nxy_p, dxy_p, up, vp, re, im, w, **kw))
    out["sweep_out"] = ref.sweep(I, Rmin, dR, 48, dxy_p * 3, 30 * deg)
    out["sweep_scalars"] = np.array([Rmin, dR, 48, dxy_p * 3, 30 * deg])

    # --- expert stages ---
    dra, ddec, urot, vrot = ref.uv_rotate(0.8, 0.3 * arcsec, -0.2 * arcsec, u, v)
    out.update(rot_out=np.array([dra, ddec]), rot_urot=urot, rot_vrot=vrot)
    spec = np.ascontiguousarray(np.fft.fftshift(np.fft.rfft2(np.fft.fftshift(img.astype(np.float64))), axes=0)
                                .astype(ref.cplx))
    out["interp_spec"] = spec
    out["interp_upper"] = ref.interpolate(spec, duv, u, v, origin="upper")
    out["interp_lower"] = ref.interpolate(spec, duv, u, v, origin="lower")
    vis0 = (rng.standard_normal(nd) + 1j * rng.standard_normal(nd)).astype(ref.cplx)
    out["phase_in"] = vis0
    out["phase_out"] = ref.apply_phase_vis(0.3 * arcsec, -0.2 * arcsec, u, v, vis0)
    out["chi2_reduce"] = np.array(ref.reduce_chi2(re, im, w, vis0))
    return out


def main():
    if not O.have_ref():
        raise SystemExit("oracle/_ref is not built: run `make -C oracle ref` first (needs the reference sources)")
    for prec in ("double", "single"):
        O.get("ref", prec).threads(1)  # deterministic chi2 summation order
        data = gen(prec)
        path = os.path.join(HERE, "golden_%s.npz" % prec)
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path), "bytes,", len(data), "arrays")


if __name__ == "__main__":
    main()
