"""Replays the golden fixtures (tests/golden/golden_*.npz, produced by the
reference's own CPU code) against any implementation with the galario module
API (the oracle port, or galario_gb300 on the GPU)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(precision):
    return dict(np.load(os.path.join(HERE, "golden", "golden_%s.npz" % precision)))


def run_all(impl, d):
    """Yield (name, computed, expected) for every golden case."""
    for n in (8, 12, 64):
        yield "fft%d" % n, impl._fft2d(d["fft%d_in" % n]), d["fft%d_out" % n]
    img, u, v = d["img_image"], d["img_u"], d["img_v"]
    re, im, w = d["img_re"], d["img_im"], d["img_w"]
    dxy = float(d["img_dxy"])
    for i in range(3):
        dRA, dDec, PA, vo = d["img_case%d_params" % i]
        origin = "upper" if vo > 0 else "lower"
        kw = dict(dRA=float(dRA), dDec=float(dDec), PA=float(PA), origin=origin)
        yield "sampleImage%d" % i, impl.sampleImage(img, dxy, u, v, **kw), d["img_case%d_vis" % i]
        yield "chi2Image%d" % i, np.array(impl.chi2Image(img, dxy, u, v, re, im, w, **kw)), d["img_case%d_chi2" % i]
    I, up, vp = d["pro_I"], d["pro_u"], d["pro_v"]
    Rmin, dR, dxy_p, nxy_p = d["pro_scalars"]
    nxy_p = int(nxy_p)
    for i in range(2):
        inc, PA, dRA, dDec = (float(x) for x in d["pro_case%d_params" % i])
        kw = dict(inc=inc, PA=PA, dRA=dRA, dDec=dDec)
        yield ("sampleProfile%d" % i, impl.sampleProfile(I, float(Rmin), float(dR), nxy_p, float(dxy_p), up, vp, **kw),
               d["pro_case%d_vis" % i])
        yield ("chi2Profile%d" % i,
               np.array(impl.chi2Profile(I, float(Rmin), float(dR), nxy_p, float(dxy_p), up, vp, re, im, w, **kw)),
               d["pro_case%d_chi2" % i])
    s = d["sweep_scalars"]
    yield "sweep", impl.sweep(I, float(s[0]), float(s[1]), int(s[2]), float(s[3]), float(s[4])), d["sweep_out"]
    dra, ddec, ur, vr = impl.uv_rotate(0.8, 0.3 * 4.84813681109536e-06, -0.2 * 4.84813681109536e-06, u, v)
    yield "uv_rotate_offsets", np.array([dra, ddec]), d["rot_out"]
    yield "uv_rotate_u", ur, d["rot_urot"]
    yield "uv_rotate_v", vr, d["rot_vrot"]
    duv = 1. / (img.shape[0] * dxy)
    yield "interpolate_upper", impl.interpolate(d["interp_spec"], duv, u, v, origin="upper"), d["interp_upper"]
    yield "interpolate_lower", impl.interpolate(d["interp_spec"], duv, u, v, origin="lower"), d["interp_lower"]
    yield ("apply_phase", impl.apply_phase_vis(0.3 * 4.84813681109536e-06, -0.2 * 4.84813681109536e-06, u, v,
                                               d["phase_in"]), d["phase_out"])
    yield "reduce_chi2", np.array(impl.reduce_chi2(re, im, w, d["phase_in"])), d["chi2_reduce"]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())
