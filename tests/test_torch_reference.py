"""The float64 torch reference (tests/torch_reference.py) against the CPU oracle."""
import numpy as np
import pytest

from helpers import arcsec, deg, uv_log_uniform


def test_torch_reference_matches_oracle(oracle_port):
    torch = pytest.importorskip("torch")
    from torch_reference import chi2_profile_t
    orc = oracle_port.get("port", "double")
    nxy, dxy, Rmin, dR, nr = 128, 0.03 * arcsec, 1e-4 * arcsec, 1.5e-3 * arcsec, 800
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(2000, 0.5 * duv, 0.4 * nxy / 2 * duv, seed=3)
    R = Rmin + dR * np.arange(nr)
    I = np.exp(-0.5 * ((R - 0.5 * arcsec) / (0.1 * arcsec)) ** 2) * 1e10
    rng = np.random.default_rng(0)
    re, im, w = rng.normal(0, 1e-3, 2000), rng.normal(0, 1e-3, 2000), rng.uniform(0.5, 1.5, 2000) * 1e6
    kw = dict(inc=30 * deg, PA=1.1, dRA=0.02 * arcsec, dDec=-0.03 * arcsec)
    ref = orc.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, **kw)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    got = chi2_profile_t(t(I), t(kw["inc"]), t(kw["PA"]), t(kw["dRA"]), t(kw["dDec"]), Rmin, dR, nxy, dxy, t(u),
                         t(v), t(re), t(im), t(w))
    assert abs(float(got) - ref) / ref <= 1e-10
