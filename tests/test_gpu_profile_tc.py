"""The tensor-core spectrum of FP64 swept profiles (galario_gb300/csrc/gb_profile_tc.cu).

The FP64 chi2Profile / sampleProfile compute the spectrum window as two
cosine-matrix products on the bf16 tensor cores (eight-digit split, exact
integer sums) whenever the quadrant of the sweep has at most 2048 columns;
GALARIO_TC=0 keeps the row and column transforms.  Both must agree with the
oracle within the double tolerances, and with each other to rounding level,
on the benchmarked workload and on geometries that reach the edges of the
path: quadrants of several K tiles and one beyond 2048 (which falls back), a
profile wider than the image (rmax clamped to nxy/2, the edge row and column
carry emission), even sizes that are not powers of two, and a window that
covers every column (the flat-index wrap of the last column).
"""
import numpy as np
import pytest

from helpers import arcsec, deg, uv_log_uniform

pytestmark = pytest.mark.gpu

DP_V, DP_CHI2 = 1e-12, 1e-12


def _obs(nd, seed):
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    return rng.normal(0, sigma), rng.normal(0, sigma), 1. / sigma ** 2


def _both(monkeypatch, fn):
    """fn() with the tensor-core path (default) and with GALARIO_TC=0."""
    monkeypatch.delenv("GALARIO_TC", raising=False)
    a = fn()
    monkeypatch.setenv("GALARIO_TC", "0")
    b = fn()
    monkeypatch.delenv("GALARIO_TC", raising=False)
    return a, b


def _rel_max(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_bench_workload_tc_vs_transforms(monkeypatch, oracle_port):
    import bench
    import galario_gb300 as g
    wl = bench.Workload(seed=0)
    orc = oracle_port.get("port", "double")
    kw = wl.kw()
    args = (wl.intensity, wl.Rmin, wl.dR, wl.nxy, wl.dxy, wl.u, wl.v)
    vis_tc, vis_ft = _both(monkeypatch, lambda: g.double.sampleProfile(*args, **kw))
    vis_ref = orc.sampleProfile(*args, **kw)
    assert _rel_max(vis_tc, vis_ref) <= DP_V
    assert _rel_max(vis_ft, vis_ref) <= DP_V
    assert _rel_max(vis_tc, vis_ft) <= 1e-13
    re, im = vis_ref.real + wl.noise_re, vis_ref.imag + wl.noise_im
    c_tc, c_ft = _both(monkeypatch, lambda: g.double.chi2Profile(*args, re, im, wl.w, **kw))
    ref = orc.chi2Profile(*args, re, im, wl.w, **kw)
    assert abs(c_tc - ref) / ref <= DP_CHI2
    assert abs(c_ft - ref) / ref <= DP_CHI2
    # repeated calls give the same bits (the level buffers are cleared between calls)
    assert g.double.chi2Profile(*args, re, im, wl.w, **kw) == c_tc


@pytest.mark.parametrize("nxy,rmax_target,inc,reach", [
    (256, 500, 35 * deg, 0.45),    # profile wider than the image: rmax clamped, nF = nxy/2 + 1
    (250, 500, 10 * deg, 0.45),    # the same at an even size that is not a power of two
    (1000, 586, 60 * deg, 0.49),   # non power of two, nF = 501, window near the full half-plane
    (1536, 450, 20 * deg, 0.3),
    (2048, 511, 40 * deg, 0.3),    # quadrant of 511 columns: 8 K tiles, the last one partial
    (2048, 600, 40 * deg, 0.3),    # 10 K tiles
    (8192, 2100, 30 * deg, 0.05),  # quadrant beyond 2048 columns: the transforms run
])
def test_geometries_against_oracle(monkeypatch, oracle_port, nxy, rmax_target, inc, reach):
    import galario_gb300 as g
    orc = oracle_port.get("port", "double")
    dxy = 0.002 * arcsec * 1024 / min(nxy, 1024)
    Rmin, dR = 1e-4 * arcsec, 1e-4 * arcsec
    # the profile ends half a pixel inside pixel rmax_target
    nr = int(round(((rmax_target - 0.5) * dxy - Rmin) / dR))
    rmax = min(int(np.ceil((Rmin + nr * dR) / dxy)), nxy // 2)
    assert rmax == min(rmax_target, nxy // 2)
    ext = rmax_target * dxy
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * (np.exp(-0.5 * ((R - 0.3 * ext) / (0.05 * ext)) ** 2) + 0.3 * np.exp(-0.5 * (R / (0.4 * ext)) ** 2))
    duv = 1 / (nxy * dxy)
    nd = 20000
    u, v = uv_log_uniform(nd, 0.5 * duv, reach * nxy * duv, seed=nxy)
    re, im, w = _obs(nd, seed=nxy + 1)
    kw = dict(inc=inc, PA=1.1, dRA=0.02 * arcsec, dDec=-0.01 * arcsec)
    args = (I, Rmin, dR, nxy, dxy, u, v)
    vis_tc, vis_ft = _both(monkeypatch, lambda: g.double.sampleProfile(*args, **kw))
    vis_ref = orc.sampleProfile(*args, **kw)
    assert _rel_max(vis_tc, vis_ref) <= DP_V, (rmax, _rel_max(vis_tc, vis_ref))
    assert _rel_max(vis_ft, vis_ref) <= DP_V
    c_tc, c_ft = _both(monkeypatch, lambda: g.double.chi2Profile(*args, re, im, w, **kw))
    ref = orc.chi2Profile(*args, re, im, w, **kw)
    assert abs(c_tc - ref) / ref <= DP_CHI2, (rmax, c_tc, ref)
    assert abs(c_ft - ref) / ref <= DP_CHI2


def test_large_non_power_of_two_vs_transforms(monkeypatch):
    """nxy = 6000 (2^4 3 5^3): the tensor-core path against the mixed-radix
    transforms of the same library (the oracle's direct DFT at this size takes
    minutes); both agree to rounding level."""
    import galario_gb300 as g
    nxy, dxy = 6000, 0.002 * arcsec
    Rmin, dR = 1e-4 * arcsec, 1e-4 * arcsec
    nr = int(round((249.5 * dxy - Rmin) / dR))
    R = Rmin + dR * np.arange(nr)
    ext = 250 * dxy
    I = 1e10 * (np.exp(-0.5 * ((R - 0.3 * ext) / (0.05 * ext)) ** 2) + 0.3 * np.exp(-0.5 * (R / (0.4 * ext)) ** 2))
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(50000, 0.5 * duv, 0.2 * nxy * duv, seed=6000)
    re, im, w = _obs(50000, seed=6001)
    kw = dict(inc=45 * deg, PA=1.1, dRA=0.02 * arcsec, dDec=-0.01 * arcsec)
    args = (I, Rmin, dR, nxy, dxy, u, v)
    vis_tc, vis_ft = _both(monkeypatch, lambda: g.double.sampleProfile(*args, **kw))
    assert _rel_max(vis_tc, vis_ft) <= 1e-13
    c_tc, c_ft = _both(monkeypatch, lambda: g.double.chi2Profile(*args, re, im, w, **kw))
    assert abs(c_tc - c_ft) / c_ft <= DP_CHI2


def test_full_window_wrap(monkeypatch, oracle_port):
    """uv points past the last spectrum column: the window covers every
    column, the cells of the last column take their u+1 corners from column 0
    of the next row, and points beyond it continue on the next row (the
    reference's flat indexing, src/galario.cpp:774-780)."""
    import galario_gb300 as g
    orc = oracle_port.get("port", "double")
    nxy, dxy = 64, 1e-8
    Rmin, dR, nr = 1e-10, 5e-10, 400
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * ((R - 6e-8) / (2e-8)) ** 2)
    duv = 1 / (nxy * dxy)
    u = np.array([0.1, 32.4, 32.9, 33.3, 40.3, -32.5, 12.2]) * duv
    v = np.array([0.2, 0.1, -3.3, 2.7, 0.1, 3.7, -20.4]) * duv
    re, im, w = _obs(len(u), seed=4)
    kw = dict(inc=0.4, dRA=0.01 * arcsec)
    args = (I, Rmin, dR, nxy, dxy, u, v)
    vis_tc, vis_ft = _both(monkeypatch, lambda: g.double.sampleProfile(*args, **kw))
    vis_ref = orc.sampleProfile(*args, **kw)
    assert _rel_max(vis_tc, vis_ref) <= DP_V
    assert _rel_max(vis_ft, vis_ref) <= DP_V
    c_tc, c_ft = _both(monkeypatch, lambda: g.double.chi2Profile(*args, re, im, w, **kw))
    ref = orc.chi2Profile(*args, re, im, w, **kw)
    assert abs(c_tc - ref) / ref <= DP_CHI2
    assert abs(c_ft - ref) / ref <= DP_CHI2


def test_non_finite_profile_propagates(monkeypatch):
    """A NaN in the profile gives a NaN chi2 on both paths, as the reference's
    arithmetic does."""
    import galario_gb300 as g
    nxy, dxy = 256, 0.01 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 2e-4 * arcsec, 3000
    R = Rmin + dR * np.arange(nr)
    I = 1e10 * np.exp(-0.5 * ((R - 0.2 * arcsec) / (0.03 * arcsec)) ** 2)
    I[1500] = np.nan
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(3000, 0.5 * duv, 0.3 * nxy * duv, seed=9)
    re, im, w = _obs(3000, seed=10)
    c_tc, c_ft = _both(monkeypatch, lambda: g.double.chi2Profile(I, Rmin, dR, nxy, dxy, u, v, re, im, w, inc=0.3))
    assert np.isnan(c_ft)
    assert np.isnan(c_tc)
