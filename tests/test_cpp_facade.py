"""The C++ facade (include/galario_gb300.hpp): compiles, links and, on a GPU,
gives the oracle's numbers through the reference's C++ function names.

tests/cpp/link_test.cpp is built with g++ against the header and
libgalario_gb300.so, in double (-DGALARIO_DOUBLE_PRECISION) and float.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "galario_gb300", "_lib")
ARCSEC = 4.84813681109536e-06


def _build(tmp, double):
    from galario_gb300 import _build as B
    B.build()
    exe = os.path.join(tmp, "link_test_" + ("d" if double else "f"))
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "link_test.cpp"), "-o", exe, "-L", LIBDIR, "-lgalario_gb300",
           "-Wl,-rpath," + LIBDIR]
    if double:
        cmd.insert(1, "-DGALARIO_DOUBLE_PRECISION")
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("double", [True, False])
def test_cpp_facade_compiles_and_links(tmp_path, double):
    exe = _build(str(tmp_path), double)
    assert os.access(exe, os.X_OK)


def _inputs():
    dxy = 0.05 * ARCSEC
    nr, nd, nxy = 300, 2000, 128
    Rmin, dR = dxy / 50, dxy / 12
    duv = 1.0 / (nxy * dxy)
    R = Rmin + np.arange(nr) * dR
    I = 1e10 * np.exp(-0.5 * (R - 20 * dxy) ** 2 / (6 * dxy) ** 2)
    k = np.arange(nd)
    r, th = duv * (1.0 + 40.0 * k / nd), 2.399963229728653 * k
    u, v = r * np.cos(th), r * np.sin(th)
    re, im, w = 1e-3 * np.sin(0.1 * k), 1e-3 * np.cos(0.07 * k), 1e6 * (1 + k % 7)
    j = np.arange(nxy)
    x = (j - nxy // 2 + 3)[None, :]
    y = (j - nxy // 2 - 5)[:, None]
    img = 1e-3 * np.exp(-(x * x) / 200.0 - (y * y) / 90.0)
    kw = dict(inc=0.6, PA=1.1, dRA=0.1 * ARCSEC, dDec=-0.2 * ARCSEC)
    return dict(nr=nr, nd=nd, nxy=nxy, dxy=dxy, Rmin=Rmin, dR=dR, I=I, u=u, v=v, re=re, im=im, w=w, img=img, kw=kw)


@pytest.mark.gpu
def test_cpp_facade_matches_oracle(tmp_path, oracle_port):
    exe = _build(str(tmp_path), True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    vals = {}
    for line in out.splitlines():
        key, *nums = line.split()
        vals[key] = [float(x) for x in nums]
    assert vals["invalid_argument"] == [1.0]
    P = _inputs()
    orc = oracle_port.get("port", "double")
    kw = P["kw"]
    ref_p = orc.chi2Profile(P["I"], P["Rmin"], P["dR"], P["nxy"], P["dxy"], P["u"], P["v"], P["re"], P["im"],
                            P["w"], **kw)
    ref_i = orc.chi2Image(P["img"], P["dxy"], P["u"], P["v"], P["re"], P["im"], P["w"], dRA=kw["dRA"],
                          dDec=kw["dDec"], PA=kw["PA"])
    vis = orc.sampleProfile(P["I"], P["Rmin"], P["dR"], P["nxy"], P["dxy"], P["u"], P["v"], **kw)
    assert abs(vals["chi2_profile"][0] - ref_p) <= 1e-12 * abs(ref_p)
    assert abs(vals["chi2_image"][0] - ref_i) <= 1e-12 * abs(ref_i)
    scale = np.abs(vis).max()
    np.testing.assert_allclose(vals["vis0"], [vis[0].real, vis[0].imag], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(vals["vis%d" % (P["nd"] - 1)], [vis[-1].real, vis[-1].imag], rtol=0,
                               atol=1e-12 * scale)


@pytest.mark.gpu
def test_cpp_facade_float_runs(tmp_path):
    exe = _build(str(tmp_path), False)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert "invalid_argument 1" in out
