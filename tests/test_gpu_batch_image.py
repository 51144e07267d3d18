"""Batched FP32 chi2 of free-form images and its gradient (galario_gb300.batch.chi2_image_batch).

chi2 of each image is checked against the FP64 oracle's chi2Image (relative
1e-6); the gradient with respect to every pixel against a float64
torch.fft-composed reference differentiated by autograd
(tests/torch_reference.py); the gradient with respect to (PA, dRA, dDec)
against FP64 central finite differences of the oracle.

Images: a Gaussian ring plus N(0, 1e-4) pixel noise relative to the ring
peak, the free-form case of the batched gradient workload (2048^2 there,
512^2 here so that the float64 references finish in seconds).

Tolerances of this FP32 path: per-parameter relative 2e-3; pixel gradient
relative 2-norm 2e-2 (the modulus/argument interpolation weighs faint
spectrum values whose phase is at an FP32 FFT's rounding level, as for the
profile path).
"""
import numpy as np
import pytest

from helpers import arcsec, uv_log_uniform

pytestmark = pytest.mark.gpu

CHI2_TOL = 1e-6
GRAD_TOL = 2e-3
GRAD_PIX_TOL = 2e-2


def _images(B, nxy, dxy, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(nxy) - nxy / 2) * dxy
    X, Y = np.meshgrid(x, x)
    R = np.hypot(X, Y)
    out = []
    for b in range(B):
        r0, sig = rng.uniform(0.2, 0.8) * arcsec, rng.uniform(0.03, 0.1) * arcsec
        ring = np.exp(-0.5 * ((R - r0) / sig) ** 2)
        ring += rng.normal(0, 1e-4, ring.shape)
        out.append(ring * (0.1 / ring.sum()))
    return np.array(out)


@pytest.fixture(scope="module")
def icase():
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    from galario_gb300.batch import Dataset
    nxy, dxy, nd, B = 512, 0.01 * arcsec, 30000, 3
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(nd, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=11)
    imgs = _images(B, nxy, dxy, seed=12).astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(13)
    params = np.array([[rng.uniform(0, np.pi), rng.uniform(-0.05, 0.05) * arcsec, rng.uniform(-0.05, 0.05) * arcsec]
                       for _ in range(B)]).astype(np.float32).astype(np.float64)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd)
    vis = g.double.sampleImage(imgs[0], dxy, u, v, PA=params[0][0], dRA=params[0][1], dDec=params[0][2])
    re, im = vis.real + rng.normal(0, sigma), vis.imag + rng.normal(0, sigma)
    w = 1 / sigma ** 2
    c = dict(nxy=nxy, dxy=dxy, u=u, v=v, re=re, im=im, w=w, imgs=imgs, params=params)
    for k in ("u", "v", "re", "im", "w"):
        c[k] = c[k].astype(np.float32).astype(np.float64)
    c["ds"] = Dataset(c["u"], c["v"], c["re"], c["im"], c["w"])
    c["tI"] = torch.tensor(imgs, dtype=torch.float32, device="cuda")
    c["tp"] = torch.tensor(params, dtype=torch.float32, device="cuda")
    return c


@pytest.mark.parametrize("origin", ["upper", "lower"])
def test_image_batch_chi2_matches_oracle(icase, oracle_port, origin):
    from galario_gb300.batch import chi2_image_batch
    c = icase
    from galario_gb300.batch import status
    chi2 = chi2_image_batch(c["ds"], c["tI"], c["tp"], c["dxy"], origin=origin).cpu().numpy()
    assert status() == 0
    orc = oracle_port.get("port", "double")
    for b in range(len(chi2)):
        PA, dRA, dDec = c["params"][b]
        ref = orc.chi2Image(c["imgs"][b], c["dxy"], c["u"], c["v"], c["re"], c["im"], c["w"], PA=PA, dRA=dRA,
                            dDec=dDec, origin=origin)
        assert abs(chi2[b] - ref) / ref <= CHI2_TOL, (b, chi2[b], ref)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_image_batch_gradient_vs_torch_fp64(icase):
    import torch
    from galario_gb300.batch import chi2_image_batch
    from torch_reference import sample_image_t
    c = icase
    chi2, gI, gp = chi2_image_batch(c["ds"], c["tI"], c["tp"], c["dxy"], grad=True)
    gI, gp = gI.cpu().numpy(), gp.cpu().numpy()
    t = {k: torch.tensor(c[k], dtype=torch.float64) for k in ("u", "v", "re", "im", "w")}
    for b in range(len(gI)):
        img = torch.tensor(c["imgs"][b], dtype=torch.float64, requires_grad=True)
        p = [torch.tensor(x, dtype=torch.float64, requires_grad=True) for x in c["params"][b]]
        V = sample_image_t(img, c["dxy"], t["u"], t["v"], p[0], p[1], p[2])
        ref = torch.sum(t["w"] * ((V.real - t["re"]) ** 2 + (V.imag - t["im"]) ** 2))
        ref.backward()
        assert abs(float(chi2[b]) - ref.item()) / ref.item() <= CHI2_TOL
        assert _rel(gI[b], img.grad.numpy()) <= GRAD_PIX_TOL, (b, _rel(gI[b], img.grad.numpy()))
        ref_gp = np.array([x.grad.item() for x in p])
        for a in range(3):
            assert abs(gp[b, a] - ref_gp[a]) <= GRAD_TOL * abs(ref_gp[a]) + 1e-6 * np.abs(ref_gp).max(), \
                (b, a, gp[b, a], ref_gp[a])


def test_image_batch_params_gradient_vs_fd_oracle(icase, oracle_port):
    """FP64 central finite differences of the oracle's chi2Image with respect to PA, dRA, dDec.

    chi2(PA) has slope jumps wherever a visibility crosses a uv cell edge
    (bilinear interpolation), so the step must keep nearly all visibilities in
    their cells: 1e-6 relative (displacements below 2e-4 cells here); at 1e-5
    the central difference is already off by 0.7%.  A noiseless ring keeps
    the jumps small.
    """
    import torch
    from galario_gb300.batch import chi2_image_batch
    c = icase
    x = (np.arange(c["nxy"]) - c["nxy"] / 2) * c["dxy"]
    X, Y = np.meshgrid(x, x)
    ring = np.exp(-0.5 * ((np.hypot(X, Y) - 0.5 * arcsec) / (0.08 * arcsec)) ** 2)
    img = (ring * (0.1 / ring.sum())).astype(np.float32).astype(np.float64)
    base = [float(np.float32(v)) for v in (1.1, 0.02 * arcsec, -0.03 * arcsec)]
    _, _, gp = chi2_image_batch(c["ds"], torch.tensor(img[None], dtype=torch.float32, device="cuda"),
                                torch.tensor([base], dtype=torch.float32, device="cuda"), c["dxy"], grad=True)
    gp = gp.cpu().numpy()[0]
    orc = oracle_port.get("port", "double")

    def chi2_at(p):
        return orc.chi2Image(img, c["dxy"], c["u"], c["v"], c["re"], c["im"], c["w"], PA=p[0], dRA=p[1], dDec=p[2])
    for a in range(3):
        h = 1e-6 * abs(base[a])
        pp, pm = list(base), list(base)
        pp[a] += h
        pm[a] -= h
        fd = (chi2_at(pp) - chi2_at(pm)) / (2 * h)
        assert abs(gp[a] - fd) <= GRAD_TOL * abs(fd), (a, gp[a], fd)


def test_image_autograd_through_torch(icase):
    """Gradient of sum(chi2) of images built by torch ops (a scaled image) flows to the scale."""
    import torch
    from galario_gb300.autograd import chi2_image
    from galario_gb300.batch import chi2_image_batch
    c = icase
    scale = torch.tensor([1.0, 0.8, 1.2], dtype=torch.float64, device="cuda", requires_grad=True)
    imgs = (c["tI"].double() * scale[:, None, None]).float()
    tot = chi2_image(imgs, c["tp"], c["ds"], c["dxy"]).sum()
    tot.backward()
    _, gI, _ = chi2_image_batch(c["ds"], imgs.detach(), c["tp"], c["dxy"], grad=True)
    expect = (gI.double() * c["tI"].double()).sum(dim=(1, 2))
    torch.testing.assert_close(scale.grad, expect, rtol=1e-5, atol=0)


def test_image_batch_rejects_bad_input(icase):
    import torch
    from galario_gb300.batch import chi2_image_batch
    c = icase
    with pytest.raises(AssertionError, match="origin"):
        chi2_image_batch(c["ds"], c["tI"], c["tp"], c["dxy"], origin="middle")
    with pytest.raises(ValueError):
        chi2_image_batch(c["ds"], c["tI"][:, :, :-2], c["tp"], c["dxy"])
    bad = torch.zeros((1, 24, 24), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError, match="power of two"):
        chi2_image_batch(c["ds"], bad, c["tp"][:1], c["dxy"])
