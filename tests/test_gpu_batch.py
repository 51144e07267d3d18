"""Batched FP32 chi2 and its gradient (galario_gb300.batch / .autograd).

chi2 of each model is checked against the single-model modules and the FP64
oracle (relative 1e-6); the gradient against a float64 torch.fft-composed
reference differentiated by autograd (tests/torch_reference.py) and against
FP64 central finite differences of the oracle.

Gradient tolerances of this FP32 path (measured, and reproduced by a float32
emulation of the same algorithm on the CPU):
- smooth parameters (inc, PA, dRA, dDec; ring radius, width, flux through
  torch): relative 2e-3 per component;
- the gradient with respect to every individual profile sample: relative
  2-norm 5e-2.  The modulus/argument interpolation makes this gradient depend
  on the phase of spectrum values far below the spectrum peak, where an FP32
  FFT's rounding dominates; the float64 reference of the same algorithm agrees
  to 4e-11, so the bound is FP32 arithmetic, not the adjoint.
"""
import numpy as np
import pytest

from helpers import arcsec, deg, uv_log_uniform

pytestmark = pytest.mark.gpu

CHI2_TOL = 1e-6
GRAD_TOL = 2e-3        # smooth parameters
GRAD_SAMPLES_TOL = 5e-2  # per profile sample (see the module docstring)


def _setup(seed=0, nxy=512, nd=40000, nr=1500, B=3):
    dxy = 0.02 * arcsec
    Rmin, dR = 1e-4 * arcsec, 1e-3 * arcsec
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(nd, 0.5 * duv, 0.4 * nxy / 2 * duv, seed=seed)
    rng = np.random.default_rng(seed + 1)
    R = Rmin + dR * np.arange(nr)
    I = []
    params = []
    for b in range(B):
        r0, sig = rng.uniform(0.3, 0.9) * arcsec, rng.uniform(0.05, 0.2) * arcsec
        I.append(np.exp(-0.5 * ((R - r0) / sig) ** 2) * 1e10 * rng.uniform(0.5, 2))
        params.append([rng.uniform(0, 60) * deg, rng.uniform(0, 180) * deg, rng.uniform(-0.05, 0.05) * arcsec,
                       rng.uniform(-0.05, 0.05) * arcsec])
    I = np.array(I)
    params = np.array(params)
    sigma = rng.uniform(0.5e-3, 1.5e-3, nd) * 10
    re, im = rng.normal(0, sigma), rng.normal(0, sigma)
    w = 1 / sigma ** 2
    return dict(nxy=nxy, dxy=dxy, Rmin=Rmin, dR=dR, u=u, v=v, re=re, im=im, w=w, I=I, params=params)


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    from galario_gb300.batch import Dataset
    c = _setup()
    # observations close to the first model, so residuals are not only noise
    f = np.float32
    vis = g.double.sampleProfile(c["I"][0], c["Rmin"], c["dR"], c["nxy"], c["dxy"], c["u"], c["v"],
                                 inc=c["params"][0][0], PA=c["params"][0][1], dRA=c["params"][0][2],
                                 dDec=c["params"][0][3])
    c["re"] = c["re"] + vis.real
    c["im"] = c["im"] + vis.imag
    for k in ("u", "v", "re", "im", "w"):
        c[k] = c[k].astype(f).astype(np.float64)  # the dataset is float32: test on the rounded values
    c["I"] = c["I"].astype(f).astype(np.float64)
    c["params"] = c["params"].astype(f).astype(np.float64)
    c["ds"] = Dataset(c["u"], c["v"], c["re"], c["im"], c["w"])
    c["tI"] = torch.tensor(c["I"], dtype=torch.float32, device="cuda")
    c["tp"] = torch.tensor(c["params"], dtype=torch.float32, device="cuda")
    return c


def test_batch_chi2_matches_oracle_and_single(case, oracle_port):
    import galario_gb300 as g
    from galario_gb300.batch import chi2_profile_batch
    c = case
    from galario_gb300.batch import status
    chi2 = chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"]).cpu().numpy()
    assert status() == 0  # every visibility inside the spectrum window
    orc = oracle_port.get("port", "double")
    f = np.float32
    for b in range(len(chi2)):
        inc, PA, dRA, dDec = c["params"][b]
        ref = orc.chi2Profile(c["I"][b], c["Rmin"], c["dR"], c["nxy"], c["dxy"], c["u"], c["v"], c["re"], c["im"],
                              c["w"], inc=inc, PA=PA, dRA=dRA, dDec=dDec)
        assert abs(chi2[b] - ref) / ref <= CHI2_TOL, (b, chi2[b], ref)
        single = g.single.chi2Profile(c["I"][b].astype(f), c["Rmin"], c["dR"], c["nxy"], c["dxy"], c["u"].astype(f),
                                      c["v"].astype(f), c["re"].astype(f), c["im"].astype(f), c["w"].astype(f),
                                      inc=inc, PA=PA, dRA=dRA, dDec=dDec)
        assert abs(chi2[b] - single) / ref <= CHI2_TOL


def _ref_grad(c, b):
    import torch
    from torch_reference import chi2_profile_t
    d = dict(dtype=torch.float64)
    I = torch.tensor(c["I"][b], requires_grad=True, **d)
    p = [torch.tensor(x, requires_grad=True, **d) for x in c["params"][b]]
    t = {k: torch.tensor(c[k], **d) for k in ("u", "v", "re", "im", "w")}
    chi2 = chi2_profile_t(I, p[0], p[1], p[2], p[3], c["Rmin"], c["dR"], c["nxy"], c["dxy"], t["u"], t["v"],
                          t["re"], t["im"], t["w"])
    chi2.backward()
    return float(chi2.detach()), I.grad.numpy(), np.array([x.grad.item() for x in p])


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_batch_gradient_vs_torch_fp64(case):
    from galario_gb300.batch import chi2_profile_batch
    c = case
    chi2, gI, gp = chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"], grad=True)
    chi2, gI, gp = chi2.cpu().numpy(), gI.cpu().numpy(), gp.cpu().numpy()
    for b in range(len(chi2)):
        ref_chi2, ref_gI, ref_gp = _ref_grad(c, b)
        assert abs(chi2[b] - ref_chi2) / ref_chi2 <= CHI2_TOL
        assert _rel(gI[b], ref_gI) <= GRAD_SAMPLES_TOL, (b, _rel(gI[b], ref_gI))
        for a in range(4):
            assert abs(gp[b, a] - ref_gp[a]) <= GRAD_TOL * abs(ref_gp[a]) + 1e-6 * np.abs(ref_gp).max(), \
                (b, a, gp[b, a], ref_gp[a])


def test_batch_gradient_vs_fd_oracle(case, oracle_port):
    """FP64 central finite differences (h = 1e-6 relative) of the oracle's chi2Profile."""
    from galario_gb300.batch import chi2_profile_batch
    c = case
    _, gI, gp = chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"], grad=True)
    gp = gp.cpu().numpy()
    orc = oracle_port.get("port", "double")
    b = 1
    base = list(c["params"][b])

    def chi2_at(p):
        return orc.chi2Profile(c["I"][b], c["Rmin"], c["dR"], c["nxy"], c["dxy"], c["u"], c["v"], c["re"],
                               c["im"], c["w"], inc=p[0], PA=p[1], dRA=p[2], dDec=p[3])
    for a in range(4):
        h = 1e-6 * max(abs(base[a]), 1e-3 if a < 2 else 1e-9)
        pp, pm = list(base), list(base)
        pp[a] += h
        pm[a] -= h
        fd = (chi2_at(pp) - chi2_at(pm)) / (2 * h)
        assert abs(gp[b, a] - fd) <= GRAD_TOL * abs(fd), (a, gp[b, a], fd)


def test_autograd_parametric_rings(case):
    """Gradient of sum chi2 w.r.t. ring radius, width and flux through torch + the adjoint kernels."""
    import torch
    from galario_gb300.autograd import chi2_profile
    from torch_reference import chi2_profile_t
    c = case
    nr = c["I"].shape[1]
    R = torch.tensor(c["Rmin"] + c["dR"] * np.arange(nr), dtype=torch.float64)

    def rings(theta):  # theta (B, 3): r0 [arcsec], sigma [arcsec], amplitude [1e10 Jy/sr]
        r0, sig, amp = theta[:, 0:1] * arcsec, theta[:, 1:2] * arcsec, theta[:, 2:3] * 1e10
        return amp * torch.exp(-0.5 * ((R - r0) / sig) ** 2)

    theta = torch.tensor([[0.5, 0.1, 1.0], [0.7, 0.15, 0.6]], dtype=torch.float64)
    params = torch.tensor(c["params"][:2], dtype=torch.float64)
    th_gpu = theta.clone().cuda().requires_grad_(True)
    p_gpu = params.clone().cuda().requires_grad_(True)
    R_gpu = R.cuda()
    r0, sig, amp = th_gpu[:, 0:1] * arcsec, th_gpu[:, 1:2] * arcsec, th_gpu[:, 2:3] * 1e10
    I_gpu = (amp * torch.exp(-0.5 * ((R_gpu - r0) / sig) ** 2)).float()
    chi2 = chi2_profile(I_gpu, p_gpu.float(), c["ds"], c["Rmin"], c["dR"], c["dxy"], c["nxy"])
    chi2.sum().backward()
    th_ref = theta.clone().requires_grad_(True)
    p_ref = params.clone().requires_grad_(True)
    I_ref = rings(th_ref)
    t = {k: torch.tensor(c[k], dtype=torch.float64) for k in ("u", "v", "re", "im", "w")}
    tot = 0
    for b in range(2):
        tot = tot + chi2_profile_t(I_ref[b], p_ref[b, 0], p_ref[b, 1], p_ref[b, 2], p_ref[b, 3], c["Rmin"], c["dR"],
                                   c["nxy"], c["dxy"], t["u"], t["v"], t["re"], t["im"], t["w"])
    tot.backward()
    assert _rel(th_gpu.grad.cpu().numpy(), th_ref.grad.numpy()) <= GRAD_TOL
    assert _rel(p_gpu.grad.cpu().numpy(), p_ref.grad.numpy()) <= GRAD_TOL


def test_batch_rejects_bad_geometry(case):
    from galario_gb300.batch import chi2_profile_batch
    c = case
    with pytest.raises(ValueError, match="Try reducing dR"):
        chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dxy"] / 4, c["dxy"], c["nxy"])
    with pytest.raises(ValueError, match="is odd"):
        chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], 511)


def test_batch_visibility_sets(case, oracle_port):
    """Uneven visibility sets: chi2 per set against the oracle, total and gradient against one set."""
    from galario_gb300.batch import Dataset, chi2_profile_batch
    c = case
    cuts = [0, 7001, 7001 + 25000, len(c["u"])]  # uneven; the last set is short
    parts = [slice(cuts[k], cuts[k + 1]) for k in range(3)]
    ds = Dataset(*[[c[k][p] for p in parts] for k in ("u", "v", "re", "im", "w")])
    assert ds.nsets == 3 and ds.nvis_per_set == [cuts[k + 1] - cuts[k] for k in range(3)]
    table = chi2_profile_batch(ds, c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"], per_set=True)
    table = table.cpu().numpy()
    assert table.shape == (len(c["I"]), 3)
    orc = oracle_port.get("port", "double")
    for b in range(len(c["I"])):
        inc, PA, dRA, dDec = c["params"][b]
        for k, p in enumerate(parts):
            ref = orc.chi2Profile(c["I"][b], c["Rmin"], c["dR"], c["nxy"], c["dxy"], c["u"][p], c["v"][p],
                                  c["re"][p], c["im"][p], c["w"][p], inc=inc, PA=PA, dRA=dRA, dDec=dDec)
            assert abs(table[b, k] - ref) / ref <= CHI2_TOL, (b, k, table[b, k], ref)
    tot, gI, gp = chi2_profile_batch(ds, c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"], grad=True)
    tot1, gI1, gp1 = chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"], grad=True)
    tot_fwd = chi2_profile_batch(ds, c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"], c["nxy"])
    np.testing.assert_allclose(tot_fwd.cpu().numpy(), table.sum(axis=1), rtol=1e-14)  # same launches
    np.testing.assert_allclose(tot.cpu().numpy(), table.sum(axis=1), rtol=CHI2_TOL)
    np.testing.assert_allclose(tot.cpu().numpy(), tot1.cpu().numpy(), rtol=CHI2_TOL)
    for b in range(len(c["I"])):
        assert _rel(gI[b].cpu().numpy(), gI1[b].cpu().numpy()) <= 1e-3
        assert _rel(gp[b].cpu().numpy(), gp1[b].cpu().numpy()) <= 1e-4


def test_batch_rejects_bad_sets():
    import ctypes as C
    from galario_gb300 import _lib
    from galario_gb300.batch import _bind
    L = _bind()
    u = np.zeros(8, np.float32)
    h = C.c_void_p()
    off = np.array([0, 5, 3, 8], np.int32)  # decreasing
    p = u.ctypes.data_as(C.c_void_p)
    st = L.galario_dataset_create_f(8, p, p, p, p, p, 3, off.ctypes.data_as(C.c_void_p), 0, C.byref(h))
    assert st == _lib.EINVAL
    off = np.array([0, 5, 7], np.int32)  # does not end at nd
    st = L.galario_dataset_create_f(8, p, p, p, p, p, 2, off.ctypes.data_as(C.c_void_p), 0, C.byref(h))
    assert st == _lib.EINVAL


def test_batch_graph_replay_matches_eager(case, monkeypatch):
    """From the second call of a combination on, the call replays a captured CUDA graph."""
    import torch
    from galario_gb300.batch import chi2_profile_batch
    c = case
    args = (c["Rmin"], c["dR"], c["dxy"], c["nxy"])
    scales = [1.0, 0.7, 1.3, 0.9]
    monkeypatch.setenv("GALARIO_GRAPHS", "0")
    eager = [chi2_profile_batch(c["ds"], c["tI"] * f, c["tp"], *args, grad=True) for f in scales]
    monkeypatch.setenv("GALARIO_GRAPHS", "1")
    for f, (e_chi2, e_gI, e_gp) in zip(scales, eager):
        tI = (c["tI"] * f).clone()  # a fresh input buffer every call
        chi2, gI, gp = chi2_profile_batch(c["ds"], tI, c["tp"].clone(), *args, grad=True)
        torch.testing.assert_close(chi2, e_chi2, rtol=0, atol=0)  # fixed-order reduction
        torch.testing.assert_close(gI, e_gI, rtol=1e-4, atol=1e-6 * float(e_gI.abs().max()))
        torch.testing.assert_close(gp, e_gp, rtol=1e-4, atol=1e-6 * float(e_gp.abs().max()))
    # forward-only calls are a separate combination (their own launch shapes)
    for f in scales[:3]:
        chi2 = chi2_profile_batch(c["ds"], c["tI"] * f, c["tp"], *args)
        torch.testing.assert_close(chi2, eager[scales.index(f)][0], rtol=CHI2_TOL, atol=0)


def test_batch_rejects_uv_beyond_image(case):
    from galario_gb300.batch import Dataset, chi2_profile_batch
    c = case
    with pytest.raises(ValueError, match="beyond the image's uv range"):
        chi2_profile_batch(c["ds"], c["tI"], c["tp"], c["Rmin"], c["dR"], c["dxy"] * 4, c["nxy"] // 4)
    u = c["u"].copy()
    u[5] = np.nan
    with pytest.raises(ValueError, match="must be finite"):
        Dataset(u, c["v"], c["re"], c["im"], c["w"])


def test_batch_profile_wider_than_image(oracle_port):
    """Batched path with the profile support beyond the image (rmax = nxy/2)."""
    import torch
    from galario_gb300.batch import Dataset, chi2_profile_batch, status
    nxy, dxy = 256, 0.02 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 1e-3 * arcsec, 4000
    R = Rmin + dR * np.arange(nr)
    I = np.stack([1e10 * np.exp(-0.5 * (R / (1.5 * arcsec)) ** 2), 5e9 * np.exp(-0.5 * (R / (2.5 * arcsec)) ** 2)])
    I = I.astype(np.float32).astype(np.float64)
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(5000, 0.5 * duv, 0.45 * nxy / 2 * duv, seed=7)
    rng = np.random.default_rng(8)
    re, im, w = rng.normal(0, 1e-3, 5000), rng.normal(0, 1e-3, 5000), rng.uniform(0.5, 2, 5000) * 1e6
    c = {k: np.asarray(x, dtype=np.float32).astype(np.float64) for k, x in dict(u=u, v=v, re=re, im=im, w=w).items()}
    params = np.array([[0.3, 1.0, 0.01 * arcsec, 0.0], [0.6, 2.0, 0.0, -0.02 * arcsec]]).astype(np.float32)
    ds = Dataset(c["u"], c["v"], c["re"], c["im"], c["w"])
    chi2 = chi2_profile_batch(ds, torch.tensor(I, dtype=torch.float32, device="cuda"),
                              torch.tensor(params, device="cuda"), Rmin, dR, dxy, nxy).cpu().numpy()
    assert status() == 0
    orc = oracle_port.get("port", "double")
    f = lambda x: float(np.float32(x))  # noqa: E731
    for b in range(2):
        inc, PA, dRA, dDec = (float(x) for x in params[b])
        ref = orc.chi2Profile(I[b], f(Rmin), f(dR), nxy, f(dxy), c["u"], c["v"], c["re"], c["im"], c["w"], inc=inc,
                              PA=PA, dRA=dRA, dDec=dDec)
        assert abs(chi2[b] - ref) / ref <= CHI2_TOL, (b, chi2[b], ref)


@pytest.mark.parametrize("nxy", [1000, 1536])
def test_batch_non_power_of_two_nxy(nxy, oracle_port, monkeypatch):
    """Swept profiles at an even nxy that is not a power of two: the spectrum
    passes are products with cosine matrices, where nxy enters only the
    angles.  chi2 against the FP64 oracle, the gradient against the float64
    torch reference; with the tensor-core passes off (FFT passes, powers of two
    only) the call is refused, and so is a batch of images at that size."""
    import torch
    from galario_gb300.batch import Dataset, chi2_image_batch, chi2_profile_batch, status
    c = _setup(seed=3, nxy=nxy, nd=30000, B=2)
    f = np.float32
    for k in ("u", "v", "re", "im", "w", "I", "params"):
        c[k] = c[k].astype(f).astype(np.float64)
    ds = Dataset(c["u"], c["v"], c["re"], c["im"], c["w"])
    tI = torch.tensor(c["I"], dtype=torch.float32, device="cuda")
    tp = torch.tensor(c["params"], dtype=torch.float32, device="cuda")
    args = (c["Rmin"], c["dR"], c["dxy"], nxy)
    chi2, gI, gp = chi2_profile_batch(ds, tI, tp, *args, grad=True)
    chi2_fwd = chi2_profile_batch(ds, tI, tp, *args).cpu().numpy()
    assert status() == 0
    chi2, gI, gp = chi2.cpu().numpy(), gI.cpu().numpy(), gp.cpu().numpy()
    orc = oracle_port.get("port", "double")
    for b in range(2):
        inc, PA, dRA, dDec = c["params"][b]
        ref = orc.chi2Profile(c["I"][b], c["Rmin"], c["dR"], nxy, c["dxy"], c["u"], c["v"], c["re"], c["im"],
                              c["w"], inc=inc, PA=PA, dRA=dRA, dDec=dDec)
        assert abs(chi2_fwd[b] - ref) / ref <= CHI2_TOL, (b, chi2_fwd[b], ref)
        assert abs(chi2[b] - ref) / ref <= CHI2_TOL, (b, chi2[b], ref)
        ref_chi2, ref_gI, ref_gp = _ref_grad(dict(c, nxy=nxy), b)
        assert abs(ref_chi2 - ref) / ref <= 1e-12
        assert _rel(gI[b], ref_gI) <= GRAD_SAMPLES_TOL, (b, _rel(gI[b], ref_gI))
        for a in range(4):
            assert abs(gp[b, a] - ref_gp[a]) <= GRAD_TOL * abs(ref_gp[a]) + 1e-6 * np.abs(ref_gp).max(), \
                (b, a, gp[b, a], ref_gp[a])
    monkeypatch.setenv("GALARIO_TC", "0")
    with pytest.raises(ValueError, match="power of two"):
        chi2_profile_batch(ds, tI, tp, *args)
    monkeypatch.delenv("GALARIO_TC")
    imgs = torch.zeros((1, nxy, nxy), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError, match="power of two"):
        chi2_image_batch(ds, imgs, torch.zeros((1, 3), dtype=torch.float32, device="cuda"), c["dxy"])
