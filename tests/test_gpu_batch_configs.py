"""The batched FP32 path at the full sizes of its two workloads.

Datasets: 8 visibility sets (spectral windows) of uneven size, set k with
nd_k ~ U[2e5, 3e6] visibilities (seed 1000 + k), radius log-uniform in
[1e4, 2e6] wavelengths and uniform angle, noise sigma ~ U[0.5, 1.5] mJy,
w = 1/sigma^2 (7.74M visibilities in all); the observations are a Gaussian
ring (r0 0.4", sigma 0.05", 0.1 Jy, inc 40 deg, PA 70 deg, offsets
0.01"/-0.02") plus the noise.  nxy = 2048, dxy = 5e-3", profile grid
Rmin = 1e-4", dR = 4e-4", nr = 4096.  Everything the batched call receives
is float32, so the references take the same float32-rounded values.

- B = 256 single-ring walkers (r0 ~ U[0.1, 0.8]", sigma ~ U[0.01, 0.1]",
  flux ~ U[0.05, 0.2] Jy, inc ~ U[0, 70] deg, PA ~ U[0, 180] deg): chi2 of
  every set, for 16 of the walkers, against the FP64 oracle (relative 1e-6).
- B = 64 ring walkers, the gradient of the total chi2 with respect to
  theta = (r0, sigma, flux, inc, PA, dRA, dDec) through the autograd
  Function: against the float64 torch restatement of chi2Profile and against
  FP64 central finite differences of the oracle.  The FP32 bulk keeps a
  component's relative error below C * 2^-24 * kappa, kappa = sum_k |t_k| /
  |sum_k t_k| the condition number of the component's sum over the
  visibilities (tests/grad_conditioning.py); C = 512 (measured ratios up to
  112).  Where kappa is O(1) that is a few 1e-6; near the optimum kappa
  reaches 1e4 and the error follows it.
- B = 2 free-form 2048^2 images (ring plus N(0, 1e-4) pixel noise): the
  gradient with respect to every pixel against the float64 torch reference.
"""
import numpy as np
import pytest

from helpers import arcsec, deg

pytestmark = pytest.mark.gpu

CHI2_TOL = 1e-6
U32 = 2.0 ** -24
KAPPA_C = 512.0
NXY, DXY, RMIN, DR, NR = 2048, 5e-3 * arcsec, 1e-4 * arcsec, 4e-4 * arcsec, 4096
TRUTH = (0.4, 0.05, 0.1, 40 * deg, 70 * deg, 0.01 * arcsec, -0.02 * arcsec)


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def sets():
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    from galario_gb300.batch import Dataset
    from grad_conditioning import ring_profile_t
    geo32 = [float(np.float32(x)) for x in (DXY, RMIN, DR)]
    dxy, Rmin, dR = geo32
    us, vs, ws, nre, nim = [], [], [], [], []
    for k in range(8):
        r = np.random.default_rng(1000 + k)
        n = int(r.uniform(2e5, 3e6))
        rad = np.exp(r.uniform(np.log(1e4), np.log(2e6), n))
        th = r.uniform(0, 2 * np.pi, n)
        sig = r.uniform(0.5e-3, 1.5e-3, n)
        us.append(rad * np.cos(th))
        vs.append(rad * np.sin(th))
        ws.append(1 / sig ** 2)
        nre.append(r.normal(0, sig))
        nim.append(r.normal(0, sig))
    cuts = np.cumsum([0] + [len(x) for x in us])
    u, v, w = f32(np.concatenate(us)), f32(np.concatenate(vs)), f32(np.concatenate(ws))
    R = torch.tensor(Rmin + dR * np.arange(NR), dtype=torch.float64)
    I_t = f32(ring_profile_t(torch.tensor(TRUTH, dtype=torch.float64), R, dR).numpy())
    p_t = f32(TRUTH[3:])
    V = g.double.sampleProfile(I_t, Rmin, dR, NXY, dxy, u, v, inc=p_t[0], PA=p_t[1], dRA=p_t[2], dDec=p_t[3])
    re = f32(V.real + np.concatenate(nre))
    im = f32(V.imag + np.concatenate(nim))
    ds = Dataset(*[[a[cuts[k]:cuts[k + 1]] for k in range(8)] for a in (u, v, re, im, w)])
    return dict(u=u, v=v, re=re, im=im, w=w, cuts=cuts, ds=ds, dxy=dxy, Rmin=Rmin, dR=dR, R=R)


def test_config3_chi2_per_set_256_walkers(sets, oracle_port):
    import torch
    from galario_gb300.batch import chi2_profile_batch, status
    from grad_conditioning import ring_profile_t
    c = sets
    B = 256
    rng = np.random.default_rng(7)
    theta = np.c_[rng.uniform(0.1, 0.8, B), rng.uniform(0.01, 0.1, B), rng.uniform(0.05, 0.2, B),
                  rng.uniform(0, 70, B) * deg, rng.uniform(0, 180, B) * deg, np.zeros(B), np.zeros(B)]
    prof = torch.stack([ring_profile_t(torch.tensor(t), c["R"], c["dR"]) for t in theta]).float()
    tp = torch.tensor(theta[:, 3:], dtype=torch.float32)
    table = chi2_profile_batch(c["ds"], prof.cuda(), tp.cuda(), c["Rmin"], c["dR"], c["dxy"], NXY,
                               per_set=True).cpu().numpy()
    assert status() == 0
    assert table.shape == (B, 8)
    orc = oracle_port.get("port", "double")
    worst = 0.0
    for b in range(0, B, 16):
        I = prof[b].double().numpy()
        inc, PA = (float(x) for x in tp[b, :2].double())
        for k in range(8):
            s = slice(c["cuts"][k], c["cuts"][k + 1])
            ref = orc.chi2Profile(I, c["Rmin"], c["dR"], NXY, c["dxy"], c["u"][s], c["v"][s], c["re"][s],
                                  c["im"][s], c["w"][s], inc=inc, PA=PA)
            rel = abs(table[b, k] - ref) / ref
            worst = max(worst, rel)
            assert rel <= CHI2_TOL, (b, k, table[b, k], ref, rel)
    print("config 3: worst per-set relative chi2 %.2e over 16 walkers x 8 sets" % worst)


@pytest.fixture(scope="module")
def walkers64():
    rng = np.random.default_rng(5)
    B = 64
    th = np.c_[rng.uniform(0.1, 0.8, B), rng.uniform(0.01, 0.1, B), rng.uniform(0.05, 0.2, B),
               rng.uniform(0, 70, B) * deg, rng.uniform(0, 180, B) * deg, rng.uniform(-0.05, 0.05, (B, 2)) * arcsec]
    th[-8:] = np.array(TRUTH) * (1 + rng.uniform(-1e-3, 1e-3, (8, 7)))  # 8 walkers near the optimum
    return th


def test_config4_parameter_gradient_vs_torch_fp64(sets, walkers64):
    """d(sum chi2)/d theta of 64 ring walkers over the 8 sets; 16 of them
    (8 far from the optimum, 8 near it) against the float64 reference."""
    import torch
    from grad_conditioning import NAMES, gpu_gradient, reference_gradient
    c = sets
    geo = dict(nxy=NXY, dxy=c["dxy"], Rmin=c["Rmin"], dR=c["dR"], R=c["R"].cuda())
    thetas = torch.tensor(walkers64, dtype=torch.float64)
    chi2, grad = gpu_gradient(thetas, dict(geo, R=c["R"]), c["ds"])
    t = {k: torch.tensor(c[k], device="cuda") for k in ("u", "v", "re", "im", "w")}
    ratios, met = [], 0
    for b in list(range(8)) + list(range(56, 64)):
        ref_chi2, g, kappa, _, amb_chi2, amb_g = reference_gradient(thetas[b].cuda(), geo, t["u"], t["v"], t["re"],
                                                                   t["im"], t["w"])
        assert abs(chi2[b] - ref_chi2) <= CHI2_TOL * ref_chi2 + amb_chi2, (b, chi2[b], ref_chi2, amb_chi2)
        for j in range(7):
            rel = abs(grad[b, j] - g[j]) / abs(g[j])
            ratios.append(rel / (U32 * kappa[j]))
            met += rel <= 1e-6
            assert abs(grad[b, j] - g[j]) <= KAPPA_C * U32 * kappa[j] * abs(g[j]) + amb_g[j], \
                (b, NAMES[j], rel, kappa[j], amb_g[j] / abs(g[j]))
    print("config 4: error / (2^-24 kappa) median %.1f max %.1f; %d of %d components within 1e-6"
          % (np.median(ratios), np.max(ratios), met, len(ratios)))


def test_config4_parameter_gradient_vs_fd_oracle(sets, walkers64, oracle_port):
    """FP64 central finite differences of the oracle's chi2Profile over all 8
    sets, for two walkers.  The step is 1e-9 relative: chi2 of the reference
    jumps where a visibility's interpolated real spectrum changes sign
    (V = A sign(z)), and a step of 1e-6 relative already crosses such a jump
    on 7.7M visibilities (it moved d chi2/d r0 by 7 % for walker 3); the FP64
    evaluation noise at 1e-9 is about 1e-6 of the gradient."""
    import torch
    from grad_conditioning import gpu_gradient, reference_gradient, ring_profile_t
    c = sets
    orc = oracle_port.get("port", "double")
    geo = dict(nxy=NXY, dxy=c["dxy"], Rmin=c["Rmin"], dR=c["dR"], R=c["R"].cuda())
    idx = [3, 60]
    thetas = torch.tensor(walkers64[idx], dtype=torch.float64)
    _, grad = gpu_gradient(thetas, dict(geo, R=c["R"]), c["ds"])
    t = {k: torch.tensor(c[k], device="cuda") for k in ("u", "v", "re", "im", "w")}

    def chi2_at(th):
        # the float64 model: float32 rounding of a 1e-6 perturbation would be
        # a step function (the gradient at the rounded point differs by O(1e-7))
        I = ring_profile_t(torch.tensor(th), c["R"], c["dR"]).numpy()
        return orc.chi2Profile(I, c["Rmin"], c["dR"], NXY, c["dxy"], c["u"], c["v"], c["re"], c["im"], c["w"],
                               inc=th[3], PA=th[4], dRA=th[5], dDec=th[6])

    for i, b in enumerate(idx):
        _, _, kappa, _, _, amb_g = reference_gradient(thetas[i].cuda(), geo, t["u"], t["v"], t["re"], t["im"],
                                                       t["w"])
        base = walkers64[b]
        scale = (1.0, 1.0, 1.0, 1.0, 1.0, arcsec, arcsec)  # floors of the step: 1e-9 of these
        for j in range(7):
            h = 1e-9 * max(abs(base[j]), scale[j])
            pp, pm = base.copy(), base.copy()
            pp[j] += h
            pm[j] -= h
            fd = (chi2_at(pp) - chi2_at(pm)) / (2 * h)
            assert abs(grad[i, j] - fd) <= (KAPPA_C * U32 * kappa[j] + 1e-5) * abs(fd) + amb_g[j], \
                (b, j, grad[i, j], fd)


def test_config4_pixel_gradient_2048(sets):
    """The gradient of chi2 with respect to all 2048^2 pixels of two
    free-form images against the float64 torch reference."""
    import torch
    from galario_gb300.batch import chi2_image_batch
    from torch_reference import sample_image_t
    c = sets
    dxy = c["dxy"]
    rng = np.random.default_rng(8)
    x = (np.arange(NXY) - NXY / 2) * dxy
    rad = np.hypot(x[None, :], x[:, None])
    imgs, prm = [], []
    for b in range(2):
        ring = np.exp(-0.5 * ((rad - rng.uniform(0.2, 0.8) * arcsec) / (rng.uniform(0.03, 0.1) * arcsec)) ** 2)
        ring += rng.normal(0, 1e-4, ring.shape)
        imgs.append(f32(ring * (0.1 / ring.sum())))
        prm.append(f32([rng.uniform(0, np.pi), rng.uniform(-0.05, 0.05) * arcsec, rng.uniform(-0.05, 0.05) * arcsec]))
    ti = torch.tensor(np.array(imgs), dtype=torch.float32, device="cuda")
    tp = torch.tensor(np.array(prm), dtype=torch.float32, device="cuda")
    chi2, gI, gp = chi2_image_batch(c["ds"], ti, tp, dxy, grad=True)
    t = {k: torch.tensor(c[k], device="cuda") for k in ("u", "v", "re", "im", "w")}
    for b in range(2):
        img = torch.tensor(imgs[b], device="cuda", requires_grad=True)
        p = torch.tensor(prm[b], device="cuda", requires_grad=True)
        V = sample_image_t(img, dxy, t["u"], t["v"], p[0], p[1], p[2])
        ref = torch.sum(t["w"] * ((V.real - t["re"]) ** 2 + (V.imag - t["im"]) ** 2))
        ref.backward()
        assert abs(float(chi2[b]) - float(ref)) / float(ref) <= CHI2_TOL
        gref = img.grad.double()
        rel = float(torch.linalg.norm(gI[b].double() - gref) / torch.linalg.norm(gref))
        print("config 4 images: pixel-gradient relative 2-norm error %.2e (image %d)" % (rel, b))
        assert rel <= 2e-2, (b, rel)
