"""uv-table ingest (galario_gb300.uvtable) and the ensemble MCMC driver
(galario_gb300.mcmc): the sampler against an analytic target on the CPU, the
Gaussian-profile posterior through the batched GPU path."""
import os
import subprocess
import sys

import numpy as np
import pytest

from galario_gb300.mcmc import EnsembleSampler
from galario_gb300.uvtable import load_uvtable, write_uvtable

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_uvtable_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    u, v = rng.normal(0, 1e5, 50), rng.normal(0, 1e5, 50)
    re, im, w = rng.normal(0, 1, 50), rng.normal(0, 1, 50), rng.uniform(1, 2, 50)
    p = tmp_path / "t.txt"
    write_uvtable(p, u, v, re, im, w, wle=1e-3, header="a uv-table\nu v Re Im w")
    got = load_uvtable(p, wle=1e-3)
    for a, b in zip(got, (u, v, re, im, w)):
        np.testing.assert_allclose(a, b, rtol=1e-15)
        assert a.flags["C_CONTIGUOUS"] and a.dtype == np.float64


def test_uvtable_rejects_bad_tables(tmp_path):
    p = tmp_path / "bad.txt"
    np.savetxt(p, np.ones((3, 4)))
    with pytest.raises((ValueError, IndexError)):
        load_uvtable(p)
    np.savetxt(p, np.c_[np.ones((3, 4)), -np.ones(3)])
    with pytest.raises(ValueError, match="negative weights"):
        load_uvtable(p)
    with pytest.raises(ValueError, match="wle"):
        load_uvtable(p, wle=0)


def test_sampler_recovers_gaussian_target():
    mean = np.array([1.0, -2.0, 0.5])
    cov = np.array([[1.0, 0.6, 0.0], [0.6, 2.0, 0.3], [0.0, 0.3, 0.5]])
    icov = np.linalg.inv(cov)

    def logp(X):
        d = X - mean
        return -0.5 * np.einsum("ni,ij,nj->n", d, icov, d)
    s = EnsembleSampler(32, 3, logp, seed=1)
    X0 = mean + np.random.default_rng(2).normal(0, 1e-2, (32, 3))
    s.run(X0, 3000)
    flat = s.get_chain(discard=500, flat=True)
    np.testing.assert_allclose(flat.mean(axis=0), mean, atol=0.15)
    np.testing.assert_allclose(np.cov(flat.T), cov, atol=0.25)
    assert 0.2 < s.acceptance_fraction.mean() < 0.9


def test_sampler_rejects_bad_setup():
    with pytest.raises(ValueError):
        EnsembleSampler(5, 3, lambda X: np.zeros(len(X)))
    with pytest.raises(ValueError):
        EnsembleSampler(8, 3, lambda X: np.zeros(len(X)), a=1.0)


def _synthetic_table(path):
    import galario_gb300 as g
    from helpers import uv_log_uniform
    arcsec, deg = g.arcsec, g.deg
    nxy, dxy = 512, 0.01 * arcsec
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(20000, 0.5 * duv, 0.4 * nxy / 2 * duv, seed=5)
    Rmin, dR, nR = 1e-4 * arcsec, 5e-4 * arcsec, 4000  # (dxy/2 - Rmin)/dR = 9.8 >= 5
    R = Rmin + dR * np.arange(nR)
    truth = np.array([10.3, 0.4, 35.0, 60.0, 0.05, -0.08])
    I = 10 ** truth[0] * np.exp(-0.5 * (R / (truth[1] * arcsec)) ** 2)
    vis = g.double.sampleProfile(I, Rmin, dR, nxy, dxy, u, v, inc=truth[2] * deg, PA=truth[3] * deg,
                                 dRA=truth[4] * arcsec, dDec=truth[5] * arcsec)
    rng = np.random.default_rng(6)
    sigma = 0.05 * np.abs(vis).max()
    write_uvtable(path, u, v, vis.real + rng.normal(0, sigma, len(u)), vis.imag + rng.normal(0, sigma, len(u)),
                  np.full(len(u), 1 / sigma ** 2), wle=1e-3)
    return truth, (Rmin, dR, nR, nxy, dxy)


@pytest.mark.gpu
def test_mcmc_recovers_gaussian_profile(tmp_path):
    from galario_gb300.batch import Dataset
    from galario_gb300.mcmc import GaussianProfileModel
    p = tmp_path / "uv.txt"
    truth, (Rmin, dR, nR, nxy, dxy) = _synthetic_table(p)
    u, v, re, im, w = load_uvtable(p, wle=1e-3)
    ds = Dataset(u, v, re, im, w)
    ranges = [[8, 12], [0.05, 2], [0, 90], [0, 180], [-1, 1], [-1, 1]]
    model = GaussianProfileModel(ds, ranges, Rmin, dR, nR, nxy, dxy)
    rng = np.random.default_rng(3)
    X0 = truth + rng.normal(0, 1, (24, 6)) * np.array([0.01, 0.005, 0.5, 0.5, 0.005, 0.005])
    s = EnsembleSampler(24, 6, model, seed=4)
    s.run(X0, 200)
    flat = s.get_chain(discard=100, flat=True)
    med, sd = np.median(flat, axis=0), flat.std(axis=0)
    assert np.all(np.abs(med - truth) <= 5 * sd + 1e-9), (med, truth, sd)
    assert 0.1 < s.acceptance_fraction.mean() < 0.9
    assert 0.99 * (24 + 200 * 24) <= model.evals <= 24 + 200 * 24  # proposals inside the prior box


@pytest.mark.gpu
def test_mcmc_command_line(tmp_path):
    p = tmp_path / "uv.txt"
    _synthetic_table(p)
    out = subprocess.run([sys.executable, "-m", "galario_gb300.mcmc", "--uvtable", str(p), "--wle", "1e-3",
                          "--steps", "20", "--walkers", "16"], cwd=ROOT, check=True, capture_output=True,
                         text=True).stdout
    assert "acceptance fraction" in out and "log10_f0" in out
