"""An ensemble MCMC driver over the batched chi2 (the workflow of galario's
quickstart, reference docs/quickstart.rst:100-200, with the walkers evaluated
together on the GPU instead of one chi2Profile call per walker).

``EnsembleSampler`` is the affine-invariant stretch-move sampler of Goodman &
Weare (2010, Comm. App. Math. Comp. Sci. 5, 65), the algorithm the emcee
package implements: the walkers are split into two halves; every walker of
one half proposes Y = X_j + z (X_k - X_j) towards a random walker X_j of the
other half, z drawn from g(z) ~ 1/sqrt(z) on [1/a, a], and accepts with
probability min(1, z^(D-1) p(Y) / p(X_k)).  The log-probability is called
once per half-step with all proposals of that half, so one batched chi2 call
evaluates nwalkers/2 models.

``GaussianProfileModel`` is the quickstart's model: a Gaussian radial profile
f0 exp(-R^2 / (2 sigma^2)) with parameters (log10 f0 [Jy/sr], sigma
[arcsec], inc [deg], PA [deg], dRA [arcsec], dDec [arcsec]), uniform priors
on a box, log-posterior -chi2/2.

    python -m galario_gb300.mcmc --uvtable uvtable.txt --wle 1e-3 --steps 500
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from ._module import arcsec, deg


class EnsembleSampler:
    """Stretch-move ensemble sampler; ``log_prob(X)`` maps (n, D) -> (n,)."""

    def __init__(self, nwalkers: int, ndim: int, log_prob, a: float = 2.0, seed: int = 0):
        if nwalkers < 2 * ndim or nwalkers % 2:
            raise ValueError("need an even number of walkers, at least 2 * ndim")
        if not a > 1:
            raise ValueError("the stretch scale a must exceed 1")
        self.nwalkers, self.ndim, self.log_prob, self.a = nwalkers, ndim, log_prob, a
        self.rng = np.random.default_rng(seed)
        self.chain = []
        self.log_probs = []
        self.accepted = np.zeros(nwalkers)
        self.steps = 0

    def _lp(self, X):
        return np.asarray(self.log_prob(X), dtype=np.float64).reshape(-1)

    def run(self, X0, nsteps: int):
        X = np.array(X0, dtype=np.float64, copy=True)
        if X.shape != (self.nwalkers, self.ndim):
            raise ValueError("X0 must be (nwalkers, ndim)")
        lp = self._lp(X)
        half = self.nwalkers // 2
        halves = (np.arange(half), np.arange(half, self.nwalkers))
        for _ in range(nsteps):
            for s in (0, 1):
                act, oth = halves[s], halves[1 - s]
                z = ((self.a - 1.0) * self.rng.random(half) + 1.0) ** 2 / self.a
                partner = X[self.rng.choice(oth, half)]
                Y = partner + z[:, None] * (X[act] - partner)
                lpy = self._lp(Y)
                log_r = (self.ndim - 1) * np.log(z) + lpy - lp[act]
                acc = np.log(self.rng.random(half)) < log_r
                X[act[acc]] = Y[acc]
                lp[act[acc]] = lpy[acc]
                self.accepted[act[acc]] += 1
            self.chain.append(X.copy())
            self.log_probs.append(lp.copy())
            self.steps += 1
        return X, lp

    @property
    def acceptance_fraction(self):
        return self.accepted / max(self.steps, 1)

    def get_chain(self, discard: int = 0, flat: bool = False):
        c = np.array(self.chain[discard:])
        return c.reshape(-1, self.ndim) if flat else c


class GaussianProfileModel:
    """Log-posterior of the quickstart's Gaussian profile, evaluated batched on the GPU."""

    names = ("log10_f0", "sigma_arcsec", "inc_deg", "PA_deg", "dRA_arcsec", "dDec_arcsec")

    def __init__(self, dataset, p_ranges, Rmin, dR, nR, nxy, dxy):
        import torch
        self.ds = dataset
        self.p_ranges = np.asarray(p_ranges, dtype=np.float64)
        if self.p_ranges.shape != (6, 2):
            raise ValueError("p_ranges must be 6 (low, high) pairs")
        self.Rmin, self.dR, self.nR, self.nxy, self.dxy = Rmin, dR, nR, nxy, dxy
        self.R = torch.tensor(Rmin + dR * np.arange(nR), dtype=torch.float64, device="cuda")
        self.evals = 0

    def profiles(self, P):
        """(B, 6) parameters -> (B, nR) intensity [Jy/sr] and (B, 4) (inc, PA, dRA, dDec) [rad]."""
        import torch
        t = torch.as_tensor(P, dtype=torch.float64, device="cuda")
        f0 = 10.0 ** t[:, 0:1]
        sig = t[:, 1:2] * arcsec
        I = f0 * torch.exp(-0.5 * (self.R[None, :] / sig) ** 2)
        geo = torch.stack([t[:, 2] * deg, t[:, 3] * deg, t[:, 4] * arcsec, t[:, 5] * arcsec], dim=1)
        return I.float(), geo.float()

    def __call__(self, P):
        from .batch import chi2_profile_batch
        P = np.asarray(P, dtype=np.float64)
        lo, hi = self.p_ranges[:, 0], self.p_ranges[:, 1]
        inside = np.all((P >= lo) & (P <= hi), axis=1)
        out = np.full(len(P), -np.inf)
        if inside.any():
            I, geo = self.profiles(P[inside])
            chi2 = chi2_profile_batch(self.ds, I, geo, self.Rmin, self.dR, self.dxy, self.nxy)
            out[inside] = -0.5 * chi2.cpu().numpy()
            self.evals += int(inside.sum())
        return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--uvtable", required=True, help="u, v, Re, Im, w table (see galario_gb300.uvtable)")
    ap.add_argument("--wle", type=float, default=1.0, help="observing wavelength [m] dividing u, v")
    ap.add_argument("--walkers", type=int, default=40)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    from . import double
    from .batch import Dataset
    from .uvtable import load_uvtable
    u, v, re, im, w = load_uvtable(args.uvtable, args.wle)
    nxy, dxy = double.get_image_size(u, v)
    Rmin, dR, nR = 1e-4 * arcsec, 1e-3 * arcsec, 2000
    # the batched path needs a power-of-two image at least as large as the one galario picks
    nxy = 1 << int(math.ceil(math.log2(nxy)))
    while ((dxy / 2 - Rmin) / dR) < 5:
        dR /= 2
    ds = Dataset(u, v, re, im, w)
    p_ranges = [[1, 20], [0.01, 5], [0, 90], [0, 180], [-2, 2], [-2, 2]]
    model = GaussianProfileModel(ds, p_ranges, Rmin, dR, nR, nxy, dxy)
    rng = np.random.default_rng(args.seed)
    p0 = np.array([10, 0.5, 40, 70, 0, 0])
    X0 = p0 + rng.normal(0, 1e-2, (args.walkers, 6)) * np.array([1, 0.1, 10, 10, 0.1, 0.1])
    sampler = EnsembleSampler(args.walkers, 6, model, seed=args.seed)
    t0 = time.perf_counter()
    sampler.run(X0, args.steps)
    dt = time.perf_counter() - t0
    flat = sampler.get_chain(discard=args.steps // 2, flat=True)
    print("nxy=%d dxy=%.4g arcsec, %d visibilities, %d walkers x %d steps in %.2f s (%.0f chi2 evals/s)"
          % (nxy, dxy / arcsec, len(u), args.walkers, args.steps, dt, model.evals / dt))
    print("acceptance fraction %.3f" % sampler.acceptance_fraction.mean())
    for i, name in enumerate(GaussianProfileModel.names):
        q = np.percentile(flat[:, i], [16, 50, 84])
        print("%-13s %.5g (+%.3g / -%.3g)" % (name, q[1], q[2] - q[1], q[1] - q[0]))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
