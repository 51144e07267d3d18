"""Replica sharding (galario_gb300.replicas) on CPU: world_size 2 over gloo.

Every process evaluates its share with the CPU oracle standing in for the GPU
batched path; the combined results must equal one process evaluating all.
"""
import os
import socket
import sys

import numpy as np
import pytest

from galario_gb300.replicas import ModelShards, SetShards, shard_bounds

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_bounds_partition():
    for n in (0, 1, 5, 64, 257):
        for world in (1, 2, 3, 8):
            b = [shard_bounds(n, r, world) for r in range(world)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in b]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def _problem():
    from helpers import arcsec, uv_log_uniform
    nxy, dxy = 128, 0.05 * arcsec
    Rmin, dR, nr = 1e-4 * arcsec, 4e-3 * arcsec, 600
    duv = 1 / (nxy * dxy)
    u, v = uv_log_uniform(3000, 0.5 * duv, 0.4 * nxy / 2 * duv, seed=3)
    rng = np.random.default_rng(4)
    re, im = rng.normal(0, 1e-3, len(u)), rng.normal(0, 1e-3, len(u))
    w = rng.uniform(0.5, 2, len(u)) * 1e6
    R = Rmin + dR * np.arange(nr)
    B = 5
    I = np.array([np.exp(-0.5 * ((R - (0.3 + 0.1 * b) * arcsec) / (0.1 * arcsec)) ** 2) * 1e10 for b in range(B)])
    params = np.array([[0.1 * b, 0.3 * b, 0.01 * arcsec, -0.02 * arcsec] for b in range(B)])
    sets = [slice(0, 700), slice(700, 2100), slice(2100, 3000)]
    return dict(nxy=nxy, dxy=dxy, Rmin=Rmin, dR=dR, u=u, v=v, re=re, im=im, w=w, I=I, params=params, sets=sets)


def _chi2(orc, P, b, sl):
    inc, PA, dRA, dDec = P["params"][b]
    return orc.chi2Profile(P["I"][b], P["Rmin"], P["dR"], P["nxy"], P["dxy"], P["u"][sl], P["v"][sl], P["re"][sl],
                           P["im"][sl], P["w"][sl], inc=inc, PA=PA, dRA=dRA, dDec=dDec)


def _worker(rank, world, port, outdir):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        orc = O.get("port", "double")
        P = _problem()
        B = len(P["I"])

        def by_models(lo, hi):
            chi2 = torch.tensor([_chi2(orc, P, b, slice(None)) for b in range(lo, hi)], dtype=torch.float64)
            # a second output with a trailing dimension, as a gradient would have
            extra = torch.tensor(P["params"][lo:hi], dtype=torch.float64) * chi2[:, None]
            return chi2, extra
        chi2_m, extra_m = ModelShards(by_models)(B)

        def by_sets(share):
            lo, hi = share
            chi2 = torch.zeros(B, dtype=torch.float64)
            for k in range(lo, hi):
                chi2 += torch.tensor([_chi2(orc, P, b, P["sets"][k]) for b in range(B)], dtype=torch.float64)
            return chi2
        chi2_s = SetShards(by_sets, nsets=len(P["sets"]))()
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), chi2_m=chi2_m.numpy(), extra_m=extra_m.numpy(),
                 chi2_s=chi2_s.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replicas_world2_gloo(tmp_path, oracle_port):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    orc = oracle_port.get("port", "double")
    P = _problem()
    B = len(P["I"])
    full = np.array([_chi2(orc, P, b, slice(None)) for b in range(B)])
    by_set = np.array([sum(_chi2(orc, P, b, sl) for sl in P["sets"]) for b in range(B)])
    for r in range(world):
        out = np.load(tmp_path / f"rank{r}.npz")
        np.testing.assert_allclose(out["chi2_m"], full, rtol=1e-14)  # gathered (the oracle reduces with threads)
        np.testing.assert_allclose(out["extra_m"], P["params"] * full[:, None], rtol=1e-15)
        np.testing.assert_allclose(out["chi2_s"], by_set, rtol=1e-13)  # summed over the two shards
    np.testing.assert_allclose(by_set, full, rtol=1e-10)  # chi2 is additive over the sets


def test_replicas_single_process_passthrough():
    import torch
    r = ModelShards(lambda lo, hi: torch.arange(lo, hi, dtype=torch.float64))(7)
    assert r.tolist() == list(range(7))
    s = SetShards(lambda share: torch.tensor([float(share[1] - share[0])]), nsets=3)()
    assert s.tolist() == [3.0]
