"""Bivariate Gaussian MI over 32 seeds (n = 2000, rho = 0.8, d = 1, k = 4;
analytic MI = -ln(1 - rho^2) / 2 = 0.5108): the estimator's mean lies within
its spread of the analytic value, and the GPU equals the reference CPU path
(the oracle) on every seed."""
import math

import numpy as np
import pytest

RHO, N, K, SEEDS = 0.8, 2000, 4, 32
ANALYTIC = -0.5 * math.log(1.0 - RHO * RHO)


def _pairs():
    from netsci_gb300 import synthetic
    return [synthetic.gaussian_pair(N, RHO, seed=s) for s in range(SEEDS)]


def test_oracle_mean_near_analytic(oracle_mod):
    mis = np.array([oracle_mod.mi_pair(x, y, N, K, 1) for x, y in _pairs()], np.float64)
    mean, sd = mis.mean(), mis.std(ddof=1)
    # the KSG estimator's bias at this n and k is well inside its spread
    assert abs(mean - ANALYTIC) <= 4 * sd / math.sqrt(SEEDS) + 0.01, (mean, sd)
    assert 0.0 < sd < 0.05


@pytest.mark.gpu
def test_gpu_equals_oracle_every_seed(oracle_mod):
    import torch
    from netsci_gb300 import device
    xs = _pairs()
    X = np.stack([np.stack([x, y]) for x, y in xs]).reshape(2 * SEEDS, N)
    Xd, m = device.pack_trajectory(X, 1)
    ab = np.array([[2 * s, 2 * s + 1] for s in range(SEEDS)], np.int32)
    pairs = device.make_pairs(Xd, m, ab)
    mi = torch.empty(SEEDS, device="cuda")
    device.ksg_pairs(pairs, K, 1, mi=mi)
    got = mi.cpu().numpy()
    want = np.array([oracle_mod.mi_pair(x, y, N, K, 1) for x, y in xs], np.float32)
    assert np.array_equal(got, want)
    mean, sd = float(want.mean()), float(want.std(ddof=1))
    assert np.all(np.abs(got - mean) <= 4 * sd)
