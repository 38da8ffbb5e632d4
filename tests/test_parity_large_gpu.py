"""GPU against the oracle at the large configuration's sizes.

Per-sample outputs (n_x, n_y, eps_x, eps_y, k-th distance) and MI are
compared bit for bit with the CPU oracle (a restatement of
netcalc/src/mutual_information_cpu.cpp:6-121, pinned to the reference's own
CPU code), on:

* random pairs of the all-pairs workload's trajectory (N = 2000 nodes,
  m = 10000 frames, d = 3, k = 6; the same seeded trajectory bench.py
  times), through the per-pair call, through a plan with and without the
  block query orders, and through the drop-in CuArray API (GC, host
  transform, bit-exact);
* one pair at m = 24000, where a pair grid no longer fits the staged
  (shared-memory) build and is scattered straight to global memory;
* one pair at m = 45000, above the largest m the query orders take (the
  search and counts fall back to the Z order of cells);
* the Gaussian MI requests of the serving mix at their largest size,
  n = 20000, d = 1, k = 4.

The oracle spreads each pair's samples over the host's cores; its sum runs
in sample order, so the result is the single-threaded one."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)
KEYS = ("n_x", "n_y", "eps_x", "eps_y", "kdist")


@pytest.fixture(scope="module")
def c4_trajectory():
    from netsci_gb300 import synthetic
    X, _ = synthetic.protein_trajectory(2000, 10000, seed=2000)
    return X


@pytest.fixture(scope="module")
def c4_pairs():
    from netsci_gb300 import synthetic
    ab = synthetic.all_pairs(2000)
    rng = np.random.default_rng(44)
    return ab[np.sort(rng.choice(len(ab), size=8, replace=False))]


@pytest.fixture(scope="module")
def c4_oracle(oracle_mod, c4_trajectory, c4_pairs):
    X = c4_trajectory
    return [oracle_mod.mi_pair(X[a], X[b], 10000, 6, 3, detail=True, threads=THREADS)
            for a, b in c4_pairs]


@pytest.fixture
def knobs():
    from netsci_gb300 import device
    yield device
    device.set_ksg_search(-1)
    device.set_ksg_orders(-1)


def _detail(xa, xb, n, k, d):
    from netsci_gb300 import device
    X, m = device.pack_trajectory(np.stack([xa, xb]).reshape(2, d * n), d)
    return device.ksg_pair_detail(X[0], X[1], m, k, d)


def _same(out, det, mi):
    for key in KEYS:
        got = out[key].cpu().numpy()
        bad = np.flatnonzero(got != det[key])
        assert bad.size == 0, (key, bad[:5], got[bad[:5]], det[key][bad[:5]])
    assert float(out["mi"].item()) == mi


@pytest.mark.parametrize("search", [1, 0])
def test_c4_random_pairs_per_sample(c4_trajectory, c4_pairs, c4_oracle, knobs, search):
    knobs.set_ksg_search(search)
    X = c4_trajectory
    for (a, b), (mi, det) in zip(c4_pairs, c4_oracle):
        _same(_detail(X[a], X[b], 10000, 6, 3), det, mi)


@pytest.mark.parametrize("orders", [1, 0, -1])
def test_c4_random_pairs_one_plan(c4_trajectory, c4_pairs, c4_oracle, knobs, orders):
    """The bench's path: one autotuned, graph-replayed plan over the pairs,
    with the query orders forced on, off, or left to the planner."""
    knobs.set_ksg_orders(orders)
    Xd, m = knobs.pack_trajectory(c4_trajectory, 3)
    mi = torch.empty(len(c4_pairs), device="cuda")
    plan = knobs.KsgPlan(knobs.make_pairs(Xd, m, c4_pairs), 6, 3, mi=mi, graph=True,
                         autotune=True)
    assert plan.shape["search"] == "cell-grid"
    for _ in range(2):
        mi.fill_(float("nan"))
        plan.run()
        torch.cuda.synchronize()
        plan.check()
        assert np.array_equal(mi.cpu().numpy(), np.asarray([o[0] for o in c4_oracle], np.float32))
    plan.close()


def test_c4_random_pairs_through_cuarray_api(oracle_mod, c4_trajectory, c4_pairs, c4_oracle):
    import cuarray
    import netcalc
    Xc = cuarray.FloatCuArray()
    Xc.fromNumpy2D(c4_trajectory)
    abc = cuarray.IntCuArray()
    abc.fromNumpy2D(np.ascontiguousarray(c4_pairs, np.int32))
    R = cuarray.FloatCuArray()
    assert netcalc.generalizedCorrelation(X=Xc, R=R, ab=abc, k=6, n=10000, xd=2, d=3,
                                          platform=0) == 0
    want = np.asarray([oracle_mod.gc_from_mi(mi, 3) for mi, _ in c4_oracle], np.float32)
    assert np.array_equal(R.toNumpy1D(), want)


@pytest.mark.parametrize("m,seed", [(24000, 24), (45000, 45)])
def test_large_m_pair_per_sample(oracle_mod, knobs, m, seed):
    from netsci_gb300 import synthetic
    X, _ = synthetic.protein_trajectory(3, m, seed=seed)
    mi, det = oracle_mod.mi_pair(X[0], X[2], m, 6, 3, detail=True, threads=THREADS)
    for orders in (1, 0):
        knobs.set_ksg_search(1)
        knobs.set_ksg_orders(orders)
        _same(_detail(X[0], X[2], m, 6, 3), det, mi)


def test_block_orders_at_their_largest_m_on_a_correlated_pair(oracle_mod, knobs):
    """m = 40960, the largest m the query orders take, on a pair whose two
    rows are nearly the same motion: its frames crowd the diagonal blocks of
    the pair grid, the case that made ranking a query against its whole
    block quadratic. The orders are built by counting sort now; every
    per-sample output still equals the oracle's."""
    from netsci_gb300 import synthetic
    m = 40960
    X, _ = synthetic.protein_trajectory(2, m, seed=4096)
    rng = np.random.default_rng(4096)
    xa = X[0]
    xb = (xa + 0.05 * rng.standard_normal(xa.size)).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, m, 6, 3, detail=True, threads=THREADS)
    knobs.set_ksg_search(1)
    knobs.set_ksg_orders(1)
    _same(_detail(xa, xb, m, 6, 3), det, mi)


def test_gaussian_mi_largest_request(oracle_mod, knobs):
    """The serving mix's Gaussian MI at n = 20000, d = 1, k = 4, on both
    searches and through the reference's per-pair call."""
    import cuarray
    import netcalc
    from netsci_gb300 import synthetic
    n = 20000
    x, y = synthetic.gaussian_pair(n, 0.95, seed=2020)
    mi, det = oracle_mod.mi_pair(x, y, n, 4, 1, detail=True, threads=THREADS)
    for search in (1, 0):
        knobs.set_ksg_search(search)
        _same(_detail(x, y, n, 4, 1), det, mi)
    knobs.set_ksg_search(-1)
    xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    xa.fromNumpy1D(x)
    xb.fromNumpy1D(y)
    assert netcalc.mutualInformationGpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=1) == mi
