"""Cell-grid neighbour search (ksg_grid.cuh) against the oracle: the grid
only skips frames whose cells cannot reach a query, so every output must be
bit-identical to the exhaustive kernel's and the reference's."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _detail(xa, xb, n, k, d):
    from netsci_gb300 import device
    X, m = device.pack_trajectory(np.stack([xa, xb]).reshape(2, d * n), d)
    return device.ksg_pair_detail(X[0], X[1], m, k, d)


@pytest.fixture
def grid_search():
    from netsci_gb300 import device
    device.set_ksg_search(1)
    yield
    device.set_ksg_search(-1)


@pytest.mark.parametrize("d,k,n", [(1, 4, 2500), (2, 6, 3001), (3, 6, 4096), (3, 1, 2100),
                                   (3, 17, 2600), (2, 31, 2200), (3, 62, 2300), (3, 6, 50),
                                   (1, 3, 9), (2, 5, 300)])
def test_grid_matches_oracle_per_sample(oracle_mod, grid_search, d, k, n):
    rng = np.random.default_rng(d * 1000 + k + n)
    xa = rng.standard_normal(d * n).astype(np.float32)
    xb = (0.6 * xa + rng.standard_normal(d * n)).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
    out = _detail(xa, xb, n, k, d)
    for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
        assert np.array_equal(out[key].cpu().numpy(), det[key]), key
    assert float(out["mi"].item()) == mi


@pytest.mark.parametrize("d,k", [(1, 4), (2, 6), (3, 6), (3, 10)])
def test_grid_ties_follow_reference(oracle_mod, grid_search, d, k):
    """Coarse-grid coordinates: many equal distances and equal edges."""
    n = 2600
    rng = np.random.default_rng(d * 31 + k)
    xa = (np.round(rng.standard_normal(d * n) * 8) / 8).astype(np.float32)
    xb = (np.round((0.5 * xa + rng.standard_normal(d * n)) * 8) / 8).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
    assert det["ties"] > 0
    out = _detail(xa, xb, n, k, d)
    for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
        assert np.array_equal(out[key].cpu().numpy(), det[key]), key
    assert float(out["mi"].item()) == mi


def test_grid_plan_protein_uneven(oracle_mod):
    """Automatic choice picks the grid for large m; pairs of several
    trajectories with different m in one plan; graph replay."""
    from netsci_gb300 import device, synthetic
    pairs, expect, keep = [], [], []
    for t, (N, m) in enumerate(((6, 2048), (5, 3333), (4, 5000))):
        X, _ = synthetic.protein_trajectory(N, m, seed=50 + t)
        Xd, mm = device.pack_trajectory(X, 3)
        keep.append(Xd)
        ab = synthetic.all_pairs(N)
        pairs += device.make_pairs(Xd, mm, ab)
        expect += list(oracle_mod.pairs(X, m, 3, ab, 6, gc=False, threads=8))
    mi = torch.empty(len(pairs), device="cuda")
    plan = device.KsgPlan(pairs, 6, 3, mi=mi, graph=True)
    assert plan.shape["search"] == "cell-grid"
    for _ in range(2):
        mi.zero_()
        plan.run()
        torch.cuda.synchronize()
        plan.check()
        assert np.array_equal(mi.cpu().numpy(), np.asarray(expect, np.float32))


def test_grid_and_exhaustive_agree_large(grid_search):
    """m = 10000 (the large configuration's frame count): grid == exhaustive."""
    from netsci_gb300 import device, synthetic
    X, _ = synthetic.protein_trajectory(8, 10000, seed=81)
    Xd, m = device.pack_trajectory(X, 3)
    pairs = device.make_pairs(Xd, m, synthetic.all_pairs(8))
    g = torch.empty(len(pairs), device="cuda")
    plan = device.KsgPlan(pairs, 6, 3, gc=g)
    assert plan.shape["search"] == "cell-grid"
    plan.run()
    torch.cuda.synchronize()
    device.set_ksg_search(0)
    e = torch.empty(len(pairs), device="cuda")
    plan0 = device.KsgPlan(pairs, 6, 3, gc=e)
    assert plan0.shape["search"] == "exhaustive"
    plan0.run()
    torch.cuda.synchronize()
    assert np.array_equal(g.cpu().numpy(), e.cpu().numpy())


@pytest.mark.parametrize("d,k,n", [(1, 4, 3000), (2, 6, 2600), (3, 5, 2100)])
def test_grid_query_orders_forced_match_oracle(oracle_mod, grid_search, d, k, n):
    """Query orders forced on for small plans (the planner would skip them):
    the search's block order and the counts' box order, for one, two and
    three coordinates per node (one coordinate: node grids without a second
    axis). Orders only change the scan, so MI equals the oracle's."""
    from netsci_gb300 import device, synthetic
    rng = np.random.default_rng(d * 100 + k)
    N = 5
    base = rng.standard_normal((N, d, n)).astype(np.float32)
    mix = rng.standard_normal((N, N)).astype(np.float32) * 0.6
    X = np.ascontiguousarray(np.einsum("ab,bcn->acn", mix, base).reshape(N, d * n))
    ab = synthetic.all_pairs(N)
    expect = np.asarray(oracle_mod.pairs(X, n, d, ab, k, gc=False, threads=8), np.float32)
    device.set_ksg_orders(1)
    try:
        Xd, m = device.pack_trajectory(X, d)
        mi = torch.empty(len(ab), device="cuda")
        plan = device.KsgPlan(device.make_pairs(Xd, m, ab), k, d, mi=mi)
        assert plan.shape["search"] == "cell-grid"
        plan.run()
        torch.cuda.synchronize()
        plan.check()
        plan.close()
    finally:
        device.set_ksg_orders(-1)
    assert np.array_equal(mi.cpu().numpy(), expect)


@pytest.mark.parametrize("k", [6, 17])
def test_grid_tie_record_matches_rescan(oracle_mod, grid_search, k):
    """Resampled rows tie on many samples (copies of one frame). A plan of
    frame-mapped pairs checks ties through the record kept during the scan;
    a plan of the same rows copied out by hand checks them by scanning again.
    Both must list the same tied samples and give the oracle's MI."""
    from netsci_gb300 import device, synthetic
    N, m = 5, 2300
    X, _ = synthetic.protein_trajectory(N, m, seed=11)
    Xd, mm = device.pack_trajectory(X, 3)
    ab = synthetic.all_pairs(N)
    idx = np.random.default_rng(12).integers(0, m, size=m).astype(np.int32)
    fmap = torch.from_numpy(idx).cuda()
    Xr = np.ascontiguousarray(X.reshape(N, 3, m)[:, :, idx].reshape(N, 3 * m))
    Xrd, _ = device.pack_trajectory(Xr, 3)
    out = []
    for pairs in (device.make_pairs(Xd, mm, ab, fmap=fmap, m_samples=m), device.make_pairs(Xrd, mm, ab)):
        mi = torch.empty(len(pairs), device="cuda")
        plan = device.KsgPlan(pairs, k, 3, mi=mi)
        assert plan.shape["search"] == "cell-grid"
        plan.run()
        torch.cuda.synchronize()
        plan.check()
        out.append((mi.cpu().numpy(), plan.tied_samples()))
        plan.close()
    expect = np.asarray(oracle_mod.pairs(Xr, m, 3, ab, k, gc=False, threads=8), np.float32)
    assert np.array_equal(out[0][0], expect)
    assert np.array_equal(out[1][0], expect)
    assert out[0][1] == out[1][1]


def test_grid_two_resamples_one_plan(oracle_mod, grid_search):
    """Pairs of two bootstrap resamples (two frame maps over the same rows)
    in one cell-grid plan: each resampled row is copied out once, and every
    MI equals the oracle's on the resampled data."""
    from netsci_gb300 import device, synthetic
    N, m, k = 4, 2200, 6
    X, _ = synthetic.protein_trajectory(N, m, seed=1)
    Xd, mm = device.pack_trajectory(X, 3)
    rng = np.random.default_rng(2)
    ab = synthetic.all_pairs(N)
    pairs, expect, keep = [], [], []
    for r in range(2):
        idx = rng.integers(0, m, size=m).astype(np.int32)
        fmap = torch.from_numpy(idx).cuda()
        keep.append(fmap)
        pairs += device.make_pairs(Xd, mm, ab, fmap=fmap, m_samples=m)
        Xr = X.reshape(N, 3, m)[:, :, idx].reshape(N, 3 * m)
        expect += list(oracle_mod.pairs(Xr, m, 3, ab, k, gc=False, threads=8))
    mi = torch.empty(len(pairs), device="cuda")
    plan = device.KsgPlan(pairs, k, 3, mi=mi)
    assert plan.shape["search"] == "cell-grid"
    # gather, node grids, then pair grids, search, counts, combine, ties, finalize
    assert plan.launches == 2 + 6
    plan.run()
    torch.cuda.synchronize()
    plan.check()
    assert np.array_equal(mi.cpu().numpy(), np.asarray(expect, np.float32))
