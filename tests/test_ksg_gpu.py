"""KSG mutual information / generalized correlation on the GPU against the
CPU oracle and the reference's golden values.

Bar: MI bit-exact (the kernels reproduce the reference's distances, counts
and float summation order), per-sample n_x / n_y / eps bit-exact, GC
bit-exact through the CuArray API (host transform, as the reference) and
within 1e-6 absolute through the device transform.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN_MI = {1000: 0.8449974060058594, 2000: 0.8485465049743652}


def _dev_pair(xa, xb, d, m):
    """(d, ld) device rows for one pair."""
    from netsci_gb300 import device
    X, mm = device.pack_trajectory(np.stack([xa, xb]).reshape(2, d * m), d)
    assert mm == m
    return X


def _mi_device(xa, xb, m, k, d):
    from netsci_gb300 import device
    X = _dev_pair(xa, xb, d, m)
    return device.ksg_pair_detail(X[0], X[1], m, k, d)


@pytest.mark.parametrize("n", [1000, 2000])
def test_gaussian_goldens_gpu_equals_cpu(golden, n):
    import cuarray
    import netcalc
    g = golden("gaussian")
    xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    xa.fromNumpy1D(g[f"x{n}"])
    xb.fromNumpy1D(g[f"y{n}"])
    gpu = netcalc.mutualInformationGpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=1)
    cpu = netcalc.mutualInformationCpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=1)
    assert gpu == cpu == GOLDEN_MI[n]


@pytest.mark.parametrize("n", [1000, 2000])
def test_per_sample_counts_match_oracle(golden, n):
    g = golden("gaussian")
    out = _mi_device(g[f"x{n}"], g[f"y{n}"], n, 4, 1)
    for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
        got = out[key].cpu().numpy()
        assert np.array_equal(got, g[f"{key}{n}"]), key
    assert float(out["mi"].item()) == GOLDEN_MI[n]


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("n", [1000, 2000])
def test_reference_curves(golden, d, n):
    import cuarray
    import netcalc
    c = golden("curves")
    xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    xa.fromNumpy1D(c[f"xa_d{d}_n{n}"])
    xb.fromNumpy1D(c[f"xb_d{d}_n{n}"])
    mi = netcalc.mutualInformationGpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=d)
    assert mi == float(c[f"mi_d{d}_n{n}"]) == netcalc.mutualInformationCpu(
        Xa=xa, Xb=xb, k=4, n=n, xd=2, d=d)
    gc = netcalc.generalizedCorrelationGpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=d)
    assert gc == float(c[f"gc_d{d}_n{n}"]) == netcalc.generalizedCorrelationCpu(
        Xa=xa, Xb=xb, k=4, n=n, xd=2, d=d)


def test_random_cases_bit_exact(golden):
    r = golden("random")
    for i in range(int(r["count"])):
        d, k, n = (int(v) for v in r[f"meta{i}"])
        out = _mi_device(r[f"xa{i}"], r[f"xb{i}"], n, k, d)
        assert float(out["mi"].item()) == float(r[f"mi{i}"]), (i, d, k, n)


def test_per_sample_outputs_random_vs_oracle(oracle_mod):
    rng = np.random.default_rng(11)
    for d, k, n in ((1, 3, 777), (2, 6, 1031), (3, 6, 1500), (3, 17, 640), (2, 32, 500)):
        xa = rng.standard_normal(d * n).astype(np.float32)
        xb = (0.5 * xa + rng.standard_normal(d * n)).astype(np.float32)
        mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
        out = _mi_device(xa, xb, n, k, d)
        for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
            assert np.array_equal(out[key].cpu().numpy(), det[key]), (d, k, n, key)
        assert float(out["mi"].item()) == mi


SHAPES = [(256, 1, 1024), (128, 1, 1024), (128, 2, 1024), (256, 2, 1024), (64, 1, 512),
          (512, 1, 1024)]


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_every_shape_and_variant_agrees(oracle_mod, variant):
    from netsci_gb300 import device
    rng = np.random.default_rng(3)
    n, k, d = 1500, 6, 3
    xa = rng.standard_normal(d * n).astype(np.float32)
    xb = (0.8 * xa + 0.6 * rng.standard_normal(d * n)).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
    try:
        for shape in SHAPES:
            device.set_ksg_shape(*shape, variant=variant)
            out = _mi_device(xa, xb, n, k, d)
            assert float(out["mi"].item()) == mi, shape
            assert np.array_equal(out["n_x"].cpu().numpy(), det["n_x"]), shape
    finally:
        device.set_ksg_shape(0)


def test_protein56_all_pairs_cuarray_api(golden):
    import cuarray
    import netcalc
    z = golden("protein56")
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(z["X"])
    ab = cuarray.IntCuArray()
    ab.fromNumpy2D(z["ab"])
    R = cuarray.FloatCuArray()
    assert netcalc.generalizedCorrelation(X=X, R=R, ab=ab, k=6, n=1000, xd=2, d=3,
                                          platform=netcalc.GPU_PLATFORM) == 0
    assert np.array_equal(R.toNumpy1D(), z["gc"])


def test_protein56_device_plan_graph(golden, oracle_mod):
    from netsci_gb300 import device
    z = golden("protein56")
    X, m = device.pack_trajectory(z["X"], 3)
    pairs = device.make_pairs(X, m, z["ab"])
    P = len(pairs)
    mi = torch.empty(P, device="cuda")
    gc = torch.empty(P, device="cuda")
    w = torch.empty(P, device="cuda")
    plan = device.KsgPlan(pairs, 6, 3, mi=mi, gc=gc, w=w, graph=True)
    plan.run()
    torch.cuda.synchronize()
    g1 = gc.cpu().numpy()
    np.testing.assert_allclose(g1, z["gc"], rtol=0, atol=1e-6)
    assert (g1 == z["gc"]).mean() > 0.999  # device exp/sqrt may differ in the last bit
    mis = mi.cpu().numpy()
    for p in (0, 100, 1539):
        a, b = z["ab"][p]
        assert mis[p] == oracle_mod.mi_pair(z["X"][a], z["X"][b], 1000, 6, 3)
    wv = w.cpu().numpy()
    ref_w = np.where(g1 > 0, (-np.log(g1.astype(np.float64))).astype(np.float32), np.inf)
    np.testing.assert_array_max_ulp(wv[np.isfinite(ref_w)], ref_w[np.isfinite(ref_w)], maxulp=1)
    assert np.all(np.isinf(wv[~np.isfinite(ref_w)]))
    # replays are deterministic
    for _ in range(2):
        gc.zero_()
        plan.run()
        torch.cuda.synchronize()
        assert np.array_equal(gc.cpu().numpy(), g1)
    # exhaustive: count, ties, finalize; cell grids (m = 1000 selects them):
    # node grids, pair grids, search, counts, combine, ties, finalize, and
    # for a batch of at least eight waves of search warps (32 per SM) the node
    # scale estimates and the search and count orders
    if plan.shape["search"] == "cell-grid":
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        ordered = len(pairs) * ((1000 + 31) // 32) >= 8 * 32 * sms
        assert plan.launches == 7 + (3 if ordered else 0)
    else:
        assert plan.launches == 3


def test_uneven_trajectories_one_plan(oracle_mod):
    from netsci_gb300 import device, synthetic
    rng = np.random.default_rng(9)
    pairs, expect, keep = [], [], []
    for t in range(4):
        N = int(rng.integers(4, 8))
        m = int(rng.integers(150, 700))
        X, _ = synthetic.protein_trajectory(N, m, seed=100 + t)
        Xd, mm = device.pack_trajectory(X, 3)
        keep.append(Xd)
        ab = synthetic.all_pairs(N)
        pairs += device.make_pairs(Xd, mm, ab)
        expect += list(oracle_mod.pairs(X, m, 3, ab, 6, gc=False, threads=8))
    mi = torch.empty(len(pairs), device="cuda")
    device.ksg_pairs(pairs, 6, 3, mi=mi)
    assert np.array_equal(mi.cpu().numpy(), np.asarray(expect, np.float32))


def test_bootstrap_frame_map_matches_resampled_data(oracle_mod):
    from netsci_gb300 import device, synthetic
    N, m, k = 6, 400, 6
    X, _ = synthetic.protein_trajectory(N, m, seed=4)
    Xd, mm = device.pack_trajectory(X, 3)
    rng = np.random.default_rng(1)
    idx = rng.integers(0, m, size=m).astype(np.int32)   # with replacement
    fmap = torch.from_numpy(idx).cuda()
    ab = synthetic.all_pairs(N)
    pairs = device.make_pairs(Xd, mm, ab, fmap=fmap, m_samples=m)
    mi = torch.empty(len(pairs), device="cuda")
    device.ksg_pairs(pairs, k, 3, mi=mi)
    Xr = X.reshape(N, 3, m)[:, :, idx].reshape(N, 3 * m)
    expect = oracle_mod.pairs(Xr, m, 3, ab, k, gc=False, threads=8)
    assert np.array_equal(mi.cpu().numpy(), expect)


def test_edge_sizes_and_duplicates(oracle_mod):
    rng = np.random.default_rng(21)
    for d, k, n in ((1, 1, 2), (2, 1, 3), (3, 4, 5), (1, 6, 7), (3, 6, 33), (2, 32, 33),
                    (3, 31, 1029)):
        xa = rng.standard_normal(d * n).astype(np.float32)
        xb = rng.standard_normal(d * n).astype(np.float32)
        mi = oracle_mod.mi_pair(xa, xb, n, k, d)
        assert float(_mi_device(xa, xb, n, k, d)["mi"].item()) == mi, (d, k, n)
    # exact duplicate frames (ties with equal marginals are benign)
    n, d, k = 300, 3, 4
    base = rng.standard_normal((d, n // 3)).astype(np.float32)
    xa = np.concatenate([base, base, base], axis=1).ravel()
    xb = np.concatenate([base * 2, base * 2, base * 2], axis=1).ravel().astype(np.float32)
    mi = oracle_mod.mi_pair(xa, xb, n, k, d)
    assert float(_mi_device(xa, xb, n, k, d)["mi"].item()) == mi


def test_invalid_k_statuses():
    from netsci_gb300 import NsgError, device
    xa = np.random.default_rng(0).standard_normal(200).astype(np.float32)
    X = _dev_pair(xa, xa, 1, 200)
    with pytest.raises(NsgError) as e:
        device.ksg_pair_detail(X[0], X[1], 200, 70, 1)
    assert e.value.status == 4  # k > 62 unsupported on the GPU
    with pytest.raises(NsgError) as e:
        device.ksg_pair_detail(X[0], X[1], 200, 200, 1)
    assert e.value.status == 1  # k >= m


def test_large_pair_properties():
    """m = 10000 (the large configuration's frame count): symmetry in the
    pair order and run-to-run determinism."""
    from netsci_gb300 import device, synthetic
    X, _ = synthetic.protein_trajectory(3, 10000, seed=77)
    Xd, m = device.pack_trajectory(X, 3)
    pairs = device.make_pairs(Xd, m, [[0, 1], [1, 0], [0, 2], [2, 0], [0, 1]])
    mi = torch.empty(5, device="cuda")
    device.ksg_pairs(pairs, 6, 3, mi=mi)
    v = mi.cpu().numpy()
    assert v[0] == v[1] == v[4] and v[2] == v[3]


def test_large_pair_against_oracle_m4000(oracle_mod):
    from netsci_gb300 import synthetic
    X, _ = synthetic.protein_trajectory(2, 4000, seed=78)
    mi = oracle_mod.mi_pair(X[0], X[1], 4000, 6, 3)
    assert float(_mi_device(X[0], X[1], 4000, 6, 3)["mi"].item()) == mi


def test_platform_contract_gpu():
    import cuarray
    import netcalc
    n = 1000
    x = np.linspace(0.001, np.pi, n).astype(np.float32)
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(np.stack([np.sin(x), np.cos(x)]).astype(np.float32))
    I = cuarray.FloatCuArray()
    ab = cuarray.IntCuArray()
    ab.fromNumpy2D(np.array([[0, 1]], np.int32))
    assert netcalc.mutualInformation(X=X, I=I, ab=ab, k=4, n=n, xd=2, d=1,
                                     platform=netcalc.GPU_PLATFORM) == 0
    I2 = cuarray.FloatCuArray()
    assert netcalc.mutualInformation(X=X, I=I2, ab=ab, k=4, n=n, xd=2, d=1,
                                     platform=netcalc.CPU_PLATFORM) == 1
    assert I.get(0, 0) == I2.get(0, 0)


def test_checkpointed_gpu_matches_plain(tmp_path):
    import cuarray
    import netcalc
    from netsci_gb300 import synthetic
    X0, _ = synthetic.protein_trajectory(6, 300, seed=8)
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(X0)
    ab = cuarray.IntCuArray()
    ab.fromNumpy2D(synthetic.all_pairs(6))
    R1, R2 = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    netcalc.generalizedCorrelation(X=X, R=R1, ab=ab, k=6, n=300, xd=2, d=3, platform=0)
    netcalc.generalizedCorrelationWithCheckpointing(
        X=X, R=R2, ab=ab, k=6, n=300, xd=2, d=3, platform=0, checkpointFrequency=4,
        checkpointFileName=str(tmp_path / "run.npy"))
    assert np.array_equal(R1.toNumpy1D(), R2.toNumpy1D())
    assert sorted(p.name for p in tmp_path.iterdir()) == ["run_12.npy", "run_ab.npy"]


@pytest.mark.parametrize("d,k,n", [(1, 4, 700), (2, 6, 900), (3, 6, 1000), (3, 10, 600)])
def test_tied_samples_follow_reference_sort_order(oracle_mod, d, k, n):
    """Coordinates on a coarse grid make many samples' k-th and (k+1)-th
    joint distances equal; the GPU must then pick the neighbours the
    reference's std::sort picks (the oracle makes the reference's call)."""
    rng = np.random.default_rng(d * 100 + k)
    xa = (np.round(rng.standard_normal(d * n) * 8) / 8).astype(np.float32)
    xb = (np.round((0.5 * xa + rng.standard_normal(d * n)) * 8) / 8).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
    assert det["ties"] > 0
    out = _mi_device(xa, xb, n, k, d)
    for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
        assert np.array_equal(out[key].cpu().numpy(), det[key]), key
    assert float(out["mi"].item()) == mi


def test_autotuned_plan_same_results_and_cached(tmp_path, monkeypatch):
    from netsci_gb300 import device, synthetic
    X, _ = synthetic.protein_trajectory(12, 900, seed=31)
    Xd, m = device.pack_trajectory(X, 3)
    pairs = device.make_pairs(Xd, m, synthetic.all_pairs(12))
    a = torch.empty(len(pairs), device="cuda")
    b = torch.empty(len(pairs), device="cuda")
    device.KsgPlan(pairs, 6, 3, mi=a, graph=False).run()
    tuned = device.KsgPlan(pairs, 6, 3, mi=b, graph=True, autotune=True)
    tuned.run()
    torch.cuda.synchronize()
    assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())
    sh = tuned.shape
    assert sh["threads"] in (64, 128, 256, 512) and sh["r"] in (1, 2)


TMA_SHAPES = [(256, 1, 1024), (128, 1, 1024), (512, 1, 1024), (256, 1, 512)]


@pytest.mark.parametrize("d,k", [(1, 4), (2, 6), (3, 6)])
def test_bulk_copy_staging_agrees(oracle_mod, d, k):
    """The bulk-copy (TMA) staged kernels against the oracle at sample counts
    that give one tile, several tiles and ragged tails (m mod 4 = 0..3)."""
    from netsci_gb300 import device
    rng = np.random.default_rng(40 + d)
    try:
        for n in (9, 130, 1023, 1026, 2049, 3075):
            xa = rng.standard_normal(d * n).astype(np.float32)
            xb = (0.6 * xa + rng.standard_normal(d * n)).astype(np.float32)
            mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True)
            for shape in TMA_SHAPES:
                device.set_ksg_shape(*shape)
                device.set_ksg_staging(1)
                out = _mi_device(xa, xb, n, k, d)
                assert float(out["mi"].item()) == mi, (n, shape)
                for key in ("n_x", "n_y", "eps_x", "eps_y"):
                    assert np.array_equal(out[key].cpu().numpy(), det[key]), (n, shape, key)
    finally:
        device.set_ksg_staging(-1)
        device.set_ksg_shape(0)


def test_bulk_copy_plan_many_pairs(oracle_mod):
    """A multi-pair plan with bulk-copy staging, replayed through a graph."""
    from netsci_gb300 import device, synthetic
    X, _ = synthetic.protein_trajectory(9, 1500, seed=12)
    Xd, m = device.pack_trajectory(X, 3)
    ab = synthetic.all_pairs(9)
    pairs = device.make_pairs(Xd, m, ab)
    expect = oracle_mod.pairs(X, m, 3, ab, 6, gc=False, threads=8)
    try:
        device.set_ksg_staging(1)
        mi = torch.empty(len(pairs), device="cuda")
        plan = device.KsgPlan(pairs, 6, 3, mi=mi, graph=True)
        assert plan.shape["staging"] == "bulk-copy"
        for _ in range(2):
            plan.run()
            torch.cuda.synchronize()
            plan.check()
            assert np.array_equal(mi.cpu().numpy(), expect)
    finally:
        device.set_ksg_staging(-1)


def test_bootstrap_duplicates_and_real_ties(oracle_mod):
    """Bootstrap resampling makes copies of frames (ties that cannot change
    eps, not listed) and a coarse grid makes genuine ties (listed and
    resolved in the reference's sort order); both together, on enough pairs
    that listing every tied sample would overflow the tie list."""
    from netsci_gb300 import device
    rng = np.random.default_rng(17)
    N, m, k = 8, 2500, 6
    X = (np.round(rng.standard_normal((N, 3 * m)) * 6) / 6).astype(np.float32)
    X[1::2] = rng.standard_normal((N // 2, 3 * m)).astype(np.float32)
    Xd, mm = device.pack_trajectory(X, 3)
    idx = rng.integers(0, m, size=m).astype(np.int32)
    fmap = torch.from_numpy(idx).cuda()
    ab = np.array([[a, b] for a in range(N) for b in range(N) if a != b], np.int32)
    pairs = device.make_pairs(Xd, mm, ab, fmap=fmap, m_samples=m)
    Xr = X.reshape(N, 3, m)[:, :, idx].reshape(N, 3 * m)
    expect = oracle_mod.pairs(Xr, m, 3, ab, k, gc=False, threads=8)
    # both searches: exhaustive (copies filtered in its count pass) and cell
    # grids (resampled rows copied out; copies filtered in the search pass)
    try:
        for mode, name in ((0, "exhaustive"), (1, "cell-grid")):
            device.set_ksg_search(mode)
            mi = torch.empty(len(pairs), device="cuda")
            plan = device.KsgPlan(pairs, k, 3, mi=mi, graph=True)
            assert plan.shape["search"] == name
            for _ in range(2):
                mi.zero_()
                plan.run()
                torch.cuda.synchronize()
                plan.check()
                assert np.array_equal(mi.cpu().numpy(), expect), name
    finally:
        device.set_ksg_search(-1)


def test_cached_device_memory_reused_and_released(oracle_mod):
    """Plans built one after another reuse the blocks earlier plans freed;
    nsg_release_cached_memory returns them to the driver, and plans built
    afterwards still give the oracle's results."""
    from netsci_gb300 import device, synthetic
    N, m, k = 4, 1500, 6
    X, _ = synthetic.protein_trajectory(N, m, seed=9)
    Xd, mm = device.pack_trajectory(X, 3)
    ab = synthetic.all_pairs(N)
    expect = oracle_mod.pairs(X, m, 3, ab, k, gc=False, threads=8)
    mi = torch.empty(len(ab), device="cuda")
    torch.cuda.synchronize()

    def run_once():
        plan = device.KsgPlan(device.make_pairs(Xd, mm, ab), k, 3, mi=mi)
        plan.run()
        torch.cuda.synchronize()
        plan.check()
        plan.close()
        assert np.array_equal(mi.cpu().numpy(), expect)

    for _ in range(3):
        run_once()
    held = torch.cuda.mem_get_info()[0]
    device.release_cached_memory()
    assert torch.cuda.mem_get_info()[0] > held
    run_once()
