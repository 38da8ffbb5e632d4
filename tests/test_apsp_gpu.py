"""Hedetniemi all-pairs shortest paths on the GPU against the CPU oracle.

Bar: lengths bit-exact against the oracle's Jacobi iteration for float and
integer weights (each entry is a minimum of single roundings, independent
of evaluation order), and equal to Floyd-Warshall on integer weights;
paths bit-exact against the oracle's walk. Where repeated squaring applies
(the fixed point of a symmetric, zero-diagonal, non-negative graph) it is
bit-exact on integer weights and, when forced on float weights, within
1e-6 relative of the Jacobi fixed point.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(A):
    return torch.from_numpy(np.ascontiguousarray(A, np.float32)).cuda()


def test_protein56_contact_graph_lengths(golden):
    from netsci_gb300 import device
    z = golden("protein56")
    H, steps = device.apsp_lengths(_dev(z["A"]), 56)
    assert steps == int(z["steps"])
    assert np.array_equal(H.cpu().numpy(), z["H"])


@pytest.fixture
def apsp_method():
    from netsci_gb300 import device
    yield device.set_apsp_method
    device.set_apsp_method(-1)


@pytest.mark.parametrize("n", [1, 7, 128, 300, 257])
def test_integer_rgg_matches_floyd_warshall(oracle_mod, apsp_method, n):
    """Automatic schedule (repeated squaring on these graphs) and Jacobi
    steps: both equal Floyd-Warshall; Jacobi takes the oracle's step count,
    squaring about log2 of it."""
    from netsci_gb300 import device, synthetic
    A = synthetic.random_geometric_graph(n, 8, seed=n, integer_weights=True)
    D = oracle_mod.floyd_warshall(A)
    Ho, so, conv = oracle_mod.apsp_lengths(A, n)
    H, products = device.apsp_lengths(_dev(A), n)
    assert np.array_equal(H.cpu().numpy(), D)
    if n > 1:
        # Jacobi's count is the hop diameter h; squaring runs ceil(log2 h)
        # products to reach it and one more that changes nothing
        assert products == int(np.ceil(np.log2(so))) + 1
    apsp_method(0)
    H, steps = device.apsp_lengths(_dev(A), n)
    assert np.array_equal(H.cpu().numpy(), D)
    assert steps == so


def test_squaring_schedule_rules(oracle_mod, apsp_method):
    """Squaring only where it reaches the Jacobi fixed point: asymmetric,
    truncated (maxPathLength < n-1) or non-integer inputs take Jacobi steps
    in the automatic mode (the step count tells which schedule ran)."""
    from netsci_gb300 import device, synthetic
    n = 200
    A = synthetic.random_geometric_graph(n, 5, seed=9, integer_weights=True)
    Ho, so, _ = oracle_mod.apsp_lengths(A, n)
    assert so > 8
    _, p = device.apsp_lengths(_dev(A), n)
    assert p < so
    _, p = device.apsp_lengths(_dev(A), n - 2)     # truncated: Jacobi
    assert p == min(so, n - 2)
    B = A.copy()
    B[3, 7] = B[7, 3] + 1 if np.isfinite(B[7, 3]) else 5.0   # asymmetric: Jacobi
    Hb, pb = device.apsp_lengths(_dev(B), n)
    Hob, sob, _ = oracle_mod.apsp_lengths(B, n)
    assert pb == sob and np.array_equal(Hb.cpu().numpy(), Hob)
    C = A.copy()
    C[np.isfinite(C) & (C > 0)] += 0.5                         # non-integer: Jacobi
    Hc, pc = device.apsp_lengths(_dev(C), n)
    Hoc, soc, _ = oracle_mod.apsp_lengths(C, n)
    assert pc == soc and np.array_equal(Hc.cpu().numpy(), Hoc)
    # forced squaring on float weights: within 1e-6 relative of Jacobi
    apsp_method(1)
    Hf, pf = device.apsp_lengths(_dev(C), n)
    assert pf < soc
    np.testing.assert_allclose(Hf.cpu().numpy(), Hoc, rtol=1e-6)


@pytest.mark.parametrize("n", [200, 383])
def test_float_weights_bit_exact_vs_oracle(oracle_mod, n):
    from netsci_gb300 import device, synthetic
    A = synthetic.random_geometric_graph(n, 10, seed=2 * n, integer_weights=False)
    H, steps = device.apsp_lengths(_dev(A), n)
    Ho, so, conv = oracle_mod.apsp_lengths(A, n)
    assert conv and steps == so
    assert np.array_equal(H.cpu().numpy(), Ho)
    np.testing.assert_allclose(H.cpu().numpy(), oracle_mod.floyd_warshall(A), rtol=1e-6)


def test_truncated_path_length_matches_jacobi(oracle_mod):
    from netsci_gb300 import device, synthetic
    A = synthetic.random_geometric_graph(150, 4, seed=5, integer_weights=True)
    for L in (0, 1, 2, 3):
        H, steps = device.apsp_lengths(_dev(A), L)
        Ho, so, _ = oracle_mod.apsp_lengths(A, L)
        assert steps == so and np.array_equal(H.cpu().numpy(), Ho), L


def test_asymmetric_matrix_follows_reference_formula(oracle_mod):
    from netsci_gb300 import device
    rng = np.random.default_rng(3)
    n = 90
    A = np.where(rng.random((n, n)) < 0.1, rng.integers(1, 20, (n, n)), np.inf).astype(np.float32)
    np.fill_diagonal(A, 0)
    H, steps = device.apsp_lengths(_dev(A), 30)
    Ho, so, _ = oracle_mod.apsp_lengths(A, 30)
    assert steps == so and np.array_equal(H.cpu().numpy(), Ho)


def test_paths_match_oracle_and_are_shortest(oracle_mod):
    import cuarray
    import netcalc
    from netsci_gb300 import synthetic
    n, L = 60, 24
    A = synthetic.random_geometric_graph(n, 6, seed=12, integer_weights=True)
    Ho, Po = oracle_mod.apsp_paths(A, L, 1e-3)
    Ac, Hc, Pc = cuarray.FloatCuArray(), cuarray.FloatCuArray(), cuarray.IntCuArray()
    Ac.fromNumpy2D(A)
    netcalc.hedetniemiAllShortestPaths(A=Ac, H=Hc, paths=Pc, maxPathLength=L, tolerance=1e-3,
                                       platform=netcalc.GPU_PLATFORM)
    assert np.array_equal(Hc.toNumpy2D(), Ho)
    assert np.array_equal(Pc.toNumpy1D(), Po)
    D = oracle_mod.floyd_warshall(A)
    for i in range(0, n, 7):
        for j in range(n):
            if i == j or not np.isfinite(D[i, j]):
                continue
            seq = netcalc.recoverSingleShortestPath(Pc, L, i, j).tolist()
            assert seq[0] == i and seq[-1] == j
            assert sum(A[seq[t], seq[t + 1]] for t in range(len(seq) - 1)) == D[i, j]


def test_lengths_cuarray_api(golden):
    import cuarray
    import netcalc
    z = golden("protein56")
    A, H = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    A.fromNumpy2D(z["A"])
    netcalc.hedetniemiAllShortestPathLengths(A=A, H=H, maxPathLength=56,
                                             platform=netcalc.GPU_PLATFORM)
    assert np.array_equal(H.toNumpy2D(), z["H"])


def test_correlation_to_adjacency(oracle_mod, golden):
    import cuarray
    import netcalc
    from netsci_gb300 import device
    rng = np.random.default_rng(4)
    n = 77
    C = rng.random((n, n)).astype(np.float32)
    C[rng.random((n, n)) < 0.2] = 0.0
    A, Cc = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    Cc.fromNumpy2D(C)
    netcalc.correlationToAdjacency(A=A, C=Cc, n=n, platform=0)
    assert np.array_equal(A.toNumpy2D(), oracle_mod.corr_to_adj(C))
    W = device.corr_to_adjacency(_dev(C), mode=1).cpu().numpy()
    ref = oracle_mod.corr_to_neglog_adj(C)
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(W), fin)
    np.testing.assert_array_max_ulp(W[fin], ref[fin], maxulp=1)
