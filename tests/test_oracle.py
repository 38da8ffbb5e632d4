"""The CPU oracle against the reference's golden values and, where the
reference sources were compiled into oracle/_ref, against the reference CPU
functions themselves (CPU only)."""
import numpy as np
import pytest

GOLDEN_MI = {1000: 0.8449974060058594, 2000: 0.8485465049743652}


def test_psi_table_recurrence(oracle_mod):
    psi = oracle_mod.psi(10000)
    assert psi[0] == 0.0
    assert psi[1] == np.float32(-0.57721566490153)
    # float recurrence psi[i+1] = psi[i] + (float)(1/(float)i)
    for i in (1, 2, 17, 9999):
        assert psi[i + 1] == np.float32(psi[i] + np.float32(1.0 / np.float32(i)))


@pytest.mark.parametrize("n", [1000, 2000])
def test_gaussian_goldens(oracle_mod, golden, n):
    g = golden("gaussian")
    mi, det = oracle_mod.mi_pair(g[f"x{n}"], g[f"y{n}"], n, 4, 1, detail=True)
    assert mi == GOLDEN_MI[n] == float(g[f"mi{n}"])
    assert np.array_equal(det["n_x"], g[f"n_x{n}"]) and np.array_equal(det["n_y"], g[f"n_y{n}"])
    assert det["ties"] == 0
    # MI recomputed from the counts in the reference's summation order
    assert oracle_mod.mi_from_counts(det["n_x"], det["n_y"], n, 4) == mi


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("n", [1000, 2000])
def test_curves_match_reference_values(oracle_mod, golden, d, n):
    c = golden("curves")
    mi = oracle_mod.mi_pair(c[f"xa_d{d}_n{n}"], c[f"xb_d{d}_n{n}"], n, 4, d)
    assert mi == float(c[f"mi_d{d}_n{n}"])
    assert oracle_mod.gc_from_mi(mi, d) == float(c[f"gc_d{d}_n{n}"])


def test_random_cases_match_reference_values(oracle_mod, golden):
    r = golden("random")
    for i in range(int(r["count"])):
        d, k, n = (int(v) for v in r[f"meta{i}"])
        mi = oracle_mod.mi_pair(r[f"xa{i}"], r[f"xb{i}"], n, k, d)
        assert mi == float(r[f"mi{i}"]), (i, d, k, n)


def test_against_reference_library_when_built(oracle_mod):
    R = oracle_mod.ref_lib()
    if R is None:
        pytest.skip("reference sources not compiled here (oracle/_ref absent)")
    rng = np.random.default_rng(7)
    for d in (1, 2, 3):
        n, k = 300, 5
        xa = rng.standard_normal(d * n).astype(np.float32)
        xb = (0.6 * xa + 0.8 * rng.standard_normal(d * n)).astype(np.float32)
        assert oracle_mod.mi_pair(xa, xb, n, k, d) == R.ref_mi_cpu(xa, xb, n, k, d)
        assert oracle_mod.gc_from_mi(oracle_mod.mi_pair(xa, xb, n, k, d), d) == \
            R.ref_gc_cpu(xa, xb, n, k, d)
    p = np.zeros(5001, np.float32)
    R.ref_psi(p, 5000)
    assert np.array_equal(p, oracle_mod.psi(5000))


def test_protein_fixture_pairs_sampled(oracle_mod, golden):
    z = golden("protein56")
    X, ab, gc, k = z["X"], z["ab"], z["gc"], int(z["k"])
    for p in (0, 17, 777, 1539):
        a, b = ab[p]
        mi = oracle_mod.mi_pair(X[a], X[b], 1000, k, 3)
        assert oracle_mod.gc_from_mi(mi, 3) == gc[p]


def test_oracle_pairs_driver_threads(oracle_mod, golden):
    z = golden("protein56")
    sel = z["ab"][:16]
    one = oracle_mod.pairs(z["X"], 1000, 3, sel, 6, gc=True, threads=1)
    many = oracle_mod.pairs(z["X"], 1000, 3, sel, 6, gc=True, threads=4)
    assert np.array_equal(one, many) and np.array_equal(one, z["gc"][:16])


def test_apsp_oracle_matches_floyd_warshall_integer(oracle_mod):
    from netsci_gb300 import synthetic
    A = synthetic.random_geometric_graph(120, 6, seed=3, integer_weights=True)
    H, steps, conv = oracle_mod.apsp_lengths(A, 120)
    assert conv
    assert np.array_equal(H, oracle_mod.floyd_warshall(A))


def test_apsp_oracle_fixture(oracle_mod, golden):
    z = golden("protein56")
    H, steps, conv = oracle_mod.apsp_lengths(z["A"], 56)
    assert conv and steps == int(z["steps"]) and np.array_equal(H, z["H"])
    np.testing.assert_allclose(H, oracle_mod.floyd_warshall(z["A"]), rtol=1e-6)


def test_apsp_paths_oracle_are_shortest(oracle_mod):
    from netsci_gb300 import synthetic
    n, L = 40, 20  # this graph needs 17 Hedetniemi steps
    A = synthetic.random_geometric_graph(n, 5, seed=11, integer_weights=True)
    H, P = oracle_mod.apsp_paths(A, L, 1e-3)
    D = oracle_mod.floyd_warshall(A)
    assert np.array_equal(H, D)
    P = P.reshape(n, n, L)
    for i in range(n):
        for j in range(n):
            if i == j or not np.isfinite(D[i, j]):
                continue
            seq = [i]
            for v in P[i, j]:
                if v not in seq:
                    seq.append(int(v))
            if seq[-1] != j:
                seq.append(j)
            length = sum(A[seq[t], seq[t + 1]] for t in range(len(seq) - 1))
            assert length == D[i, j], (i, j, seq)
