"""Host-side checks of the row-statistics oracle and argument handling."""
import numpy as np
import pytest


def test_oracle_row_stats_small_exact(oracle_mod):
    a = np.array([[1, 2, 3, 4], [2, 2, 2, 2]], np.float32)
    u, s = oracle_mod.row_stats(a, 4)
    assert u.tolist() == [2.5, 2.0]
    assert s[1] == 0.0 and abs(s[0] - np.sqrt(1.25)) < 1e-7


def test_oracle_row_stats_close_to_numpy(oracle_mod):
    a = np.random.default_rng(2).standard_normal((3, 5000)).astype(np.float32)
    u, s = oracle_mod.row_stats(a, 5000)
    np.testing.assert_allclose(u, a.astype(np.float64).mean(1), atol=1e-6)
    np.testing.assert_allclose(s, a.astype(np.float64).std(1), rtol=1e-5)


def test_mean_rejects_bad_n():
    import cuarray
    import netcalc
    from netsci_gb300 import NsgError
    A = cuarray.FloatCuArray()
    A.fromNumpy1D(np.ones(4, np.float32))
    with pytest.raises(NsgError):
        netcalc.mean(A, cuarray.FloatCuArray(), 1, 0, netcalc.CPU_PLATFORM)
