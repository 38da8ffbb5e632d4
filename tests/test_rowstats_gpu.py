"""Row mean / standard deviation (netcalc mean, meanGpu, standardDeviation,
standardDeviationGpu) against the oracle's restatement of the reference
kernels' summation order.

Bar: means bit-exact; standard deviations within 2 float ulp (the reference
squares with powf(d, 2.0), this build with d * d).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n", [(1, 1), (3, 7), (5, 1023), (4, 1024), (6, 1025), (40, 3000),
                                 (2, 70001)])
def test_row_stats_match_oracle(oracle_mod, m, n):
    import cuarray
    import netcalc
    rng = np.random.default_rng(m * 7 + n)
    a = (rng.standard_normal((m, n)) * 5 + rng.uniform(-50, 50, (m, 1))).astype(np.float32)
    A = cuarray.FloatCuArray()
    A.fromNumpy2D(a)
    u, s = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    netcalc.standardDeviation(A, u, s, m, n, netcalc.GPU_PLATFORM)
    ru, rs = oracle_mod.row_stats(a, n)
    assert np.array_equal(u.toNumpy1D(), ru)
    np.testing.assert_array_max_ulp(s.toNumpy1D(), rs, maxulp=2)
    u2 = cuarray.FloatCuArray()
    netcalc.mean(A, u2, m, n, netcalc.GPU_PLATFORM)
    assert np.array_equal(u2.toNumpy1D(), ru)


def test_row_stats_platform_and_views(oracle_mod):
    import cuarray
    import netcalc
    a = np.arange(24, dtype=np.float32).reshape(4, 6)
    A = cuarray.FloatCuArray()
    A.fromNumpy2D(a)
    u = cuarray.FloatCuArray()
    # m is recomputed from the size: 24 values in rows of 8 -> 3 rows
    netcalc.mean(A, u, 99, 8, netcalc.GPU_PLATFORM)
    assert u.toNumpy1D().tolist() == [3.5, 11.5, 19.5]
    # the CPU platform only re-initialises the outputs, as the reference
    u, s = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    netcalc.standardDeviation(A, u, s, 4, 6, netcalc.CPU_PLATFORM)
    assert u.toNumpy1D().tolist() == [0.0] * 4 and s.toNumpy1D().tolist() == [0.0] * 4
    # the *Gpu variants take m as given and need initialised outputs
    u = cuarray.FloatCuArray()
    u.init(1, 2)
    netcalc.meanGpu(A, u, 2, 6)
    assert u.toNumpy1D().tolist() == [2.5, 8.5]


def test_row_stats_device_entry(oracle_mod):
    import torch
    from netsci_gb300._lib import call
    rng = np.random.default_rng(5)
    a = rng.standard_normal((300, 5000)).astype(np.float32)
    ad = torch.from_numpy(a).cuda()
    u = torch.empty(300, device="cuda")
    s = torch.empty(300, device="cuda")
    call("nsg_row_stats_device", ad.data_ptr(), u.data_ptr(), s.data_ptr(), 300, 5000, None)
    torch.cuda.synchronize()
    ru, rs = oracle_mod.row_stats(a, 5000)
    assert np.array_equal(u.cpu().numpy(), ru)
    np.testing.assert_array_max_ulp(s.cpu().numpy(), rs, maxulp=2)
