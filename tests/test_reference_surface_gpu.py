"""The reference's Python test scenarios through the drop-in modules.

Same calls, keyword arguments and assertions as
tests/netcalc/python/test_MutualInformation.py,
tests/netcalc/python/test_GeneralizedCorrelation.py and
tests/cuarray/python/test_FloatCuArray.py of the reference, with the input
data read from tests/golden instead of the reference tree. Inputs are built
element by element through CuArray.set, as those tests do.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fill(arr, planes):
    """Write planes (list of 1-D arrays) into rows of a CuArray with set()."""
    for r, plane in enumerate(planes):
        for i, v in enumerate(plane):
            arr.set(float(v), r, i)


@pytest.mark.parametrize("n,gold", [(1000, 0.8449974060058594), (2000, 0.8485465049743652)])
def test_mutual_information_2x1d_gaussian_gpu_cpu(golden, n, gold):
    import cuarray
    import netcalc
    g = golden("gaussian")
    X = np.concatenate([g[f"x{n}"], g[f"y{n}"]])
    Xa, Xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    Xa.fromNumpy1D(X[:n])
    Xb.fromNumpy1D(X[n:])
    gpu = netcalc.mutualInformationGpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=1)
    cpu = netcalc.mutualInformationCpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=1)
    assert gpu == cpu == gold


@pytest.mark.parametrize("n", [1000, 2000])
def test_mutual_information_2x2d_curves_gpu_cpu(golden, n):
    import cuarray
    import netcalc
    c = golden("curves")
    xa = c[f"xa_d2_n{n}"].reshape(2, n)
    xb = c[f"xb_d2_n{n}"].reshape(2, n)
    Xa, Xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    Xa.init(2, n)
    Xb.init(2, n)
    _fill(Xa, xa)
    _fill(Xb, xb)
    gpu = netcalc.mutualInformationGpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=2)
    cpu = netcalc.mutualInformationCpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=2)
    assert gpu == cpu


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("n", [1000, 2000])
def test_generalized_correlation_curves_gpu_cpu(golden, d, n):
    import cuarray
    import netcalc
    c = golden("curves")
    Xa, Xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    Xa.init(d, n)
    Xb.init(d, n)
    _fill(Xa, c[f"xa_d{d}_n{n}"].reshape(d, n))
    _fill(Xb, c[f"xb_d{d}_n{n}"].reshape(d, n))
    gpu = netcalc.generalizedCorrelationGpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=d)
    cpu = netcalc.generalizedCorrelationCpu(Xa=Xa, Xb=Xb, k=4, n=n, xd=2, d=d)
    assert gpu == cpu


def _sincos_X(n):
    import cuarray
    X = cuarray.FloatCuArray()
    X.init(2, n)
    x = 0.001
    for i in range(n):
        X.set(float(np.sin(x)), 0, i)
        X.set(float(np.cos(x)), 1, i)
        x += float(np.pi / n)
    return X


@pytest.mark.parametrize("platform,expected", [(1, 1), (0, 0)])
def test_mutual_information_platform_return(platform, expected):
    import cuarray
    import netcalc
    n = 1000
    X = _sincos_X(n)
    I = cuarray.FloatCuArray()
    ab = cuarray.IntCuArray()
    ab.init(1, 2)
    ab.set(0, 0, 0)
    ab.set(1, 0, 1)
    assert netcalc.mutualInformation(X=X, I=I, ab=ab, k=4, n=n, xd=2, d=1,
                                     platform=platform) == expected


@pytest.mark.parametrize("platform,expected", [(1, 1), (0, 0)])
def test_generalized_correlation_platform_return(platform, expected):
    import cuarray
    import netcalc
    n = 1000
    X = _sincos_X(n)
    R = cuarray.FloatCuArray()
    ab = cuarray.IntCuArray()
    ab.init(1, 2)
    ab.set(0, 0, 0)
    ab.set(1, 0, 1)
    assert netcalc.generalizedCorrelation(X=X, R=R, ab=ab, k=4, n=n, xd=2, d=1,
                                          platform=platform) == expected


def test_floatcuarray_device_allocation():
    import cuarray
    a = cuarray.FloatCuArray()
    a.init(20, 100)
    a.allocateDevice()
    a.toDevice()
    assert a.allocatedDevice() == 1
    a.deallocateDevice()
    assert a.allocatedDevice() == 0
    b = cuarray.FloatCuArray()
    data = np.random.default_rng(2).random((20, 100)).astype(np.float32)
    b.fromNumpy2D(data)
    b.allocateDevice()
    assert b.toDevice() == 0
    b.set(0.0, 3, 3)
    assert b.toHost() == 0 and b.get(3, 3) == data[3, 3]
