"""This library against the reference's own GPU code, compiled unmodified for
sm_103a into oracle/_ref/libnetcalc_ref_gpu.so (oracle/Makefile, target
``ref-gpu``, from the reference sources that ``make -C oracle stage`` copies
into baseline/_ref/netsci).

* Shortest paths: the reference has no CPU implementation
  (netcalc/src/hedetniemi_cpu.cpp:5-16), so its GPU kernel
  (hedetniemi_gpu.cu:28-45, driven by :109-146) is the only reference-held
  answer. It updates H in place, so its intermediate iterates depend on
  thread scheduling, but every entry only ever decreases towards the same
  fixed point: min over k of fl(A[j][k] + H[k][i]), which is reached once the
  launch count covers the Jacobi iteration's convergence step count. There
  the reference's lengths must equal this library's bit for bit, on integer
  and on float weights.
* Row statistics: the reference's mean and standard-deviation kernels sum in
  the order this library restates, so their outputs must be equal bit for bit.
* Mutual information: the reference's GPU per-pair call on tie-free inputs
  equals its CPU path (which the oracle restates), so it must equal this
  library's value too.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_gpu(oracle_mod):
    if oracle_mod.ref_gpu_lib() is None:
        pytest.skip("reference GPU library not built (no reference sources)")
    return oracle_mod


def _ours(A, L, method=-1):
    from netsci_gb300 import device
    device.set_apsp_method(method)
    try:
        H, steps = device.apsp_lengths(torch.from_numpy(np.ascontiguousarray(A, np.float32)).cuda(), L)
    finally:
        device.set_apsp_method(-1)
    return H.cpu().numpy(), steps


@pytest.mark.parametrize("n,degree,integer", [(2000, 12, True), (2000, 12, False), (300, 6, True),
                                              (257, 8, False), (64, 3, True)])
def test_apsp_fixed_point_equals_reference_kernel(ref_gpu, n, degree, integer):
    """Jacobi steps and the automatic schedule (repeated squaring on the
    integer graphs) both give the reference kernel's fixed point; the
    reference runs the Jacobi step count plus two launches."""
    from netsci_gb300 import synthetic
    A = synthetic.random_geometric_graph(n, degree, seed=11 if n == 2000 else n,
                                         integer_weights=integer)
    Hj, steps = _ours(A, n, method=0)
    Href = ref_gpu.ref_gpu_apsp_lengths(A, steps + 2)
    assert np.array_equal(Hj, Href)
    H, products = _ours(A, n)
    assert np.array_equal(H, Href)
    if integer and n > 64:
        assert products < steps


def test_apsp_protein56_contact_graph_equals_reference_kernel(ref_gpu, golden):
    z = golden("protein56")
    H, steps = _ours(z["A"], 56)
    Href = ref_gpu.ref_gpu_apsp_lengths(z["A"], steps + 2)
    assert np.array_equal(H, Href)
    assert np.array_equal(H, z["H"])


def test_mi_equals_reference_gpu_call(ref_gpu, golden):
    """Reference GPU per-pair MI and GC on the reference's Gaussian fixtures
    and on protein56 pairs equal this library's (and the oracle's)."""
    import cuarray
    import netcalc
    g = golden("gaussian")
    for n in (1000, 2000):
        x, y = g[f"x{n}"], g[f"y{n}"]
        want = ref_gpu.ref_gpu_lib().refgpu_mi(x, y, n, 4, 1)
        xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
        xa.fromNumpy1D(x)
        xb.fromNumpy1D(y)
        assert netcalc.mutualInformationGpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=1) == want
    z = golden("protein56")
    X = z["X"]
    for a, b in z["ab"][::97]:
        ref_gc = ref_gpu.ref_gpu_lib().refgpu_gc(X[a], X[b], 1000, 6, 3)
        xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
        xa.fromNumpy1D(X[a])
        xb.fromNumpy1D(X[b])
        assert netcalc.generalizedCorrelationGpu(Xa=xa, Xb=xb, k=6, n=1000, xd=2, d=3) == ref_gc


@pytest.mark.parametrize("m,n", [(1, 1), (3, 7), (5, 1023), (4, 1024), (6, 1025), (40, 3000),
                                 (2, 70001)])
def test_row_stats_equal_reference_kernels(ref_gpu, m, n):
    """netcalc mean / standardDeviation (GPU platform) against the reference's
    own meanKernel / standardDeviationKernel (math_utils_gpu.cu:22-158): the
    same summation order, so bit for bit."""
    import cuarray
    import netcalc
    rng = np.random.default_rng(m * 11 + n)
    a = (rng.standard_normal((m, n)) * 5 + rng.uniform(-50, 50, (m, 1))).astype(np.float32)
    ru, ru2, rs = ref_gpu.ref_gpu_row_stats(a)
    A = cuarray.FloatCuArray()
    A.fromNumpy2D(a)
    u = cuarray.FloatCuArray()
    netcalc.mean(A, u, m, n, netcalc.GPU_PLATFORM)
    u2, s = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    netcalc.standardDeviation(A, u2, s, m, n, netcalc.GPU_PLATFORM)
    assert np.array_equal(u.toNumpy1D(), ru)
    assert np.array_equal(u2.toNumpy1D(), ru2)
    assert np.array_equal(s.toNumpy1D(), rs)
