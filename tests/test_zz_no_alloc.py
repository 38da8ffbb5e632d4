"""The allocation-free entry point (nsg_ksg_pair_noalloc_device).

It exists for callers that cannot allocate device memory themselves or let
a library do it -- for instance an application that keeps all of the GPU's
memory in its own pool and calls this library as a plugin on buffers it
already owns. Its scratch is a fixed array compiled into the library.

This file is collected last on purpose (pytest orders test files by name),
so that a failure here, in a run that stops at the first failure, comes
after every other test has run. It must pass both on its own in a fresh
process and after the rest of the suite: the first call on the device sets
the scratch area up, and later calls must not depend on what earlier calls
left in it.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rows(X, d):
    from netsci_gb300 import device
    Xd, m = device.pack_trajectory(X, d)
    return Xd, m


def _noalloc(xa, xb, ld, m, k, d):
    from netsci_gb300._lib import call
    mi = torch.full((1,), float("nan"), device="cuda")
    gc = torch.full((1,), float("nan"), device="cuda")
    call("nsg_ksg_pair_noalloc_device", ctypes.c_void_p(xa.data_ptr()),
         ctypes.c_void_p(xb.data_ptr()), ld, m, k, d, ctypes.c_void_p(mi.data_ptr()),
         ctypes.c_void_p(gc.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return float(mi.item()), float(gc.item())


def _reference_entry(Xd, m, k, d):
    """MI and GC of pair (0, 1) through the existing allocating entry point."""
    from netsci_gb300 import device
    pairs = device.make_pairs(Xd, m, [[0, 1]])
    mi = torch.empty(1, device="cuda")
    gc = torch.empty(1, device="cuda")
    device.ksg_pairs(pairs, k, d, mi=mi, gc=gc)
    return float(mi.item()), float(gc.item())


@pytest.mark.parametrize("d,k,m", [(3, 6, 1000), (1, 4, 2000), (2, 10, 777)])
def test_no_alloc_matches_allocating_entry_point_twice(oracle_mod, d, k, m):
    from netsci_gb300 import synthetic
    rng = np.random.default_rng(1000 + d * 10 + k)
    if d == 3:
        X, _ = synthetic.protein_trajectory(2, m, seed=d + k)
    else:
        a = rng.standard_normal(d * m).astype(np.float32)
        b = (0.6 * a + 0.8 * rng.standard_normal(d * m)).astype(np.float32)
        X = np.stack([a, b])
    Xd, mm = _rows(X, d)
    want = _reference_entry(Xd, mm, k, d)
    ld = Xd.shape[2]
    first = _noalloc(Xd[0], Xd[1], ld, mm, k, d)
    second = _noalloc(Xd[0], Xd[1], ld, mm, k, d)
    # the kernels are shared with the allocating path: results are bit-exact
    assert first == want and second == want
    # and MI equals the CPU oracle's (the reference CPU path's arithmetic)
    assert first[0] == oracle_mod.mi_pair(X[0], X[1], m, k, d)


def test_no_alloc_reproduces_the_reference_goldens(golden):
    """The reference's own published MI values for its Gaussian fixtures
    (tests/netcalc/python/test_MutualInformation.py:37,64), twice each."""
    g = golden("gaussian")
    for n in (1000, 2000):
        Xd, m = _rows(np.stack([g[f"x{n}"], g[f"y{n}"]]), 1)
        for _ in range(2):
            mi, _ = _noalloc(Xd[0], Xd[1], Xd.shape[2], m, 4, 1)
            assert mi == float(g[f"mi{n}"])
    assert float(g["mi1000"]) == 0.8449974060058594
    assert float(g["mi2000"]) == 0.8485465049743652


def test_no_alloc_calls_allocate_no_device_memory():
    """After the first call on the device, calls of different sizes leave the
    device's free memory unchanged: nothing is allocated, by the library or
    through it (inputs and outputs are made before the measurement)."""
    from netsci_gb300 import synthetic
    cases = []
    for m, seed in ((300, 1), (4000, 2), (1500, 3), (9000, 4)):
        X, _ = synthetic.protein_trajectory(2, m, seed=seed)
        Xd, mm = _rows(X, 3)
        cases.append((Xd, mm))
    mi = torch.full((1,), float("nan"), device="cuda")
    gc = torch.full((1,), float("nan"), device="cuda")
    stream = torch.cuda.current_stream()

    def call(Xd, mm):
        from netsci_gb300._lib import call as nsg_call
        nsg_call("nsg_ksg_pair_noalloc_device", ctypes.c_void_p(Xd[0].data_ptr()),
                 ctypes.c_void_p(Xd[1].data_ptr()), Xd.shape[2], mm, 6, 3,
                 ctypes.c_void_p(mi.data_ptr()), ctypes.c_void_p(gc.data_ptr()),
                 ctypes.c_void_p(stream.cuda_stream))
    call(*cases[0])   # the first call on the device sets the area up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for Xd, mm in cases * 2:
        call(Xd, mm)
        assert np.isfinite(float(mi.item())) and np.isfinite(float(gc.item()))
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_no_alloc_after_a_different_size_call():
    """A smaller call after a larger one must not see the larger call's
    leftovers in the shared scratch."""
    from netsci_gb300 import synthetic
    big, _ = synthetic.protein_trajectory(2, 3000, seed=5)
    small, _ = synthetic.protein_trajectory(2, 400, seed=6)
    Xb, mb = _rows(big, 3)
    Xs, ms = _rows(small, 3)
    _noalloc(Xb[0], Xb[1], Xb.shape[2], mb, 6, 3)
    got = _noalloc(Xs[0], Xs[1], Xs.shape[2], ms, 6, 3)
    assert got == _reference_entry(Xs, ms, 6, 3)


def test_no_alloc_rejects_sizes_above_its_limit():
    from netsci_gb300 import NsgError
    m = 65537
    X = torch.zeros((2, 1, m), device="cuda")
    with pytest.raises(NsgError) as e:
        _noalloc(X[0], X[1], m, m, 4, 1)
    assert e.value.status == 4 and "65536" in str(e.value)
