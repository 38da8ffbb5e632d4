"""C-ABI boundary and host-side semantics (CPU only).

* The library loads and exports every function include/netsci_gb300.h
  declares (and the Python binding declares no others).
* CuArray semantics of tests/cuarray/python/test_FloatCuArray.py and the
  reference container (cuarray/src/cuarray.cu).
* netcalc host logic: platform return values and errors, checkpoint files,
  restart ab, Settings dataclasses, the CPU platform against the goldens.
* The GPU platform fails loudly (a CUDA error status) when no GPU is usable.
"""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "netsci_gb300.h"


def header_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nsg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(nsg_lib):
    from netsci_gb300 import _lib
    declared = header_functions()
    assert len(declared) >= 50
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (nsg_[a-z0-9_]+)", out))
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        getattr(nsg_lib, s)  # resolvable through ctypes
    assert sorted(_lib.exported_symbols()) == declared


def test_floatcuarray_nodata_fixture_semantics(nsg_lib):
    import cuarray
    a = cuarray.FloatCuArray()
    a.init(20, 100)
    assert (a.m(), a.n(), a.bytes(), a.size()) == (20, 100, 8000, 2000)
    assert a.allocatedHost() == 1 and a.allocatedDevice() == 0
    assert all(a.get(i, j) == 0.0 for i in range(20) for j in range(0, 100, 7))
    assert a.toDevice() == 1 and a.allocatedDevice() == 0  # not allocated -> 1, no-op
    assert a.deallocateDevice() == 0


def test_fromcuarray_deep_copy(nsg_lib):
    import cuarray
    src = cuarray.FloatCuArray()
    data = np.random.default_rng(0).random((20, 100)).astype(np.float32)
    src.fromNumpy2D(data)
    c = cuarray.FloatCuArray()
    assert c.fromCuArray(cuArray=src, start=18, end=19, m=2, n=100) == 0
    assert (c.m(), c.n(), c.bytes(), c.size(), c.owner()) == (2, 100, 800, 200, 1)
    assert c.allocatedHost() == 1 and c.allocatedDevice() == 0
    assert np.array_equal(c.toNumpy2D(), data[18:20])
    bad = cuarray.FloatCuArray()
    assert bad.fromCuArray(cuArray=src, start=18, end=19, m=3, n=100) == 1


def test_shallow_copy_views_parent(nsg_lib):
    import cuarray
    src = cuarray.FloatCuArray()
    src.fromNumpy2D(np.arange(12, dtype=np.float32).reshape(3, 4))
    v = cuarray.FloatCuArray()
    assert v.fromCuArrayShallowCopy(src, 1, 1, 1, 4) == 0
    assert v.owner() == 0 and v.get(0, 2) == 6.0
    src.set(42.0, 1, 2)
    assert v.get(0, 2) == 42.0


def test_set_bounds_rows_and_repr(nsg_lib):
    import cuarray
    a = cuarray.IntCuArray()
    a.init(2, 3)
    assert a.set(5, 1, 2) == 0 and a.set(5, 2, 0) == 1 and a.set(5, 0, 3) == 1
    assert a[1][2] == 5 and len(a) == 2 and len(a[0]) == 3
    a[0] = [7, 8, 9]
    assert a.toNumpy2D().tolist() == [[7, 8, 9], [0, 0, 5]]
    with pytest.raises(IndexError):
        a[2]
    assert "7 8 9" in repr(a)


def test_npy_roundtrip_sort_argsort(tmp_path, nsg_lib):
    import cuarray
    a = cuarray.FloatCuArray()
    data = np.array([[3.0, 1.0, 2.0], [0.5, 9.0, -1.0]], np.float32)
    a.fromNumpy2D(data)
    f = tmp_path / "a.npy"
    a.save(f)
    assert np.array_equal(np.load(f), data)
    b = cuarray.FloatCuArray()
    assert b.load(f) == 0 and np.array_equal(b.toNumpy2D(), data)
    np.save(tmp_path / "one.npy", np.arange(5, dtype=np.float64))
    c = cuarray.FloatCuArray()
    c.load(tmp_path / "one.npy")
    assert (c.m(), c.n()) == (1, 5) and c.get(0, 4) == 4.0
    s = a.sort(0)
    assert s.toNumpy1D().tolist() == [3.0, 2.0, 1.0]
    assert a.argsort(1).toNumpy1D().tolist() == [1, 0, 2]


def _xy(n=200, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n).astype(np.float32)
    y = (0.7 * x + 0.7 * rng.standard_normal(n)).astype(np.float32)
    return x, y


def test_cpu_platform_goldens(golden, nsg_lib):
    import cuarray
    import netcalc
    g = golden("gaussian")
    for n, gold in ((1000, 0.8449974060058594), (2000, 0.8485465049743652)):
        xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
        xa.fromNumpy1D(g[f"x{n}"])
        xb.fromNumpy1D(g[f"y{n}"])
        assert netcalc.mutualInformationCpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=1) == gold


def test_cpu_platform_curves_gc(golden, nsg_lib):
    import cuarray
    import netcalc
    c = golden("curves")
    for d in (1, 2, 3):
        n = 1000
        xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
        xa.fromNumpy1D(c[f"xa_d{d}_n{n}"])
        xb.fromNumpy1D(c[f"xb_d{d}_n{n}"])
        assert netcalc.generalizedCorrelationCpu(Xa=xa, Xb=xb, k=4, n=n, xd=2, d=d) == \
            float(c[f"gc_d{d}_n{n}"])


def test_platform_contract_cpu(nsg_lib):
    import cuarray
    import netcalc
    n = 300
    x, y = _xy(n)
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(np.stack([x, y]))
    I = cuarray.FloatCuArray()
    ab = cuarray.IntCuArray()
    ab.init(1, 2)
    ab.set(0, 0, 0)
    ab.set(1, 0, 1)
    assert netcalc.mutualInformation(X=X, I=I, ab=ab, k=4, n=n, xd=2, d=1,
                                     platform=netcalc.CPU_PLATFORM) == 1
    assert (I.m(), I.n()) == (1, 1) and I.get(0, 0) > 0.2
    with pytest.raises(RuntimeError):
        netcalc.mutualInformation(X=X, I=I, ab=ab, k=4, n=n, xd=2, d=1, platform=7)
    with pytest.raises(RuntimeError):
        netcalc.generalizedCorrelation(X=X, R=I, ab=ab, k=4, n=n, xd=2, d=1, platform=-1)
    A, H, P = cuarray.FloatCuArray(), cuarray.FloatCuArray(), cuarray.IntCuArray()
    A.init(3, 3)
    with pytest.raises(ValueError):
        netcalc.hedetniemiAllShortestPaths(A=A, H=H, paths=P, maxPathLength=2, tolerance=1e-3,
                                           platform=5)
    # lengths on the CPU platform: no solver in the reference either; H zeros
    netcalc.hedetniemiAllShortestPathLengths(A=A, H=H, maxPathLength=2, platform=1)
    assert (H.m(), H.n()) == (3, 3) and H.toNumpy2D().sum() == 0


def test_gpu_platform_fails_loudly_without_gpu(nsg_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    import cuarray
    import netcalc
    from netsci_gb300 import NsgError
    x, y = _xy(100)
    xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    xa.fromNumpy1D(x)
    xb.fromNumpy1D(y)
    with pytest.raises(NsgError) as e:
        netcalc.mutualInformationGpu(Xa=xa, Xb=xb, k=4, n=100, xd=2, d=1)
    assert e.value.status == 2  # NSG_ERR_CUDA, no silent CPU result


def test_invalid_arguments_are_errors(nsg_lib):
    import cuarray
    import netcalc
    from netsci_gb300 import NsgError
    x, y = _xy(50)
    xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
    xa.fromNumpy1D(x)
    xb.fromNumpy1D(y)
    for kw in (dict(k=50), dict(k=0), dict(xd=3), dict(d=4)):
        args = dict(Xa=xa, Xb=xb, k=4, n=50, xd=2, d=1)
        args.update(kw)
        with pytest.raises(NsgError) as e:
            netcalc.mutualInformationCpu(**args)
        assert e.value.status == 1
    with pytest.raises(NsgError):
        netcalc.mutualInformationCpu(Xa=xa, Xb=xb, k=4, n=51, xd=2, d=1)  # row too short


def test_checkpoint_files_and_restart(tmp_path, nsg_lib):
    import cuarray
    import netcalc
    rng = np.random.default_rng(5)
    N, n = 5, 120
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(rng.standard_normal((N, n)).astype(np.float32))
    a, b = np.triu_indices(N, 1)
    ab = cuarray.IntCuArray()
    ab.fromNumpy2D(np.stack([a, b], 1).astype(np.int32))
    I = cuarray.FloatCuArray()
    base = tmp_path / "ckpt.npy"
    r = netcalc.mutualInformationWithCheckpointing(X=X, I=I, ab=ab, k=3, n=n, xd=2, d=1,
                                                   platform=1, checkpointFrequency=3,
                                                   checkpointFileName=str(base))
    assert r == 1
    files = sorted(p.name for p in tmp_path.iterdir())
    # pairs 0..9: checkpoints after pairs 0, 3, 6, 9; each replaces the previous
    assert files == ["ckpt_9.npy", "ckpt_ab.npy"]
    assert np.array_equal(np.load(tmp_path / "ckpt_ab.npy"), np.stack([a, b], 1))
    full = I.toNumpy1D()
    assert np.array_equal(np.load(tmp_path / "ckpt_9.npy").ravel(), full)
    I2 = cuarray.FloatCuArray()
    netcalc.mutualInformation(X=X, I=I2, ab=ab, k=3, n=n, xd=2, d=1, platform=1)
    assert np.array_equal(I2.toNumpy1D(), full)
    restart = cuarray.IntCuArray()
    netcalc.generateRestartAbFromCheckpointFile(ab, restart, str(tmp_path / "ckpt_6.npy"))
    assert np.array_equal(restart.toNumpy2D(), np.stack([a, b], 1)[7:])


def test_checkpoint_intermediate_file_contents(tmp_path, nsg_lib):
    import cuarray
    import netcalc
    rng = np.random.default_rng(6)
    N, n = 4, 80
    X = cuarray.FloatCuArray()
    X.fromNumpy2D(rng.standard_normal((N, n)).astype(np.float32))
    ab = cuarray.IntCuArray()
    ab.fromNumpy2D(np.array([[0, 1], [0, 2], [1, 3], [2, 3], [0, 3]], np.int32))
    I = cuarray.FloatCuArray()
    netcalc.generalizedCorrelationWithCheckpointing(X=X, R=I, ab=ab, k=2, n=n, xd=2, d=1,
                                                    platform=1, checkpointFrequency=4,
                                                    checkpointFileName=str(tmp_path / "gc"))
    ck = np.load(tmp_path / "gc_4.npy").ravel()
    assert np.array_equal(ck, I.toNumpy1D())
    assert not (tmp_path / "gc_0.npy").exists()


def test_settings_dataclasses(nsg_lib):
    import cuarray
    import netcalc
    X = cuarray.FloatCuArray()
    X.init(1, 3 * 10)
    ab = cuarray.IntCuArray()
    s = netcalc.GeneralizedCorrelationSettings(X=X, R=cuarray.FloatCuArray(), ab=ab, k=6, n=10,
                                               xd=2, d=3)
    # the reference sizes the auto-filled pair list as (X.n() / d)**2
    # (netcalc/python/netcalc/__init__.py:90-102); mirrored as is
    assert (ab.m(), ab.n()) == (100, 2)
    assert ab.toNumpy2D()[:3].tolist() == [[0, 0], [0, 1], [0, 2]]
    assert "checkpointFrequency" not in list(s)
    assert set(s.keys()) == {"X", "R", "ab", "k", "n", "xd", "d", "platform"}
    m = netcalc.MutualInformationSettings(X=X, I=cuarray.FloatCuArray(), ab=ab, k=6, n=10, xd=2,
                                          d=3, checkpointFrequency=5, checkpointFileName="f")
    assert list(m)[-2:] == ["checkpointFrequency", "checkpointFileName"]


def test_generate_psi_matches_oracle(oracle_mod, nsg_lib):
    import cuarray
    import netcalc
    p = cuarray.FloatCuArray()
    p.init(1, 1001)
    netcalc.generatePsi(p, 1000)
    assert np.array_equal(p.toNumpy1D(), oracle_mod.psi(1000))


def test_recover_single_shortest_path_host(nsg_lib):
    import cuarray
    import netcalc
    n, L = 4, 3
    P = np.full(n * L * n, -1, np.int32)
    # cell (0, 3): walk stored 1, 2, 3
    P[0 * L * n + 3 * L: 0 * L * n + 3 * L + 3] = [1, 2, 3]
    paths = cuarray.IntCuArray()
    paths.fromNumpy1D(P)
    assert netcalc.recoverSingleShortestPath(paths, L, 0, 3).tolist() == [0, 1, 2, 3]
    assert netcalc.recoverSingleShortestPath(paths, L, 1, 2).tolist() == [1, -1, 2]
