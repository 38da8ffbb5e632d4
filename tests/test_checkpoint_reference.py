"""Checkpoint files pinned to the reference's own pair-list drivers.

The reference's ``mutualInformation`` / ``generalizedCorrelation`` with
checkpointing (netcalc/src/mutual_information.cpp:8-101,
generalized_correlation.cpp:8-102) and ``generateRestartAbFromCheckpointFile``
(mutual_information.cpp:174-201) are compiled unmodified into
oracle/_ref/liboracle_ref.so. Both implementations write their checkpoint
files into separate folders for the same inputs; the folders must hold the
same file names with byte-identical contents (the .npy headers included),
and the restart lists must agree. The CPU platform runs here; the GPU
platform of this library is checked against the same reference files in
the gpu-marked test."""
from pathlib import Path

import numpy as np
import pytest

CASES = [(5, 1, 3, "mi"), (7, 4, 2, "gc"), (6, 10, 1, "mi"), (4, 1, 1, "gc"), (6, 25, 3, "gc")]


def _ref_or_skip(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("reference CPU library not built (no reference sources)")


def _inputs(N, n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, d * n)).astype(np.float32)
    X[1::2] = (0.6 * X[0] + X[1::2]).astype(np.float32)
    a, b = np.triu_indices(N, 1)
    return X, np.stack([a, b], 1).astype(np.int32)


def _ours(X, ab, n, d, k, kind, freq, path, platform):
    import cuarray
    import netcalc
    Xc = cuarray.FloatCuArray()
    Xc.fromNumpy2D(X)
    abc = cuarray.IntCuArray()
    abc.fromNumpy2D(ab)
    R = cuarray.FloatCuArray()
    fn = (netcalc.generalizedCorrelationWithCheckpointing if kind == "gc"
          else netcalc.mutualInformationWithCheckpointing)
    kw = dict(R=R) if kind == "gc" else dict(I=R)
    rc = fn(X=Xc, ab=abc, k=k, n=n, xd=2, d=d, platform=platform, checkpointFrequency=freq,
            checkpointFileName=str(path), **kw)
    return rc, R.toNumpy1D()


def _files(folder: Path):
    return {p.name: p.read_bytes() for p in sorted(folder.iterdir())}


def run_case(oracle_mod, tmp_path, N, freq, d, kind, platform, suffix):
    n, k = 160, 3
    X, ab = _inputs(N, n, d, seed=N * 100 + freq)
    ref_dir, our_dir = tmp_path / "ref", tmp_path / "ours"
    ref_dir.mkdir()
    our_dir.mkdir()
    rc_ref, out_ref = oracle_mod.ref_pairs_checkpoint(X, n, d, ab, k, kind == "gc", freq,
                                                      str(ref_dir / ("ckpt" + suffix)))
    assert rc_ref == 1
    rc, out = _ours(X, ab, n, d, k, kind, freq, our_dir / ("ckpt" + suffix), platform)
    assert rc == platform
    assert np.array_equal(out, out_ref)
    ref_files, our_files = _files(ref_dir), _files(our_dir)
    assert sorted(our_files) == sorted(ref_files)
    for name in ref_files:
        assert our_files[name] == ref_files[name], name
    return ref_dir, ab


@pytest.mark.parametrize("N,freq,d,kind", CASES)
@pytest.mark.parametrize("suffix", [".npy", ""])
def test_checkpoint_files_equal_reference_cpu(oracle_mod, nsg_lib, tmp_path, N, freq, d, kind,
                                              suffix):
    _ref_or_skip(oracle_mod)
    run_case(oracle_mod, tmp_path, N, freq, d, kind, 1, suffix)


@pytest.mark.parametrize("last", [0, 3, 6, 9, 14])
@pytest.mark.parametrize("folder", [True, False])
def test_restart_list_equals_reference(oracle_mod, nsg_lib, tmp_path, last, folder):
    _ref_or_skip(oracle_mod)
    import cuarray
    import netcalc
    a, b = np.triu_indices(6, 1)
    ab = np.stack([a, b], 1).astype(np.int32)
    name = (str(tmp_path / f"run_{last}.npy") if folder else f"run_{last}.npy")
    want = oracle_mod.ref_restart_ab(ab, name)
    abc = cuarray.IntCuArray()
    abc.fromNumpy2D(ab)
    r = cuarray.IntCuArray()
    netcalc.generateRestartAbFromCheckpointFile(abc, r, name)
    got = r.toNumpy2D() if r.m() else np.zeros((0, 2), np.int32)
    assert np.array_equal(got.reshape(-1, 2), want.reshape(-1, 2))


@pytest.mark.gpu
@pytest.mark.parametrize("N,freq,d,kind", CASES[:3])
def test_checkpoint_files_equal_reference_gpu_platform(oracle_mod, nsg_lib, tmp_path, N, freq, d,
                                                       kind):
    _ref_or_skip(oracle_mod)
    run_case(oracle_mod, tmp_path, N, freq, d, kind, 0, ".npy")
