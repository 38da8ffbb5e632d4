"""Python surface of netcalc: mutual information, generalized correlation and
Hedetniemi shortest paths over CuArray objects.

Mirrors the reference's SWIG module ``netcalc`` and its package re-exports
(netcalc/swig/python_netcalc_rename.i:1-51, netcalc/python/netcalc/
__init__.py:7-128): the same function names, the C++ parameter names as
keyword arguments, the platform return values, and the Settings
dataclasses. Where the reference throws (an invalid platform), these raise:
RuntimeError for the mutual-information and correlation calls
(std::runtime_error there) and ValueError for the shortest-path calls
(std::invalid_argument there).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields
from pathlib import Path
from typing import ItemsView, KeysView, Mapping, Union, ValuesView

import numpy as np

from . import _lib
from ._lib import NsgError, call, lib
from .cuarray import FloatCuArray, IntCuArray

GPU_PLATFORM = 0
CPU_PLATFORM = 1


def _raise_platform(e: NsgError, apsp: bool):
    if e.status == _lib.NSG_ERR_PLATFORM:
        raise (ValueError if apsp else RuntimeError)("Invalid platform") from None
    raise e


def _pair_list(name: str, X, out, ab, k, n, xd, d, platform, *extra) -> int:
    r = ctypes.c_int()
    try:
        call(name, X.handle, out.handle, ab.handle, int(k), int(n), int(xd), int(d),
             int(platform), *extra, ctypes.byref(r))
    except NsgError as e:
        _raise_platform(e, apsp=False)
    return r.value


def mutualInformation(X, I, ab, k, n, xd, d, platform=GPU_PLATFORM) -> int:
    """KSG MI of every (a, b) row of ``ab`` into ``I`` (1 x P); returns the platform."""
    return _pair_list("nsg_mutual_information", X, I, ab, k, n, xd, d, platform)


def mutualInformationWithCheckpointing(X, I, ab, k, n, xd, d, platform, checkpointFrequency,
                                       checkpointFileName) -> int:
    return _pair_list("nsg_mutual_information_checkpointed", X, I, ab, k, n, xd, d, platform,
                      int(checkpointFrequency), str(checkpointFileName).encode())


def _pair(name: str, Xa, Xb, k, n, xd, d) -> float:
    r = ctypes.c_float()
    call(name, Xa.handle, Xb.handle, int(k), int(n), int(xd), int(d), ctypes.byref(r))
    return float(r.value)


def mutualInformationGpu(Xa, Xb, k, n, xd, d) -> float:
    return _pair("nsg_mutual_information_gpu", Xa, Xb, k, n, xd, d)


def mutualInformationCpu(Xa, Xb, k, n, xd, d) -> float:
    return _pair("nsg_mutual_information_cpu", Xa, Xb, k, n, xd, d)


def generalizedCorrelation(X, R, ab, k, n, xd, d, platform=GPU_PLATFORM) -> int:
    return _pair_list("nsg_generalized_correlation", X, R, ab, k, n, xd, d, platform)


def generalizedCorrelationWithCheckpointing(X, R, ab, k, n, xd, d, platform, checkpointFrequency,
                                            checkpointFileName) -> int:
    return _pair_list("nsg_generalized_correlation_checkpointed", X, R, ab, k, n, xd, d,
                      platform, int(checkpointFrequency), str(checkpointFileName).encode())


def generalizedCorrelationGpu(Xa, Xb, k, n, xd, d) -> float:
    return _pair("nsg_generalized_correlation_gpu", Xa, Xb, k, n, xd, d)


def generalizedCorrelationCpu(Xa, Xb, k, n, xd, d) -> float:
    return _pair("nsg_generalized_correlation_cpu", Xa, Xb, k, n, xd, d)


def generateRestartAbFromCheckpointFile(ab, restartAb, checkpointFileName) -> None:
    call("nsg_generate_restart_ab_from_checkpoint_file", ab.handle, restartAb.handle,
         str(checkpointFileName).encode())


def hedetniemiAllShortestPaths(A, H, paths, maxPathLength, tolerance, platform=GPU_PLATFORM):
    try:
        call("nsg_hedetniemi_all_shortest_paths", A.handle, H.handle, paths.handle,
             int(maxPathLength), float(tolerance), int(platform))
    except NsgError as e:
        _raise_platform(e, apsp=True)


def hedetniemiAllShortestPathsGpu(A, H, paths, tolerance, maxPathLength):
    call("nsg_hedetniemi_all_shortest_paths_gpu", A.handle, H.handle, paths.handle,
         float(tolerance), int(maxPathLength))


def hedetniemiAllShortestPathLengths(A, H, maxPathLength, platform=GPU_PLATFORM):
    call("nsg_hedetniemi_all_shortest_path_lengths", A.handle, H.handle, int(maxPathLength),
         int(platform))


def hedetniemiAllShortestPathLengthsGpu(A, H, maxPathLength):
    call("nsg_hedetniemi_all_shortest_path_lengths_gpu", A.handle, H.handle, int(maxPathLength))


def correlationToAdjacency(A, C, n, platform=GPU_PLATFORM):
    call("nsg_correlation_to_adjacency", A.handle, C.handle, int(n), int(platform))


def mean(a, u, m, n, platform=GPU_PLATFORM):
    """Row means of a (rows of n values) into u, re-initialised to 1 x (size/n);
    computed for the GPU platform only, as the reference."""
    call("nsg_mean", a.handle, u.handle, int(m), int(n), int(platform))


def meanGpu(a, u, m, n):
    call("nsg_mean_gpu", a.handle, u.handle, int(m), int(n))


def standardDeviation(a, u, sigma, m, n, platform=GPU_PLATFORM):
    """Row means into u and population standard deviations into sigma."""
    call("nsg_standard_deviation", a.handle, u.handle, sigma.handle, int(m), int(n),
         int(platform))


def standardDeviationGpu(a, u, sigma, m, n):
    call("nsg_standard_deviation_gpu", a.handle, u.handle, sigma.handle, int(m), int(n))


def recoverSingleShortestPath(paths, maxPathLength, i, j) -> np.ndarray:
    """Node sequence from i to j as an int32 numpy array."""
    p = ctypes.POINTER(ctypes.c_int)()
    ln = ctypes.c_int()
    call("nsg_recover_single_shortest_path", paths.handle, int(maxPathLength), int(i), int(j),
         ctypes.byref(p), ctypes.byref(ln))
    try:
        return np.ctypeslib.as_array(p, shape=(ln.value,)).astype(np.int32).copy()
    finally:
        lib().nsg_free(p)


def generatePsi(psi, n) -> None:
    call("nsg_generate_psi", psi.handle, int(n))


class _SettingsMapping(Mapping):
    """Mapping view of a settings dataclass, so ``f(**settings)`` works; the
    checkpoint fields appear only when checkpointFrequency != -1."""

    def __iter__(self):
        names = [f.name for f in fields(self)]
        if self.checkpointFrequency == -1:
            names = [k for k in names if k not in ("checkpointFrequency", "checkpointFileName")]
        yield from names

    def items(self) -> ItemsView:
        return ItemsView({k: self[k] for k in self})

    def keys(self) -> KeysView:
        return KeysView(self)

    def values(self) -> ValuesView:
        return ValuesView({k: self[k] for k in self})

    def __len__(self) -> int:
        return sum(1 for _ in self)

    def __getitem__(self, key: str):
        return getattr(self, key)


@dataclass
class MutualInformationSettings(_SettingsMapping):
    """Keyword bundle for mutualInformation[WithCheckpointing]
    (netcalc/python/netcalc/__init__.py:30-71)."""

    X: FloatCuArray
    I: FloatCuArray
    ab: IntCuArray
    k: int
    n: int
    xd: int
    d: int
    platform: int = GPU_PLATFORM
    checkpointFrequency: int = -1
    checkpointFileName: Union[str, Path] = None

    def __post_init__(self):
        if self.checkpointFileName is not None:
            self.checkpointFileName = str(self.checkpointFileName)

    def __repr__(self):
        return (f"MutualInformationSettings(k={self.k}, n={self.n}, xd={self.xd}, d={self.d}, "
                f"platform={self.platform}, checkpointFrequency={self.checkpointFrequency}, "
                f"checkpointFileName={self.checkpointFileName})")


@dataclass
class GeneralizedCorrelationSettings(_SettingsMapping):
    """Keyword bundle for generalizedCorrelation[WithCheckpointing]
    (netcalc/python/netcalc/__init__.py:74-128). An empty ``ab`` is filled
    with all N*N ordered node pairs, N = X.n() / d."""

    X: FloatCuArray
    R: FloatCuArray
    ab: IntCuArray
    k: int
    n: int
    xd: int
    d: int
    platform: int = GPU_PLATFORM
    checkpointFrequency: int = -1
    checkpointFileName: Union[str, Path] = None

    def __post_init__(self):
        if self.checkpointFileName is not None:
            self.checkpointFileName = str(self.checkpointFileName)
        if not self.ab.size():
            print("Initializing ab")
            num_random_variables = int(self.X.n() / self.d)
            idx = np.arange(num_random_variables, dtype=np.int32)
            pairs = np.stack([np.repeat(idx, num_random_variables),
                              np.tile(idx, num_random_variables)], axis=1)
            self.ab.fromNumpy2D(pairs)

    def __repr__(self):
        return (f"GeneralizedCorrelationSettings(k={self.k}, n={self.n}, xd={self.xd}, "
                f"d={self.d}, platform={self.platform}, "
                f"checkpointFrequency={self.checkpointFrequency}, "
                f"checkpointFileName={self.checkpointFileName})")


__all__ = [
    "mutualInformation", "mutualInformationWithCheckpointing", "mutualInformationGpu",
    "mutualInformationCpu", "generalizedCorrelation", "generalizedCorrelationWithCheckpointing",
    "generalizedCorrelationGpu", "generalizedCorrelationCpu", "hedetniemiAllShortestPaths",
    "hedetniemiAllShortestPathsGpu", "hedetniemiAllShortestPathLengths",
    "hedetniemiAllShortestPathLengthsGpu", "correlationToAdjacency", "recoverSingleShortestPath",
    "mean", "meanGpu", "standardDeviation", "standardDeviationGpu",
    "GPU_PLATFORM", "CPU_PLATFORM", "generateRestartAbFromCheckpointFile", "generatePsi",
    "MutualInformationSettings", "GeneralizedCorrelationSettings", "FloatCuArray", "IntCuArray",
]
