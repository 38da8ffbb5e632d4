"""netsci_gb300: GB300-native implementation of NetSci's netcalc hot path.

KSG mutual information, generalized correlation and Hedetniemi all-pairs
shortest paths as hand-written sm_103a CUDA kernels behind a C ABI
(include/netsci_gb300.h), with the reference's CuArray / netcalc surface
on top:

* ``netsci_gb300.cuarray``  -- FloatCuArray / IntCuArray
* ``netsci_gb300.netcalc``  -- mutualInformation, generalizedCorrelation,
  hedetniemiAllShortestPaths, ... (reference names and keywords)
* ``netsci_gb300.device``   -- device-resident batched entry points
* ``netsci_gb300/dropin``   -- put this directory on sys.path to import the
  modules under the reference's names ``cuarray`` and ``netcalc``.
"""
from ._lib import NsgError, lib  # noqa: F401
from .build import build  # noqa: F401

__version__ = "0.1.0"
