"""netchem: trajectory -> node coordinates (netchem/python/netchem/__init__.py,
netchem/swig/python_netchem*.i).

``Network().init(trajectoryFile, topologyFile, firstFrame, lastFrame,
stride)`` groups the PDB's atoms into residue nodes and computes each node's
mass-weighted centre for the selected DCD frames on the GPU
(include/netsci_gb300.h, section 5). ``nodeCoordinates()`` is the N x 3m
``FloatCuArray`` that ``netcalc.generalizedCorrelation`` takes as X;
``deviceCoordinates()`` is the same data already resident on the device in
the packed layout of ``netsci_gb300.device`` (no host round trip).
``Atom``, ``Atoms`` and ``Node`` are read-only views with the reference's
accessor names; iteration and ``repr`` follow the SWIG extensions.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields
from pathlib import Path
from typing import ItemsView, KeysView, Mapping, Union, ValuesView

import numpy as np

from ._lib import AtomInfo, NodeInfo, call, lib
from .cuarray import FloatCuArray


class Atom:
    def __init__(self, info: AtomInfo):
        self._i = info

    def index(self) -> int:
        return self._i.index

    def name(self) -> str:
        return self._i.name.decode()

    def element(self) -> str:
        return self._i.element.decode()

    def residueName(self) -> str:
        return self._i.residue_name.decode()

    def residueId(self) -> int:
        return self._i.residue_id

    def chainId(self) -> str:
        return self._i.chain_id.decode()

    def segmentId(self) -> str:
        return self._i.segment_id.decode()

    def temperatureFactor(self) -> float:
        return self._i.temperature_factor

    def occupancy(self) -> float:
        return self._i.occupancy

    def serial(self) -> int:
        return self._i.serial

    def tag(self) -> str:
        return self._i.tag.decode()

    def mass(self) -> float:
        return self._i.mass

    def hash(self) -> int:
        return self._i.hash

    def __repr__(self) -> str:
        return (f"Index: {self.index()}\nSerial: {self.serial()}\nName: {self.name()}\n"
                f"Element: {self.element()}\nResidue ID: {self.residueId()}\n"
                f"Residue Name: {self.residueName()}\nChain ID: {self.chainId()}\n"
                f"Segment ID: {self.segmentId()}\nMass: {self.mass():g}")


class Atoms:
    def __init__(self, net: "Network"):
        self._net = net

    def numAtoms(self) -> int:
        n = ctypes.c_int()
        call("nsg_network_num_atoms", self._net._h, ctypes.byref(n))
        return n.value

    def at(self, atomIndex: int) -> Atom:
        info = AtomInfo()
        call("nsg_network_atom", self._net._h, int(atomIndex), ctypes.byref(info))
        return Atom(info)

    def numUniqueTags(self) -> int:
        return self._net.numNodes()

    def atoms(self) -> list[Atom]:
        return [self.at(i) for i in range(self.numAtoms())]

    def __getitem__(self, atomIndex: int) -> Atom:
        return self.at(atomIndex)

    def __len__(self) -> int:
        return self.numAtoms()

    def __iter__(self):
        return (self.at(i) for i in range(self.numAtoms()))


class Node:
    def __init__(self, net: "Network", info: NodeInfo):
        self._net = net
        self._i = info

    def tag(self) -> str:
        return self._i.tag.decode()

    def numAtoms(self) -> int:
        return self._i.num_atoms

    def index(self) -> int:
        return self._i.index

    def totalMass(self) -> float:
        return self._i.total_mass

    def hash(self) -> int:
        return self._i.hash

    def atoms(self) -> list[Atom]:
        n = self._i.num_atoms
        idx = (ctypes.c_int * max(1, n))()
        cnt = ctypes.c_int()
        call("nsg_network_node_atoms", self._net._h, self._i.index, idx, n, ctypes.byref(cnt))
        a = Atoms(self._net)
        return [a.at(idx[i]) for i in range(cnt.value)]

    def __repr__(self) -> str:
        return (f"Index: {self.index()}\nTag: {self.tag()}\nTotal Mass: {self.totalMass():g}\n"
                f"Number of Atoms: {self.numAtoms()}")


class Network:
    def __init__(self):
        h = ctypes.c_void_p()
        call("nsg_network_create", ctypes.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().nsg_network_destroy(h)
            except Exception:
                pass
            self._h = None

    def init(self, trajectoryFile, topologyFile, firstFrame: int, lastFrame: int,
             stride: int = 1) -> None:
        call("nsg_network_init", self._h, str(trajectoryFile).encode(), str(topologyFile).encode(),
             int(firstFrame), int(lastFrame), int(stride))

    def parsePdb(self, fname) -> None:
        call("nsg_network_parse_pdb", self._h, str(fname).encode())

    def numNodes(self) -> int:
        n = ctypes.c_int()
        call("nsg_network_num_nodes", self._h, ctypes.byref(n))
        return n.value

    def numFrames(self) -> int:
        n = ctypes.c_int()
        call("nsg_network_num_frames", self._h, ctypes.byref(n))
        return n.value

    def nodeCoordinates(self, nodeCoordinatesFile=None):
        """Without an argument: the node coordinates as a FloatCuArray (a copy).
        With a file name: replace them by that .npy file."""
        if nodeCoordinatesFile is not None:
            call("nsg_network_load_node_coordinates", self._h, str(nodeCoordinatesFile).encode())
            return None
        out = FloatCuArray()
        call("nsg_network_node_coordinates", self._h, out.handle)
        return out

    def nodes(self) -> list[Node]:
        out = []
        for i in range(self.numNodes()):
            info = NodeInfo()
            call("nsg_network_node", self._h, i, ctypes.byref(info))
            out.append(Node(self, info))
        return out

    def nodeFromAtomIndex(self, atomIndex: int) -> Node:
        n = ctypes.c_int()
        call("nsg_network_node_from_atom", self._h, int(atomIndex), ctypes.byref(n))
        info = NodeInfo()
        call("nsg_network_node", self._h, n.value, ctypes.byref(info))
        return Node(self, info)

    def atoms(self) -> Atoms:
        return Atoms(self)

    def __iter__(self):
        return iter(self.nodes())

    def deviceCoordinates(self):
        """(X, m): a torch tensor view (N, 3, ld) of the device-resident node
        coordinates (valid while this Network lives and is not re-initialised)
        and the frame count; the layout ``device.make_pairs`` takes."""
        import torch
        p = ctypes.c_void_p()
        ld = ctypes.c_int()
        call("nsg_network_device_coordinates", self._h, ctypes.byref(p), ctypes.byref(ld))
        if not p.value:
            raise RuntimeError("no device coordinates (init() has not run)")
        N = self.numNodes()
        # borrow the buffer through __cuda_array_interface__ without a copy
        holder = _DeviceView(p.value, (N, 3, ld.value), self)
        return torch.as_tensor(holder, device="cuda"), self.numFrames()


class _DeviceView:
    def __init__(self, ptr: int, shape: tuple, owner):
        self._owner = owner
        self.__cuda_array_interface__ = dict(shape=shape, typestr="<f4", data=(ptr, False),
                                             version=3, strides=None)


Graph = Network


def dcd_info(path) -> tuple[int, int]:
    """(atoms, frames) of a DCD file."""
    na, ns = ctypes.c_int(), ctypes.c_int()
    call("nsg_dcd_info", str(path).encode(), ctypes.byref(na), ctypes.byref(ns))
    return na.value, ns.value


def dcd_read(path, first: int = 0, count: int | None = None, stride: int = 1) -> np.ndarray:
    """Frames of a DCD file as float32 [count, 3, atoms] (host reader)."""
    na, ns = dcd_info(path)
    if count is None:
        count = len(range(first, ns, stride))
    out = np.empty((count, 3, na), np.float32)
    call("nsg_dcd_read", str(path).encode(), int(first), int(count), int(stride),
         out.ctypes.data_as(ctypes.c_void_p))
    return out


@dataclass
class NetworkSettings(Mapping):
    """Keyword arguments of Network.init (netchem/python/netchem/__init__.py:17-46)."""
    trajectoryFile: Union[str, Path]
    topologyFile: Union[str, Path]
    firstFrame: int
    lastFrame: int
    stride: int = 1

    def __post_init__(self):
        self.trajectoryFile = str(self.trajectoryFile)
        self.topologyFile = str(self.topologyFile)

    def __iter__(self):
        return iter([f.name for f in fields(self)])

    def __len__(self):
        return len(fields(self))

    def __getitem__(self, key: str):
        return getattr(self, key)

    def items(self) -> ItemsView:
        return ItemsView(self)

    def keys(self) -> KeysView:
        return KeysView(self)

    def values(self) -> ValuesView:
        return ValuesView(self)


__all__ = ["Atom", "Atoms", "Node", "Network", "Graph", "NetworkSettings", "dcd_info", "dcd_read"]
