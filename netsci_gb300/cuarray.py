"""Python surface of the CuArray container: ``FloatCuArray`` and ``IntCuArray``.

Mirrors the reference's SWIG module ``cuarray`` (cuarray/swig/
python_cuarray_rename.i:1-39, python_cuarray_typemaps.i:15-142,
cuarray/python/cuarray/__init__.py:1-2): same class and method names,
the SWIG keyword names of the C++ parameters, numpy in/out through
``fromNumpy1D/2D`` and ``toNumpy1D/2D``, row proxies through ``[]``. Each
object wraps a C++ ``CuArray<T>`` owned through the C ABI.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import P_double, P_int, call, lib


class _CuArrayRow:
    """Proxy of one row (CuArrayRow<T>): indexing reads and writes the parent."""

    def __init__(self, parent: "_CuArrayBase", i: int):
        self._parent = parent
        self._i = i

    def __len__(self) -> int:
        return self._parent.n()

    def __getitem__(self, j: int):
        if j < 0 or j >= self._parent.n() or self._parent.n() == 0:
            raise IndexError("CuArrayRow index out of range")
        return self._parent.get(self._i, j)

    def __setitem__(self, j: int, value) -> None:
        if j < 0 or j >= self._parent.n() or self._parent.n() == 0:
            raise IndexError("CuArrayRow index out of range")
        self._parent.set(value, self._i, j)

    def __repr__(self) -> str:
        return " ".join(_fmt(v) for v in self._parent._row(self._i))


def _fmt(v) -> str:
    if isinstance(v, float) or isinstance(v, np.floating):
        return f"{float(v):.4f}"
    return str(int(v))


class _CuArrayBase:
    _dtype_code = _lib.DTYPE_FLOAT32
    _np = np.float32
    _cast = float

    def __init__(self, _handle: int | None = None):
        if _handle is None:
            h = ctypes.c_void_p()
            call("nsg_cuarray_create", self._dtype_code, ctypes.byref(h))
            _handle = h.value
        self._h = ctypes.c_void_p(_handle)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().nsg_cuarray_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    # -- shape ---------------------------------------------------------------
    def _shape(self):
        m, n, size, owner, ah, ad = (ctypes.c_int() for _ in range(6))
        b = ctypes.c_size_t()
        call("nsg_cuarray_shape", self._h, ctypes.byref(m), ctypes.byref(n), ctypes.byref(size),
             ctypes.byref(b), ctypes.byref(owner), ctypes.byref(ah), ctypes.byref(ad))
        return m.value, n.value, size.value, b.value, owner.value, ah.value, ad.value

    def m(self) -> int:
        return self._shape()[0]

    def n(self) -> int:
        return self._shape()[1]

    def size(self) -> int:
        return self._shape()[2]

    def bytes(self) -> int:
        return self._shape()[3]

    def owner(self) -> int:
        return self._shape()[4]

    def allocatedHost(self) -> int:
        return self._shape()[5]

    def allocatedDevice(self) -> int:
        return self._shape()[6]

    # -- storage -------------------------------------------------------------
    def _op(self, name: str) -> int:
        err = ctypes.c_int()
        call(name, self._h, ctypes.byref(err))
        return err.value

    def init(self, m: int, n: int) -> int:
        err = ctypes.c_int()
        call("nsg_cuarray_init", self._h, int(m), int(n), ctypes.byref(err))
        return err.value

    def allocateHost(self) -> int:
        return self._op("nsg_cuarray_allocate_host")

    def allocateDevice(self) -> int:
        return self._op("nsg_cuarray_allocate_device")

    def toDevice(self) -> int:
        return self._op("nsg_cuarray_to_device")

    def toHost(self) -> int:
        return self._op("nsg_cuarray_to_host")

    def deallocateHost(self) -> int:
        return self._op("nsg_cuarray_deallocate_host")

    def deallocateDevice(self) -> int:
        return self._op("nsg_cuarray_deallocate_device")

    def fromCuArray(self, cuArray: "_CuArrayBase", start: int, end: int, m: int, n: int) -> int:
        """Deep copy of rows start..end (SWIG rename of fromCuArrayDeepCopy)."""
        err = ctypes.c_int()
        call("nsg_cuarray_from_cuarray_deep", self._h, cuArray._h, int(start), int(end), int(m),
             int(n), ctypes.byref(err))
        self._keep = None
        return err.value

    def fromCuArrayShallowCopy(self, cuArray: "_CuArrayBase", start: int, end: int, m: int,
                               n: int) -> int:
        err = ctypes.c_int()
        call("nsg_cuarray_from_cuarray_shallow", self._h, cuArray._h, int(start), int(end),
             int(m), int(n), ctypes.byref(err))
        self._keep = cuArray  # the view borrows the source's host buffer
        return err.value

    # -- numpy ---------------------------------------------------------------
    def fromNumpy1D(self, NUMPY_ARRAY) -> int:
        a = np.ascontiguousarray(NUMPY_ARRAY, dtype=self._np).ravel()
        err = ctypes.c_int()
        call("nsg_cuarray_from_host", self._h, a.ctypes.data_as(ctypes.c_void_p), 1, a.size,
             ctypes.byref(err))
        return err.value

    def fromNumpy2D(self, NUMPY_ARRAY) -> int:
        a = np.ascontiguousarray(NUMPY_ARRAY, dtype=self._np)
        if a.ndim != 2:
            raise ValueError("fromNumpy2D expects a 2-D array")
        err = ctypes.c_int()
        call("nsg_cuarray_from_host", self._h, a.ctypes.data_as(ctypes.c_void_p), a.shape[0],
             a.shape[1], ctypes.byref(err))
        return err.value

    def _host_view(self) -> np.ndarray:
        m, n, size, _, _, ah, _ = self._shape()
        if not ah or size == 0:
            return np.zeros((m, n), dtype=self._np)
        p = lib().nsg_cuarray_host(self._h)
        buf = (ctypes.c_char * (size * np.dtype(self._np).itemsize)).from_address(p)
        return np.frombuffer(buf, dtype=self._np).reshape(m, n)

    def toNumpy1D(self) -> np.ndarray:
        return self._host_view().ravel().copy()

    def toNumpy2D(self) -> np.ndarray:
        return self._host_view().copy()

    def _row(self, i: int) -> np.ndarray:
        return self._host_view()[i]

    # -- elements ------------------------------------------------------------
    def get(self, i: int, j: int):
        v = ctypes.c_double()
        call("nsg_cuarray_get", self._h, int(i), int(j), ctypes.byref(v))
        return self._cast(v.value) if self._cast is int else float(self._np(v.value))

    def set(self, value, i: int, j: int) -> int:
        err = ctypes.c_int()
        call("nsg_cuarray_set", self._h, float(value), int(i), int(j), ctypes.byref(err))
        return err.value

    def load(self, fname) -> int:
        err = ctypes.c_int()
        call("nsg_cuarray_load", self._h, str(fname).encode(), ctypes.byref(err))
        return err.value

    def save(self, fname) -> None:
        call("nsg_cuarray_save", self._h, str(fname).encode())

    def sort(self, i: int):
        h = ctypes.c_void_p()
        call("nsg_cuarray_sort", self._h, int(i), ctypes.byref(h))
        return type(self)(_handle=h.value)

    def argsort(self, i: int) -> "IntCuArray":
        h = ctypes.c_void_p()
        call("nsg_cuarray_argsort", self._h, int(i), ctypes.byref(h))
        return IntCuArray(_handle=h.value)

    # -- python protocol -----------------------------------------------------
    def __len__(self) -> int:
        return self.m()

    def __getitem__(self, i: int) -> _CuArrayRow:
        if not self.allocatedHost():
            raise RuntimeError("CuArray memory not allocated")
        if i < 0 or i >= self.m():
            raise IndexError("CuArray index out of range")
        return _CuArrayRow(self, i)

    def __setitem__(self, i: int, row) -> None:
        if not self.allocatedHost():
            raise RuntimeError("CuArray memory not allocated")
        if i < 0 or i >= self.m():
            raise IndexError("CuArray index out of range")
        for j in range(len(row)):
            self.set(row[j], i, j)

    def __repr__(self) -> str:
        if not self.allocatedHost():
            return "null"
        return "\n".join(" ".join(_fmt(v) for v in r) for r in self._host_view())


class FloatCuArray(_CuArrayBase):
    """CuArray<float>."""

    _dtype_code = _lib.DTYPE_FLOAT32
    _np = np.float32
    _cast = float


class IntCuArray(_CuArrayBase):
    """CuArray<int>."""

    _dtype_code = _lib.DTYPE_INT32
    _np = np.int32
    _cast = int


__all__ = ["FloatCuArray", "IntCuArray"]
