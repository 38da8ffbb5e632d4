"""Drop-in module ``cuarray``: the reference's import name for the CuArray
classes (cuarray/python/cuarray/__init__.py:1-2)."""
from netsci_gb300.cuarray import FloatCuArray, IntCuArray  # noqa: F401
