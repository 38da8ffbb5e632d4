"""Drop-in module ``netchem``: the reference's import name for Network, Node,
Atoms, Atom, Graph and NetworkSettings (netchem/python/netchem/__init__.py:1-46)."""
from netsci_gb300.netchem import *  # noqa: F401,F403
from netsci_gb300.netchem import __all__  # noqa: F401
