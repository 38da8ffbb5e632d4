"""Drop-in module ``netcalc``: the reference's import name for the netcalc
functions, constants and Settings dataclasses
(netcalc/python/netcalc/__init__.py:5-128)."""
from netsci_gb300.netcalc import *  # noqa: F401,F403
from netsci_gb300.netcalc import __all__  # noqa: F401
