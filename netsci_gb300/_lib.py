"""ctypes binding of the native library (include/netsci_gb300.h).

The library is built in-tree (``netsci_gb300/libnetsci_gb300.so``); importing
the Python layer never falls back to another implementation: when the
library is missing or fails to load, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libnetsci_gb300.so"

NSG_OK = 0
NSG_ERR_INVALID = 1
NSG_ERR_CUDA = 2
NSG_ERR_PLATFORM = 3
NSG_ERR_UNSUPPORTED = 4
NSG_ERR_DEVICE_FAULT = 5
NSG_ERR_IO = 6

DTYPE_FLOAT32 = 0
DTYPE_INT32 = 1
DTYPE_FLOAT64 = 2

c_int = ctypes.c_int
c_float = ctypes.c_float
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_char_p = ctypes.c_char_p
c_size_t = ctypes.c_size_t
P_int = ctypes.POINTER(ctypes.c_int)
P_float = ctypes.POINTER(ctypes.c_float)
P_double = ctypes.POINTER(ctypes.c_double)
P_size_t = ctypes.POINTER(ctypes.c_size_t)
PP_void = ctypes.POINTER(ctypes.c_void_p)
PP_int = ctypes.POINTER(ctypes.POINTER(ctypes.c_int))


class KsgPair(ctypes.Structure):
    """nsg_ksg_pair: one variable pair of device rows."""

    _fields_ = [("xa", c_void_p), ("xb", c_void_p), ("fmap", c_void_p), ("ld", c_int),
                ("m", c_int)]


class AtomInfo(ctypes.Structure):
    """nsg_atom_info."""

    _fields_ = [("index", c_int), ("serial", c_int), ("residue_id", c_int),
                ("occupancy", c_float), ("temperature_factor", c_float), ("mass", c_float),
                ("hash", ctypes.c_uint), ("name", ctypes.c_char * 8), ("element", ctypes.c_char * 4),
                ("residue_name", ctypes.c_char * 8), ("chain_id", ctypes.c_char * 4),
                ("segment_id", ctypes.c_char * 8), ("tag", ctypes.c_char * 40)]


class NodeInfo(ctypes.Structure):
    """nsg_node_info."""

    _fields_ = [("index", c_int), ("num_atoms", c_int), ("total_mass", c_float),
                ("hash", ctypes.c_uint), ("tag", ctypes.c_char * 40)]


class NsgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[nsg status {status}] {message}")
        self.status = status


# name: (restype, argtypes)
_SIGNATURES = {
    "nsg_last_error": (c_char_p, []),
    "nsg_version": (c_int, []),
    "nsg_release_cached_memory": (c_int, []),
    "nsg_free": (None, [c_void_p]),
    "nsg_cuarray_create": (c_int, [c_int, PP_void]),
    "nsg_cuarray_destroy": (c_int, [c_void_p]),
    "nsg_cuarray_dtype": (c_int, [c_void_p]),
    "nsg_cuarray_init": (c_int, [c_void_p, c_int, c_int, P_int]),
    "nsg_cuarray_init_from": (c_int, [c_void_p, c_void_p, c_int, c_int, P_int]),
    "nsg_cuarray_from_cuarray_shallow": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_int]),
    "nsg_cuarray_from_cuarray_deep": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_int]),
    "nsg_cuarray_from_host": (c_int, [c_void_p, c_void_p, c_int, c_int, P_int]),
    "nsg_cuarray_shape": (c_int, [c_void_p, P_int, P_int, P_int, P_size_t, P_int, P_int, P_int]),
    "nsg_cuarray_host": (c_void_p, [c_void_p]),
    "nsg_cuarray_device": (c_void_p, [c_void_p]),
    "nsg_cuarray_allocate_host": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_allocate_device": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_to_device": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_to_host": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_deallocate_host": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_deallocate_device": (c_int, [c_void_p, P_int]),
    "nsg_cuarray_get": (c_int, [c_void_p, c_int, c_int, P_double]),
    "nsg_cuarray_set": (c_int, [c_void_p, c_double, c_int, c_int, P_int]),
    "nsg_cuarray_load": (c_int, [c_void_p, c_char_p, P_int]),
    "nsg_cuarray_save": (c_int, [c_void_p, c_char_p]),
    "nsg_cuarray_sort": (c_int, [c_void_p, c_int, PP_void]),
    "nsg_cuarray_argsort": (c_int, [c_void_p, c_int, PP_void]),
    "nsg_mutual_information": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, P_int]),
    "nsg_mutual_information_checkpointed": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_char_p, P_int]),
    "nsg_mutual_information_gpu": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_float]),
    "nsg_mutual_information_cpu": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_float]),
    "nsg_generalized_correlation": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, P_int]),
    "nsg_generalized_correlation_checkpointed": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_char_p, P_int]),
    "nsg_generalized_correlation_gpu": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_float]),
    "nsg_generalized_correlation_cpu": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P_float]),
    "nsg_generate_restart_ab_from_checkpoint_file": (c_int, [c_void_p, c_void_p, c_char_p]),
    "nsg_hedetniemi_all_shortest_paths": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_float, c_int]),
    "nsg_hedetniemi_all_shortest_paths_gpu": (c_int, [c_void_p, c_void_p, c_void_p, c_float, c_int]),
    "nsg_hedetniemi_all_shortest_path_lengths": (c_int, [c_void_p, c_void_p, c_int, c_int]),
    "nsg_hedetniemi_all_shortest_path_lengths_gpu": (c_int, [c_void_p, c_void_p, c_int]),
    "nsg_correlation_to_adjacency": (c_int, [c_void_p, c_void_p, c_int, c_int]),
    "nsg_recover_single_shortest_path": (c_int, [c_void_p, c_int, c_int, c_int, PP_int, P_int]),
    "nsg_generate_psi": (c_int, [c_void_p, c_int]),
    "nsg_mean": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int]),
    "nsg_mean_gpu": (c_int, [c_void_p, c_void_p, c_int, c_int]),
    "nsg_standard_deviation": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "nsg_standard_deviation_gpu": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int]),
    "nsg_ksg_pairs_device": (c_int, [ctypes.POINTER(KsgPair), c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsg_ksg_pair_detail_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsg_ksg_pair_noalloc_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "nsg_ksg_plan_create": (c_int, [ctypes.POINTER(KsgPair), c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, PP_void]),
    "nsg_ksg_plan_run": (c_int, [c_void_p, c_void_p]),
    "nsg_ksg_plan_prepare": (c_int, [c_void_p]),
    "nsg_ksg_plan_check": (c_int, [c_void_p]),
    "nsg_ksg_plan_shape": (c_int, [c_void_p, P_int, P_int, P_int, P_int]),
    "nsg_ksg_plan_launches": (c_int, [c_void_p, P_int]),
    "nsg_ksg_plan_count_ms": (c_int, [c_void_p, P_float]),
    "nsg_ksg_plan_destroy": (c_int, [c_void_p]),
    "nsg_ksg_set_shape": (c_int, [c_int, c_int, c_int, c_int]),
    "nsg_ksg_set_staging": (c_int, [c_int]),
    "nsg_ksg_plan_staging": (c_int, [c_void_p, P_int]),
    "nsg_ksg_set_search": (c_int, [c_int]),
    "nsg_ksg_set_orders": (c_int, [c_int]),
    "nsg_apsp_set_method": (c_int, [c_int]),
    "nsg_measure_issue_ceiling": (c_int, [c_int, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "nsg_ksg_plan_search": (c_int, [c_void_p, P_int]),
    "nsg_ksg_plan_tied_samples": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "nsg_ksg_plan_kernel_ms": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float)]),
    "nsg_ksg_plan_evaluations": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_ulonglong),
                                         ctypes.POINTER(ctypes.c_ulonglong),
                                         ctypes.POINTER(ctypes.c_ulonglong)]),
    "nsg_server_create": (c_int, [c_size_t, c_double, c_int, PP_void]),
    "nsg_server_destroy": (c_int, [c_void_p]),
    "nsg_server_register_trajectory": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, P_int]),
    "nsg_server_submit_gc": (c_int, [c_void_p, c_int, c_int, c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "nsg_server_submit_mi": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "nsg_server_submit_apsp": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "nsg_server_wait": (c_int, [c_void_p, ctypes.c_longlong, c_double, P_int]),
    "nsg_server_job_info": (c_int, [c_void_p, ctypes.c_longlong, P_int, P_double, P_double, P_double]),
    "nsg_server_stats": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), P_size_t]),
    "nsg_apsp_lengths_device": (c_int, [c_void_p, c_void_p, c_int, c_int, P_int, c_void_p]),
    "nsg_apsp_paths_device": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_float, c_void_p]),
    "nsg_corr_to_adjacency_device": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "nsg_row_stats_device": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "nsg_network_create": (c_int, [PP_void]),
    "nsg_network_destroy": (c_int, [c_void_p]),
    "nsg_network_init": (c_int, [c_void_p, c_char_p, c_char_p, c_int, c_int, c_int]),
    "nsg_network_parse_pdb": (c_int, [c_void_p, c_char_p]),
    "nsg_network_num_nodes": (c_int, [c_void_p, P_int]),
    "nsg_network_num_frames": (c_int, [c_void_p, P_int]),
    "nsg_network_num_atoms": (c_int, [c_void_p, P_int]),
    "nsg_network_node_coordinates": (c_int, [c_void_p, c_void_p]),
    "nsg_network_load_node_coordinates": (c_int, [c_void_p, c_char_p]),
    "nsg_network_node": (c_int, [c_void_p, c_int, ctypes.POINTER(NodeInfo)]),
    "nsg_network_node_atoms": (c_int, [c_void_p, c_int, P_int, c_int, P_int]),
    "nsg_network_atom": (c_int, [c_void_p, c_int, ctypes.POINTER(AtomInfo)]),
    "nsg_network_node_from_atom": (c_int, [c_void_p, c_int, P_int]),
    "nsg_network_device_coordinates": (c_int, [c_void_p, PP_void, P_int]),
    "nsg_dcd_info": (c_int, [c_char_p, P_int, P_int]),
    "nsg_dcd_read": (c_int, [c_char_p, c_int, c_int, c_int, c_void_p]),
}

_LIB = None


def lib() -> ctypes.CDLL:
    """The loaded native library. Raises when it is missing: there is no
    fallback implementation."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing; build it with `python -m netsci_gb300.build` "
                "(or __graft_entry__.build())")
        L = ctypes.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_GLOBAL", 0))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(status: int) -> None:
    """Raise NsgError for a non-zero status, with the library's message."""
    if status != NSG_OK:
        msg = lib().nsg_last_error()
        raise NsgError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
