"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes bindings for the CPU restatement (``liboracle.so``, built from
``ksg_oracle.cpp`` and ``apsp_oracle.cpp``) and, when present, for the
reference's own CPU functions compiled into ``_ref/liboracle_ref.so``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import
this package; the product (``netsci_gb300``) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None
_REF = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile the restatement (and the reference CPU library when its
    sources are present, or when ``ref`` is True)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    ref_root = os.environ.get("NETSCI_REF", "/root/reference")
    if ref is None:
        ref = Path(ref_root, "netcalc", "src").is_dir()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"NETSCI_REF={ref_root}"],
                       check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            build(ref=False)
        L = ctypes.CDLL(str(path))
        L.oracle_psi.argtypes = [_f32p, ctypes.c_int]
        L.oracle_psi.restype = None
        L.oracle_mi_pair.argtypes = [
            _f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_mi_pair.restype = ctypes.c_float
        L.oracle_mi_from_counts.argtypes = [_i32p, _i32p, ctypes.c_int, ctypes.c_int, _f32p]
        L.oracle_mi_from_counts.restype = ctypes.c_float
        L.oracle_gc_from_mi.argtypes = [ctypes.c_float, ctypes.c_int]
        L.oracle_gc_from_mi.restype = ctypes.c_float
        L.oracle_pairs.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p, ctypes.c_int]
        L.oracle_pairs.restype = None
        L.oracle_apsp_lengths.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int)]
        L.oracle_apsp_lengths.restype = ctypes.c_int
        L.oracle_floyd_warshall.argtypes = [_f32p, _f32p, ctypes.c_int]
        L.oracle_floyd_warshall.restype = None
        L.oracle_apsp_paths.argtypes = [_f32p, _f32p, _i32p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float]
        L.oracle_apsp_paths.restype = None
        L.oracle_corr_to_adj.argtypes = [_f32p, _f32p, ctypes.c_int]
        L.oracle_corr_to_adj.restype = None
        L.oracle_corr_to_neglog_adj.argtypes = [_f32p, _f32p, ctypes.c_int]
        L.oracle_corr_to_neglog_adj.restype = None
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's CPU functions, or None when oracle/_ref was not built."""
    global _REF
    if _REF is None:
        path = HERE / "_ref" / "liboracle_ref.so"
        if not path.exists():
            return None
        try:
            R = ctypes.CDLL(str(path))
        except OSError:
            return None
        for name in ("ref_mi_cpu", "ref_gc_cpu"):
            fn = getattr(R, name)
            fn.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            fn.restype = ctypes.c_float
        R.ref_psi.argtypes = [_f32p, ctypes.c_int]
        R.ref_psi.restype = None
        _REF = R
    return _REF


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def psi(n: int) -> np.ndarray:
    out = np.zeros(n + 1, np.float32)
    lib().oracle_psi(out, n)
    return out


def mi_pair(xa, xb, n: int, k: int, d: int, detail: bool = False):
    """KSG MI of one pair. With ``detail`` also returns a dict of per-sample
    n_x, n_y, eps_x, eps_y, kdist and the tie count."""
    xa = _c(xa, np.float32).ravel()
    xb = _c(xb, np.float32).ravel()
    table = psi(n)
    if not detail:
        return float(lib().oracle_mi_pair(xa, xb, n, k, d, table, None, None, None, None,
                                          None, None))
    nx = np.zeros(n, np.int32)
    ny = np.zeros(n, np.int32)
    ex = np.zeros(n, np.float32)
    ey = np.zeros(n, np.float32)
    kd = np.zeros(n, np.float32)
    ties = ctypes.c_int(0)
    mi = lib().oracle_mi_pair(xa, xb, n, k, d, table, nx.ctypes.data, ny.ctypes.data,
                              ex.ctypes.data, ey.ctypes.data, kd.ctypes.data,
                              ctypes.addressof(ties))
    return float(mi), dict(n_x=nx, n_y=ny, eps_x=ex, eps_y=ey, kdist=kd, ties=ties.value)


def mi_from_counts(nx, ny, n: int, k: int) -> float:
    return float(lib().oracle_mi_from_counts(_c(nx, np.int32), _c(ny, np.int32), n, k, psi(n)))


def gc_from_mi(mi: float, d: int) -> float:
    return float(lib().oracle_gc_from_mi(mi, d))


def pairs(X, n: int, d: int, ab, k: int, gc: bool = False, threads: int = 1) -> np.ndarray:
    X = _c(X, np.float32)
    ab = _c(ab, np.int32).reshape(-1, 2)
    out = np.zeros(ab.shape[0], np.float32)
    lib().oracle_pairs(X.ravel(), X.shape[0], n, d, ab.ravel(), ab.shape[0], k, int(gc), out,
                       threads)
    return out


def apsp_lengths(A, max_path_length: int):
    A = _c(A, np.float32)
    n = A.shape[0]
    H = np.zeros_like(A)
    conv = ctypes.c_int(0)
    steps = lib().oracle_apsp_lengths(A.ravel(), H.ravel(), n, max_path_length,
                                      ctypes.byref(conv))
    return H, steps, bool(conv.value)


def floyd_warshall(A):
    A = _c(A, np.float32)
    D = np.zeros_like(A)
    lib().oracle_floyd_warshall(A.ravel(), D.ravel(), A.shape[0])
    return D


def apsp_paths(A, max_path_length: int, tolerance: float):
    A = _c(A, np.float32)
    n = A.shape[0]
    H = np.zeros_like(A)
    P = np.zeros(n * max_path_length * n, np.int32)
    lib().oracle_apsp_paths(A.ravel(), H.ravel(), P, n, max_path_length, tolerance)
    return H, P


def corr_to_adj(C):
    C = _c(C, np.float32)
    A = np.zeros_like(C)
    lib().oracle_corr_to_adj(C.ravel(), A.ravel(), C.shape[0])
    return A


def corr_to_neglog_adj(C):
    C = _c(C, np.float32)
    A = np.zeros_like(C)
    lib().oracle_corr_to_neglog_adj(C.ravel(), A.ravel(), C.shape[0])
    return A


def _fold_1024(p: np.ndarray) -> np.float32:
    """Pairwise fold p[t] += p[t + s], s = 512 .. 1, in float32
    (netcalc/src/math_utils_gpu.cu:10-20,36-60)."""
    p = p.copy()
    s = 512
    while s >= 1:
        p[:s] = p[:s] + p[s:2 * s]
        s >>= 1
    return p[0]


def row_stats(a, n: int):
    """Row means and population standard deviations of a (rows of n values)
    in the reference kernels' summation order: thread slot t of 1024 sums
    a[t], a[t + 1024], ... sequentially in float32, then the 1024 partial sums
    are folded pairwise (netcalc/src/math_utils_gpu.cu:22-158). The square is
    d * d (the reference writes powf(d, 2.0))."""
    a = _c(a, np.float32).ravel()
    m = a.size // n
    a = a[:m * n].reshape(m, n)
    nf = np.float32(n)
    u = np.zeros(m, np.float32)
    sigma = np.zeros(m, np.float32)
    for r in range(m):
        p = np.zeros(1024, np.float32)
        for j0 in range(0, n, 1024):
            chunk = a[r, j0:j0 + 1024]
            p[:chunk.size] = p[:chunk.size] + chunk
        u[r] = np.float32(_fold_1024(p) / nf)
        q = np.zeros(1024, np.float32)
        for j0 in range(0, n, 1024):
            dv = a[r, j0:j0 + 1024] - u[r]
            q[:dv.size] = q[:dv.size] + dv * dv
        sigma[r] = np.sqrt(np.float32(_fold_1024(q) / nf), dtype=np.float32)
    return u, sigma
