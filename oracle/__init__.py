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


REPO = HERE.parent


def ref_root() -> Path:
    """Where the reference sources are compiled from: NETSCI_REF, else the
    copy that ``make -C oracle stage`` leaves in baseline/_ref/netsci."""
    return Path(os.environ.get("NETSCI_REF", str(REPO / "baseline" / "_ref" / "netsci")))


def have_ref_sources() -> bool:
    return Path(ref_root(), "netcalc", "src").is_dir()


def build(ref: bool | None = None) -> None:
    """Compile the restatement (and the reference CPU libraries when their
    sources are present, or when ``ref`` is True)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref is None:
        ref = have_ref_sources()
    if ref:
        subprocess.run(["make", "-s", "-j4", "-C", str(HERE), "ref", f"NETSCI_REF={ref_root()}"],
                       check=True)


def start_ref_gpu_build():
    """Start compiling the reference's GPU code for sm_103a in the background
    (about half a minute); returns the process, or None when the sources are
    absent. ``finish_ref_gpu_build`` waits for it."""
    if not have_ref_sources():
        return None
    jobs = str(max(2, min(8, os.cpu_count() or 2)))
    return subprocess.Popen(["make", "-s", f"-j{jobs}", "-C", str(HERE), "ref-gpu",
                             f"NETSCI_REF={ref_root()}"],
                            stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


def finish_ref_gpu_build(proc) -> None:
    if proc is None:
        return
    out, _ = proc.communicate()
    if proc.returncode != 0:
        raise RuntimeError(f"make ref-gpu failed:\n{out}")


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
        L.oracle_mi_pair_mt.argtypes = L.oracle_mi_pair.argtypes + [ctypes.c_int]
        L.oracle_mi_pair_mt.restype = ctypes.c_float
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
        R.ref_pairs_checkpoint.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_char_p, _f32p]
        R.ref_pairs_checkpoint.restype = ctypes.c_int
        R.ref_restart_ab.argtypes = [_i32p, ctypes.c_int, ctypes.c_char_p, _i32p, ctypes.c_int]
        R.ref_restart_ab.restype = ctypes.c_int
        _REF = R
    return _REF


_REF_GPU = None


def ref_gpu_lib():
    """The reference's GPU functions (``_ref/libnetcalc_ref_gpu.so``), or None
    when that library was not built."""
    global _REF_GPU
    if _REF_GPU is None:
        path = HERE / "_ref" / "libnetcalc_ref_gpu.so"
        if not path.exists():
            return None
        G = ctypes.CDLL(str(path))
        for name in ("refgpu_mi", "refgpu_gc"):
            fn = getattr(G, name)
            fn.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            fn.restype = ctypes.c_float
        G.refgpu_apsp_lengths.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int]
        G.refgpu_apsp_lengths.restype = None
        G.refgpu_row_stats.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, _f32p, _f32p, _f32p]
        G.refgpu_row_stats.restype = None
        _REF_GPU = G
    return _REF_GPU


def ref_gpu_apsp_lengths(A, max_path_length: int) -> np.ndarray:
    """The reference kernel's shortest-path lengths after max_path_length
    launches (hedetniemi_gpu.cu:109-146)."""
    A = _c(A, np.float32)
    H = np.zeros_like(A)
    ref_gpu_lib().refgpu_apsp_lengths(A.ravel(), H.ravel(), A.shape[0], int(max_path_length))
    return H


def ref_gpu_row_stats(a):
    """The reference's row means (mean) and, from standardDeviation, its row
    means and population standard deviations, GPU platform
    (math_utils.cpp:6-36, math_utils_gpu.cu:22-198); a is m x n."""
    a = _c(a, np.float32)
    m, n = a.shape
    u, u2, s = (np.zeros(m, np.float32) for _ in range(3))
    ref_gpu_lib().refgpu_row_stats(a.ravel(), m, n, u, u2, s)
    return u, u2, s


def ref_pairs_checkpoint(X, n: int, d: int, ab, k: int, gc: bool, frequency: int,
                         file_name: str):
    """The reference pair-list driver with checkpoint files, CPU platform
    (mutual_information.cpp:8-101 / generalized_correlation.cpp:8-102)."""
    X = _c(X, np.float32)
    ab = _c(ab, np.int32).reshape(-1, 2)
    out = np.zeros(ab.shape[0], np.float32)
    rc = ref_lib().ref_pairs_checkpoint(X.ravel(), X.shape[0], n, d, ab.ravel(), ab.shape[0], k,
                                        int(gc), int(frequency), file_name.encode(), out)
    return rc, out


def ref_restart_ab(ab, checkpoint_file_name: str) -> np.ndarray:
    """generateRestartAbFromCheckpointFile (mutual_information.cpp:174-201)."""
    ab = _c(ab, np.int32).reshape(-1, 2)
    out = np.zeros_like(ab)
    m = ref_lib().ref_restart_ab(ab.ravel(), ab.shape[0], checkpoint_file_name.encode(),
                                 out.reshape(-1), ab.shape[0])
    return out[:m]


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def psi(n: int) -> np.ndarray:
    out = np.zeros(n + 1, np.float32)
    lib().oracle_psi(out, n)
    return out


def mi_pair(xa, xb, n: int, k: int, d: int, detail: bool = False, threads: int = 1):
    """KSG MI of one pair, its samples spread over ``threads`` host threads
    (the result does not depend on the thread count). With ``detail`` also
    returns a dict of per-sample n_x, n_y, eps_x, eps_y, kdist and the tie
    count."""
    xa = _c(xa, np.float32).ravel()
    xb = _c(xb, np.float32).ravel()
    table = psi(n)
    if not detail:
        return float(lib().oracle_mi_pair_mt(xa, xb, n, k, d, table, None, None, None, None,
                                             None, None, int(threads)))
    nx = np.zeros(n, np.int32)
    ny = np.zeros(n, np.int32)
    ex = np.zeros(n, np.float32)
    ey = np.zeros(n, np.float32)
    kd = np.zeros(n, np.float32)
    ties = ctypes.c_int(0)
    mi = lib().oracle_mi_pair_mt(xa, xb, n, k, d, table, nx.ctypes.data, ny.ctypes.data,
                                 ex.ctypes.data, ey.ctypes.data, kd.ctypes.data,
                                 ctypes.addressof(ties), int(threads))
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


# ---------------------------------------------------------------------------
# netchem: PDB topology + DCD trajectory -> node centres of mass
# ---------------------------------------------------------------------------
_ATOMIC_WEIGHTS_G = {  # g/mol; netchem/include/chemical_properties.h:49-168 holds them / 1000
    "H": "1.00794", "He": "4.002602", "Li": "6.941", "Be": "9.01218", "B": "10.811",
    "C": "12.011", "N": "14.00674", "O": "15.9994", "F": "18.998403", "Ne": "20.1797",
    "Na": "22.989768", "Mg": "24.305", "Al": "26.981539", "Si": "28.0855", "P": "30.973762",
    "S": "32.066", "Cl": "35.4527", "Ar": "39.948", "K": "39.0983", "Ca": "40.078",
    "Sc": "44.95591", "Ti": "47.88", "Cr": "51.9961", "Mn": "54.93805", "Fe": "55.847",
    "Co": "58.9332", "Ni": "58.6934", "Cu": "63.546", "Zn": "65.39", "Ga": "69.723",
    "Ge": "72.61", "As": "74.92159", "Se": "78.96", "Br": "79.904", "Kr": "83.8",
    "Rb": "85.4678", "Sr": "87.62", "Y": "88.90585", "Zr": "91.224", "Nb": "92.90638",
    "Mo": "95.94", "Tc": "97.9072", "Ru": "101.07", "Rh": "102.9055", "Pd": "106.42",
    "Ag": "107.8682", "Cd": "112.411", "In": "114.818", "Sn": "118.71", "Sb": "121.76",
    "Te": "127.6", "I": "126.90447", "Xe": "131.29", "Cs": "132.90543", "Ba": "137.327",
    "La": "138.9055", "Ce": "140.115", "Pr": "140.90765", "Nd": "144.24", "Pm": "144.9127",
    "Sm": "150.36", "Eu": "151.965", "Gd": "157.25", "Tb": "158.92534", "Dy": "162.5",
    "Ho": "164.93032", "Er": "167.26", "Tm": "168.93421", "Yb": "173.04", "Lu": "174.967",
    "Hf": "178.49", "Ta": "180.9479", "W": "183.84", "Re": "186.207", "Os": "190.23",
    "Ir": "192.22", "Pt": "195.08", "Au": "196.96654", "Hg": "200.59", "Tl": "204.3833",
    "Pb": "207.2", "Bi": "208.98037", "Po": "208.9824", "At": "209.9871", "Rn": "222.0176",
    "Fr": "223.0197", "Ra": "226.0254", "Ac": "227.0278", "Th": "232.0381", "Pa": "231.03588",
    "U": "238.0289", "Np": "237.048", "Pu": "244.0642", "Am": "243.0614", "Cm": "247.0703",
    "Bk": "247.0703", "Cf": "251.0796", "Es": "252.083", "Fm": "257.0951", "Md": "258.1",
    "No": "259.1009", "Lr": "262.11", "Rf": "261", "Db": "262", "Sg": "266", "Bh": "264",
    "Hs": "269", "Mt": "268", "Ds": "269", "Rg": "272", "Cn": "277", "Nh": "0", "Fl": "289",
    "Mc": "0", "Lv": "0", "Ts": "0", "Og": "0",
}


def atomic_weight_kg(symbol: str) -> float:
    """kg/mol as the double the reference's table literal parses to."""
    g = _ATOMIC_WEIGHTS_G.get(symbol)
    return 0.0 if g is None else float(g + "e-3")


def _hash_string(s: str) -> int:
    """netchem/src/utils.cpp:94-110 with characters taken as signed."""
    h = 37
    for ch in s.encode():
        c = ch - 256 if ch > 127 else ch
        h = ((h * 54059) ^ ((c * 76963) & 0xFFFFFFFF)) & 0xFFFFFFFF
    return h


def pdb_atoms(path) -> list[dict]:
    """ATOM records as netchem reads them (netchem/src/network.cpp:258-278,
    netchem/src/atom.cpp:177-291)."""
    out = []
    with open(path, "r", newline="") as f:
        for raw in f:
            line = raw[:-1] if raw.endswith("\n") else raw
            if "ATOM" not in line:
                continue
            idx = len(out)

            def fld(p, n):
                if p > len(line):
                    raise ValueError(f"ATOM record {idx} too short")
                return "".join(line[p:p + n].split())
            el = fld(76, 2).lower()
            el = el[:1].upper() + el[1:]
            resid_s = fld(22, 4)
            a = dict(index=idx, serial=idx + 1, name=fld(12, 3), residueName=fld(17, 3),
                     chainId=fld(21, 1), residueId=int(resid_s), occupancy=np.float32(float(fld(54, 6))),
                     segmentId=fld(72, 4), element=el)
            a["temperatureFactor"] = a["occupancy"]
            a["tag"] = f'{a["residueName"]}_{resid_s}_{a["chainId"]}_{a["segmentId"]}'
            a["mass"] = np.float32(1000.0 * atomic_weight_kg(el))
            a["hash"] = _hash_string(f'{idx}_{a["tag"]}')
            out.append(a)
    return out


def dcd_read(path):
    """(header dict, frames) with frames float32 [nsets, 3, natoms]: a DCD
    reader written from the format (CHARMM / X-PLOR, 4- or 8-byte record
    markers, either byte order; no fixed atoms)."""
    b = Path(path).read_bytes()
    import struct
    for bo in ("<", ">"):
        for mw in (4, 8):
            fmt = bo + ("i" if mw == 4 else "q")
            if len(b) >= mw + 4 and struct.unpack(fmt, b[:mw])[0] == 84 and b[mw:mw + 4] == b"CORD":
                break
        else:
            continue
        break
    else:
        raise ValueError("not a DCD file")
    mk = bo + ("i" if mw == 4 else "q")

    def marker(p):
        return struct.unpack(mk, b[p:p + mw])[0]
    words = struct.unpack(bo + "20i", b[mw + 4:mw + 84])
    charmm = words[19] != 0
    cell = charmm and words[10] != 0
    four = charmm and words[11] == 1
    if words[8] != 0:
        raise ValueError("fixed atoms")
    p = mw + 84
    assert marker(p) == 84
    p += mw
    tlen = marker(p)
    p += mw + tlen
    assert marker(p) == tlen
    p += mw
    assert marker(p) == 4
    natoms = struct.unpack(bo + "i", b[p + mw:p + mw + 4])[0]
    p += mw + 4
    assert marker(p) == 4
    p += mw
    rec = 2 * mw + 4 * natoms
    fb = (2 * mw + 48 if cell else 0) + (4 if four else 3) * rec
    nsets = (len(b) - p) // fb
    frames = np.empty((nsets, 3, natoms), np.float32)
    dt = np.dtype(np.float32).newbyteorder(bo)
    for f in range(nsets):
        q = p + f * fb + (2 * mw + 48 if cell else 0)
        for c in range(3):
            assert marker(q) == 4 * natoms
            frames[f, c] = np.frombuffer(b, dt, natoms, q + mw)
            q += rec
    return dict(natoms=natoms, nsets=nsets, charmm=charmm, unit_cell=cell, header_nsets=words[0]), frames


def node_coordinates(trajectory, topology, first: int, last: int, stride: int = 1):
    """(X, nodes): X float32 [N, 3m] of node mass-weighted centres, nodes a
    list of (tag, atom indices, total mass): netchem/src/network.cpp:29-255,
    float32 arithmetic in the same order (per node, atoms in index order,
    acc = acc + x * mass, then / total mass)."""
    atoms = pdb_atoms(topology)
    _, frames = dcd_read(trajectory)
    if last == -1:
        last = frames.shape[0] - 1
    sel = np.arange(first, last + 1, stride)
    fr = frames[sel]
    tags, members = {}, []
    for a in atoms:
        if a["tag"] not in tags:
            tags[a["tag"]] = len(members)
            members.append([])
        members[tags[a["tag"]]].append(a["index"])
    N, m = len(members), len(sel)
    X = np.zeros((N, 3, m), np.float32)
    nodes = []
    for n, mem in enumerate(members):
        tm = np.float32(0)
        acc = np.zeros((3, m), np.float32)
        for ai in mem:
            w = atoms[ai]["mass"]
            tm = np.float32(tm + w)
            acc = acc + fr[:, :, ai].T * w
        X[n] = acc / tm
        nodes.append((atoms[mem[0]]["tag"], mem, tm))
    return X.reshape(N, 3 * m), nodes


def ref_netchem():
    """The reference's DCD plugin and Atom class compiled into
    ``_ref/libnetchem_ref.so`` (None when absent)."""
    p = HERE / "_ref" / "libnetchem_ref.so"
    if not p.exists():
        return None
    L = ctypes.CDLL(str(p))
    L.ref_dcd_frames.restype = ctypes.c_int
    L.ref_dcd_frames.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    L.ref_pdb_atoms.restype = ctypes.c_int
    L.ref_pdb_atoms.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
    return L


def ref_dcd_frames(path):
    """float32 [nsets, 3, natoms] through the reference's DCD plugin."""
    L = ref_netchem()
    na, ns = ctypes.c_int(), ctypes.c_int()
    assert L.ref_dcd_frames(str(path).encode(), ctypes.byref(na), ctypes.byref(ns), None) == 0
    out = np.zeros((ns.value, 3, na.value), np.float32)
    rc = L.ref_dcd_frames(str(path).encode(), ctypes.byref(na), ctypes.byref(ns),
                          out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, rc
    return out


def ref_pdb_atoms(path, cap: int = 200000):
    """(mass, residue id, hash, tags, elements, names) from the reference's Atom."""
    L = ref_netchem()
    mass = np.zeros(cap, np.float32)
    resid = np.zeros(cap, np.int32)
    h = np.zeros(cap, np.uint32)
    tags = ctypes.create_string_buffer(40 * cap)
    els = ctypes.create_string_buffer(4 * cap)
    names = ctypes.create_string_buffer(8 * cap)
    n = L.ref_pdb_atoms(str(path).encode(), cap, mass.ctypes.data_as(ctypes.c_void_p),
                        resid.ctypes.data_as(ctypes.c_void_p), h.ctypes.data_as(ctypes.c_void_p),
                        tags, els, names)
    n = min(n, cap)

    def strs(buf, w):
        raw = buf.raw
        return [raw[w * i:w * (i + 1)].split(b"\0")[0].decode() for i in range(n)]
    return mass[:n], resid[:n], h[:n], strs(tags, 40), strs(els, 4), strs(names, 8)
