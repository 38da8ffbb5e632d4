"""Seeded synthetic workloads with the shapes of the benchmark configurations.

* ``gaussian_pair``      -- bivariate Gaussian samples (x, y), corr rho.
* ``protein_trajectory`` -- C-alpha-like trajectory: a 3-D self-avoiding
  random walk (3.8 A steps) as mean structure, frames displaced by five
  collective modes (random orthonormal 3N vectors, amplitudes N(0, s_j),
  s = 2, 1.5, 1, 0.7, 0.5 A) plus isotropic N(0, 0.5 A) noise. Returned as
  an (N, 3m) float32 matrix, plane-major per node row (the layout netchem
  produces for netcalc).
* ``uneven_batch``       -- many trajectories of the same generator with
  N and m drawn uniformly from ranges.
* ``random_geometric_graph`` -- unit-cube RGG with a target mean degree and
  integer or float weights; +inf off-edge, 0 diagonal.
* ``contact_graph``      -- edges where the mean C-alpha distance < cutoff,
  weighted by -ln(GC) (+inf where GC == 0).
"""
from __future__ import annotations

import numpy as np

MODE_SIGMAS = (2.0, 1.5, 1.0, 0.7, 0.5)


def gaussian_pair(n: int, rho: float, seed: int) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((2, n))
    x = z[0]
    y = rho * z[0] + np.sqrt(max(0.0, 1.0 - rho * rho)) * z[1]
    return x.astype(np.float32), y.astype(np.float32)


def self_avoiding_walk(N: int, rng: np.random.Generator, step: float = 3.8,
                       min_sep: float = 3.0, tries: int = 64) -> np.ndarray:
    pos = np.zeros((N, 3))
    for i in range(1, N):
        for _ in range(tries):
            v = rng.standard_normal(3)
            v *= step / np.linalg.norm(v)
            cand = pos[i - 1] + v
            if i < 2 or np.min(np.linalg.norm(pos[: i - 1] - cand, axis=1)) >= min_sep:
                break
        pos[i] = cand
    return pos


def protein_trajectory(N: int, m: int, seed: int, noise: float = 0.5,
                       sigmas=MODE_SIGMAS) -> tuple[np.ndarray, np.ndarray]:
    """(X, mean): X is (N, 3m) float32 plane-major rows, mean is (N, 3)."""
    rng = np.random.default_rng(seed)
    mean = self_avoiding_walk(N, rng)
    q, _ = np.linalg.qr(rng.standard_normal((3 * N, len(sigmas))))
    amps = rng.standard_normal((m, len(sigmas))) * np.asarray(sigmas)[None, :]
    disp = (amps @ q.T).reshape(m, N, 3)
    disp += rng.standard_normal((m, N, 3)) * noise
    coords = disp + mean[None, :, :]                      # (m, N, 3)
    X = np.ascontiguousarray(coords.transpose(1, 2, 0)).reshape(N, 3 * m)
    return X.astype(np.float32), mean


def uneven_batch(T: int, n_range=(50, 500), m_range=(500, 5000), seed: int = 0):
    """List of (X, mean) trajectories with N, m uniform in the ranges."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(T):
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        m = int(rng.integers(m_range[0], m_range[1] + 1))
        out.append(protein_trajectory(N, m, seed=int(rng.integers(1 << 31))))
    return out


def random_geometric_graph(N: int, mean_degree: float, seed: int, integer_weights: bool = True,
                           wmax: int = 100) -> np.ndarray:
    rng = np.random.default_rng(seed)
    pts = rng.random((N, 3))
    # expected degree ~ (N-1) * (4/3) pi r^3 in the unit cube (edge effects ignored)
    r = (mean_degree / (max(N - 1, 1) * 4.0 / 3.0 * np.pi)) ** (1.0 / 3.0)
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    adj = d2 < r * r
    np.fill_diagonal(adj, False)
    if integer_weights:
        w = rng.integers(1, wmax + 1, size=(N, N)).astype(np.float32)
    else:
        w = (rng.random((N, N)) * (wmax - 1) + 1).astype(np.float32)
    w = np.triu(w, 1)
    w = w + w.T
    A = np.where(adj, w, np.float32(np.inf)).astype(np.float32)
    np.fill_diagonal(A, 0.0)
    return A


def all_pairs(N: int) -> np.ndarray:
    """(P, 2) int32 node pairs a < b, row-major in a."""
    a, b = np.triu_indices(N, 1)
    return np.stack([a, b], axis=1).astype(np.int32)


def contact_graph(mean: np.ndarray, gc_pairs: np.ndarray, ab: np.ndarray,
                  cutoff: float = 8.0) -> np.ndarray:
    """N x N weights -ln(GC) on contacts (mean distance < cutoff), +inf
    elsewhere, 0 on the diagonal; the transform is evaluated in double and
    rounded to float."""
    N = mean.shape[0]
    A = np.full((N, N), np.float32(np.inf), dtype=np.float32)
    dist = np.linalg.norm(mean[:, None, :] - mean[None, :, :], axis=-1)
    ab = np.asarray(ab, dtype=np.int64).reshape(-1, 2)
    g = np.asarray(gc_pairs, dtype=np.float32)
    a, b = ab[:, 0], ab[:, 1]
    keep = (dist[a, b] < cutoff) & (g > 0)
    w = (-np.log(g[keep].astype(np.float64))).astype(np.float32)
    A[a[keep], b[keep]] = w
    A[b[keep], a[keep]] = w
    np.fill_diagonal(A, 0.0)
    return A


# ---------------------------------------------------------------------------
# Synthetic structure files: PDB topology + DCD trajectory
# ---------------------------------------------------------------------------
_RESIDUES = {  # residue name -> atom (name, element) list
    "GLY": [("N", "N"), ("CA", "C"), ("C", "C"), ("O", "O")],
    "ALA": [("N", "N"), ("CA", "C"), ("C", "C"), ("O", "O"), ("CB", "C")],
    "SER": [("N", "N"), ("CA", "C"), ("C", "C"), ("O", "O"), ("CB", "C"), ("OG", "O")],
    "CYS": [("N", "N"), ("CA", "C"), ("C", "C"), ("O", "O"), ("CB", "C"), ("SG", "S")],
    "MET": [("N", "N"), ("H", "H"), ("CA", "C"), ("HA", "H"), ("C", "C"), ("O", "O"),
            ("CB", "C"), ("CG", "C"), ("SD", "S"), ("CE", "C")],
}


def write_pdb(path, atoms) -> None:
    """ATOM records in fixed PDB columns. atoms: dicts with name, resname,
    chain, resid, x, y, z, occupancy, segment, element."""
    with open(path, "w") as f:
        f.write("CRYST1   50.000   50.000   50.000  90.00  90.00  90.00 P 1           1\n")
        for i, a in enumerate(atoms):
            f.write(f"ATOM  {(i + 1) % 100000:5d} {a['name']:<4s} {a['resname']:>3s} {a['chain']:1s}"
                    f"{a['resid']:4d}    {a['x']:8.3f}{a['y']:8.3f}{a['z']:8.3f}"
                    f"{a['occupancy']:6.2f}{0.0:6.2f}      {a['segment']:<4s}{a['element']:>2s}\n")
        f.write("END\n")


def write_dcd(path, frames: np.ndarray, charmm: bool = True, unit_cell: bool = True,
              big_endian: bool = False, marker_bytes: int = 4, four_dims: bool = False) -> None:
    """A DCD file of frames float32 [nsets, 3, natoms]."""
    import struct
    frames = np.asarray(frames, np.float32)
    nsets, _, natoms = frames.shape
    bo = ">" if big_endian else "<"
    mk = bo + ("i" if marker_bytes == 4 else "q")

    def rec(payload: bytes) -> bytes:
        m = struct.pack(mk, len(payload))
        return m + payload + m
    words = [0] * 20
    words[0], words[1], words[2], words[3] = nsets, 0, 1, nsets
    if charmm:
        words[10] = 1 if unit_cell else 0
        words[11] = 1 if four_dims else 0
        words[19] = 24
    head = bytearray(b"CORD" + struct.pack(bo + "20i", *words))
    if charmm:
        head[4 + 36:4 + 40] = struct.pack(bo + "f", 1.0)
    else:
        head[4 + 36:4 + 44] = struct.pack(bo + "d", 1.0)
    out = [rec(bytes(head)),
           rec(struct.pack(bo + "i", 2) + b"synthetic trajectory".ljust(80) + b"netsci_gb300".ljust(80)),
           rec(struct.pack(bo + "i", natoms))]
    dt = np.dtype(np.float32).newbyteorder(bo)
    for f in range(nsets):
        if charmm and unit_cell:
            out.append(rec(struct.pack(bo + "6d", 50.0, 90.0, 50.0, 90.0, 90.0, 50.0)))
        for c in range(3):
            out.append(rec(frames[f, c].astype(dt).tobytes()))
        if charmm and four_dims:
            out.append(rec(np.zeros(natoms, dt).tobytes()))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def protein_files(directory, n_residues: int, n_frames: int, seed: int, **dcd_kw):
    """A synthetic protein (residues of 4-10 atoms of H, C, N, O, S, two
    chains, one segment per chain) moving along a random walk with thermal
    noise; writes <directory>/synthetic.pdb and .dcd and returns their
    paths and the frames [n_frames, 3, natoms]."""
    from pathlib import Path
    rng = np.random.default_rng(seed)
    names = list(_RESIDUES)
    centres = self_avoiding_walk(n_residues, rng)
    atoms, base = [], []
    for r in range(n_residues):
        rn = names[int(rng.integers(len(names)))]
        chain = "A" if r < n_residues // 2 else "B"
        for name, el in _RESIDUES[rn]:
            p = centres[r] + rng.normal(0.0, 1.2, 3)
            atoms.append(dict(name=name, resname=rn, chain=chain, resid=r % 9999 + 1, x=p[0],
                              y=p[1], z=p[2], occupancy=1.0, segment="P" + chain, element=el))
            base.append(p)
    base = np.asarray(base, np.float32)
    modes = rng.normal(0.0, 1.0, (3, len(atoms), 3)).astype(np.float32)
    amp = rng.normal(0.0, 1.0, (n_frames, 3)).astype(np.float32)
    xyz = base[None] + np.einsum("fk,kac->fac", amp, modes) \
        + rng.normal(0.0, 0.3, (n_frames, len(atoms), 3)).astype(np.float32)
    frames = np.ascontiguousarray(xyz.transpose(0, 2, 1)).astype(np.float32)
    d = Path(directory)
    pdb, dcd = d / "synthetic.pdb", d / "synthetic.dcd"
    write_pdb(pdb, atoms)
    write_dcd(dcd, frames, **dcd_kw)
    return str(dcd), str(pdb), frames
