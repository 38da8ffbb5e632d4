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
    for (a, b), g in zip(ab, gc_pairs):
        if dist[a, b] < cutoff and g > 0:
            w = np.float32(-np.log(np.float64(g)))
            A[a, b] = w
            A[b, a] = w
    np.fill_diagonal(A, 0.0)
    return A
