"""Generate the committed golden fixtures in tests/golden/.

Run in a checkout that has the reference sources (the copy that
``make -C oracle stage`` leaves in baseline/_ref/netsci, or NETSCI_REF); it
builds oracle/_ref from them and records the
reference CPU functions' outputs on fixed inputs:

* gaussian.npz -- the reference's own bivariate-Gaussian test data
  (tests/data/2X_1D_{1000,2000}_4.npy, float64 cast to float32) with the
  MI the reference tests pin (tests/netcalc/python/test_MutualInformation.py
  :37, :64), checked here against the reference library, plus per-sample
  n_x/n_y/eps from the CPU restatement.
* curves.npz   -- the deterministic sin/cos/x/log curves of the reference's
  C++ and Python tests (tests/netcalc/cpp/MutualInformation_test.cpp:99-303,
  tests/netcalc/python/test_GeneralizedCorrelation.py:12-226) for d = 1, 2, 3
  and n = 1000, 2000, k = 4, with reference MI and GC.
* random.npz   -- seeded random pairs over d, k and n (edge sizes included)
  with reference MI.
* protein56.npz -- the 56-node, 1000-frame synthetic trajectory, reference
  GC of all 1540 pairs, and the CPU-restatement shortest-path lengths of its
  -ln(GC) contact graph.

Inputs are stored, not regenerated, so the GPU host needs nothing but these
files.
"""
from __future__ import annotations

import os
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from netsci_gb300 import synthetic  # noqa: E402

REF = oracle.ref_root()
GOLDEN_MI = {1000: 0.8449974060058594, 2000: 0.8485465049743652}


def curves(n: int, d: int):
    """The reference tests' curve inputs: float domain stepping by pi/n from
    0.001 (MutualInformation_test.cpp:215-230), Xa/Xb as in the d-th case."""
    incr = np.float32(np.pi / np.float32(n))
    dom = np.zeros(n, np.float32)
    dom[0] = np.float32(0.001)
    for i in range(1, n):
        dom[i] = np.float32(dom[i - 1] + incr)
    f64 = dom.astype(np.float64)
    s, c, lg = np.sin(f64), np.cos(f64), np.log(f64)
    if d == 1:
        xa, xb = [s], [c]
    elif d == 2:
        xa, xb = [s, c], [f64, 2 * f64]
    else:
        xa, xb = [s, c, lg], [c, 2 * f64, np.log(f64 * 2.0)]
    return (np.concatenate(xa).astype(np.float32), np.concatenate(xb).astype(np.float32))


def main() -> None:
    oracle.build(ref=True)
    R = oracle.ref_lib()
    assert R is not None, "reference library did not build"

    # ---- gaussian -----------------------------------------------------------
    g = {}
    for n in (1000, 2000):
        X = np.load(REF / "tests" / "data" / f"2X_1D_{n}_4.npy").astype(np.float32)
        x, y = np.ascontiguousarray(X[:n]), np.ascontiguousarray(X[n:])
        ref = R.ref_mi_cpu(x, y, n, 4, 1)
        assert ref == GOLDEN_MI[n], (n, ref)
        mi, det = oracle.mi_pair(x, y, n, 4, 1, detail=True)
        assert mi == ref
        g[f"x{n}"], g[f"y{n}"] = x, y
        g[f"mi{n}"] = np.float32(ref)
        for key in ("n_x", "n_y", "eps_x", "eps_y", "kdist"):
            g[f"{key}{n}"] = det[key]
    np.savez_compressed(HERE / "gaussian.npz", **g)

    # ---- curves ---------------------------------------------------------------
    c = {}
    for d in (1, 2, 3):
        for n in (1000, 2000):
            xa, xb = curves(n, d)
            c[f"xa_d{d}_n{n}"], c[f"xb_d{d}_n{n}"] = xa, xb
            c[f"mi_d{d}_n{n}"] = np.float32(R.ref_mi_cpu(xa, xb, n, 4, d))
            c[f"gc_d{d}_n{n}"] = np.float32(R.ref_gc_cpu(xa, xb, n, 4, d))
            assert oracle.mi_pair(xa, xb, n, 4, d) == c[f"mi_d{d}_n{n}"]
    np.savez_compressed(HERE / "curves.npz", **c)

    # ---- random -----------------------------------------------------------------
    rng = np.random.default_rng(20261203)
    cases = []
    for d in (1, 2, 3):
        for k, n in ((1, 50), (3, 257), (6, 1000), (8, 513), (12, 700), (16, 300), (32, 400),
                     (4, 33), (7, 129)):
            z = rng.standard_normal((n, 2 * d)).astype(np.float32)
            rho = rng.uniform(0.0, 0.95)
            a = z[:, :d]
            b = rho * z[:, :d] + np.sqrt(1 - rho * rho) * z[:, d:]
            xa = np.ascontiguousarray(a.T.astype(np.float32)).ravel()
            xb = np.ascontiguousarray(b.T.astype(np.float32)).ravel()
            cases.append((d, k, n, xa, xb))
    r = {"count": np.int32(len(cases))}
    for i, (d, k, n, xa, xb) in enumerate(cases):
        r[f"meta{i}"] = np.array([d, k, n], np.int32)
        r[f"xa{i}"], r[f"xb{i}"] = xa, xb
        ref = R.ref_mi_cpu(xa, xb, n, k, d)
        mi, det = oracle.mi_pair(xa, xb, n, k, d, detail=True)
        assert mi == ref, (i, d, k, n, mi, ref)
        r[f"mi{i}"] = np.float32(ref)
        r[f"ties{i}"] = np.int32(det["ties"])
    np.savez_compressed(HERE / "random.npz", **r)

    # ---- protein56 (N=56, m=1000, d=3, k=6) ---------------------------------------
    N, m, k = 56, 1000, 6
    X, mean = synthetic.protein_trajectory(N, m, seed=56)
    ab = synthetic.all_pairs(N)

    def one(p):
        a, b = ab[p]
        return R.ref_gc_cpu(np.ascontiguousarray(X[a]), np.ascontiguousarray(X[b]), m, k, 3)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        gc = np.array(list(ex.map(one, range(len(ab)))), np.float32)
    A = synthetic.contact_graph(mean, gc, ab, cutoff=8.0)
    H, steps, conv = oracle.apsp_lengths(A, N)
    assert conv
    np.savez_compressed(HERE / "protein56.npz", X=X, mean=mean.astype(np.float32), ab=ab, gc=gc,
                        A=A, H=H, steps=np.int32(steps), k=np.int32(k))
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
