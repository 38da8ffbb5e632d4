"""Tie resolution on inputs built to stress it, against the oracle (the
reference CPU path's std::sort order, netcalc/src/mutual_information_cpu.cpp:
48-77), per sample and bit for bit, on both searches:

* tie-saturated pairs: coordinates on a coarse grid, where nearly every
  sample ties at the k-th distance between frames with different marginals,
  so nearly every sample goes to the tie list (the list holds every sample of
  a batch and cannot overflow), for k up to 62 (the replayed eps then spans
  more sorted positions than a warp has lanes);
* a sample whose distance row defeats the median-of-three pivots, so that
  the reference's introsort runs out of depth budget and heapsorts the
  segment holding the neighbours, with a tie at the k-th distance (keys made
  by tests/native/sort_prefix_check.cpp's adversary mode).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
KEYS = ("n_x", "n_y", "eps_x", "eps_y", "kdist")


@pytest.fixture(scope="module")
def adversary(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path_factory.mktemp("adv") / "sort_prefix_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "netsci_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "sort_prefix_check.cpp"), "-o", str(exe)],
                   check=True)

    def keys(n, k):
        out = subprocess.run([str(exe), "adversary", str(n), str(k)], capture_output=True,
                             text=True, check=True).stdout.split()
        return int(out[0]), np.array([int(v) for v in out[1:]], np.int64)
    return keys


@pytest.fixture
def search():
    from netsci_gb300 import device
    yield device.set_ksg_search
    device.set_ksg_search(-1)


def _detail(xa, xb, n, k, d):
    from netsci_gb300 import device
    X, m = device.pack_trajectory(np.stack([xa, xb]).reshape(2, d * n), d)
    return device.ksg_pair_detail(X[0], X[1], m, k, d)


def _same(out, det, mi):
    for key in KEYS:
        got = out[key].cpu().numpy()
        bad = np.flatnonzero(got != det[key])
        assert bad.size == 0, (key, bad[:5])
    assert float(out["mi"].item()) == mi


@pytest.mark.parametrize("d,k,n,levels", [(1, 4, 6000, 64), (2, 6, 5000, 32), (3, 6, 4000, 32),
                                          (3, 10, 2500, 32), (2, 40, 3000, 32), (1, 45, 4000, 64),
                                          (3, 62, 2600, 16)])
def test_tie_saturated_pair(oracle_mod, search, d, k, n, levels):
    rng = np.random.default_rng(n + levels)
    xa = rng.integers(0, levels, d * n).astype(np.float32)
    xb = rng.integers(0, levels, d * n).astype(np.float32)
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, d, detail=True, threads=8)
    assert det["ties"] > n // 2   # more than half the samples tie with mixed marginals
    for s in (0, 1):
        search(s)
        _same(_detail(xa, xb, n, k, d), det, mi)


@pytest.mark.parametrize("n,k", [(4000, 6), (2500, 4)])
def test_heapsorted_neighbour_segment(oracle_mod, adversary, search, n, k):
    heaps, key = adversary(n, k)
    assert heaps >= 1   # the reference's sort heapsorts the neighbours' segment
    q = int(np.flatnonzero(key == 0)[0])
    xa = np.zeros(n, np.float32)
    xb = np.zeros(n, np.float32)
    odd = (np.arange(n) % 2) == 1
    xa[~odd] = key[~odd]
    xb[odd] = key[odd]
    # the two frames at the tied k-th distance differ in their marginals
    tied = np.flatnonzero(key == k)
    assert tied.size == 2
    xa[tied[0]], xb[tied[0]] = k, 0
    xa[tied[1]], xb[tied[1]] = 0, k
    mi, det = oracle_mod.mi_pair(xa, xb, n, k, 1, detail=True, threads=8)
    assert det["kdist"][q] == k
    for s in (0, 1):
        search(s)
        _same(_detail(xa, xb, n, k, 1), det, mi)
