"""The drop-in boundary from compiled hosts: a plain-C program over the C
ABI and a C++ program over the reference-signature headers, compiled with
gcc / g++ against include/ and linked to the library; CPU platform results
equal the oracle's, and the GPU platform fails with a status (no fallback)
when no device is present."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "netsci_gb300"


def _input(tmp_path, N=4, n=600, k=4, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((N, n)).astype(np.float32)
    x[1] = (0.7 * x[0] + 0.5 * x[1]).astype(np.float32)
    p = tmp_path / "in.bin"
    with open(p, "wb") as f:
        f.write(np.array([N, n, k], np.int32).tobytes())
        f.write(x.tobytes())
    return p, x, n, k


def _build(tmp_path, src, exe, cxx):
    cmd = ["g++" if cxx else "gcc", str(ROOT / "tests" / "native" / src), "-O1",
           "-I", str(ROOT / "include"), "-L", str(LIBDIR), "-lnetsci_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(tmp_path / exe)]
    if cxx:
        cmd[2:2] = ["-std=c++17"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return tmp_path / exe


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_program_over_the_c_abi(tmp_path, nsg_lib, oracle_mod):
    inp, x, n, k = _input(tmp_path)
    exe = _build(tmp_path, "cabi_host_demo.c", "cdemo", cxx=False)
    out = subprocess.run([str(exe), str(inp), str(tmp_path / "I.npy")], capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    mis = [l.split() for l in lines if l.startswith("mi ")]
    assert len(mis) == 6
    for _, a, b, v in mis:
        want = oracle_mod.mi_pair(x[int(a)], x[int(b)], n, k, 1)
        assert np.float32(float(v)) == np.float32(want)
    psi = [l for l in lines if l.startswith("psi ")][0].split()[1]
    assert np.float32(float(psi)) == oracle_mod.psi(n)[n]
    gpu = int([l for l in lines if l.startswith("gpu_status ")][0].split()[1])
    assert (gpu == 0) == _gpu_present()
    assert np.load(tmp_path / "I.npy").shape == (1, 6)


def test_cpp_program_over_the_reference_headers(tmp_path, nsg_lib, oracle_mod):
    inp, x, n, k = _input(tmp_path)
    exe = _build(tmp_path, "cxx_api_demo.cpp", "cxxdemo", cxx=True)
    out = subprocess.run([str(exe), str(inp)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr + out.stdout
    first = out.stdout.split("\n")[0].split()
    mi, gc = float(first[1]), float(first[3])
    assert np.float32(mi) == np.float32(oracle_mod.mi_pair(x[0], x[1], n, k, 1))
    assert np.float32(gc) == np.float32(oracle_mod.gc_from_mi(np.float32(mi), 1))
    assert first[5:7] == ["1", "1"]
    assert "invalid platform throws" in out.stdout
