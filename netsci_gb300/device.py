"""Device-resident entry points over torch CUDA tensors.

Thin wrappers of the C ABI's device-pointer calls (section 3 of
include/netsci_gb300.h). Tensors are plumbing only (allocation, streams);
all arithmetic runs in the library's CUDA kernels.

Trajectory layout on the device: a float32 tensor of shape (N, d, ld) with
ld >= m; node a's coordinate plane c holds its m samples in
``X[a, c, :m]`` (the reference's plane-major rows, with a plane stride).
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _lib
from ._lib import KsgPair, call, lib


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(stream: torch.cuda.Stream | None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def pack_trajectory(x: np.ndarray | torch.Tensor, d: int, ld_multiple: int = 64,
                    device: str | torch.device = "cuda") -> tuple[torch.Tensor, int]:
    """Device copy of an (N, d*m) plane-major matrix as (N, d, ld), ld a
    multiple of ``ld_multiple`` (padding = +inf, never read as a sample)."""
    xt = torch.as_tensor(x, dtype=torch.float32)
    N, dm = xt.shape
    m = dm // d
    ld = (m + ld_multiple - 1) // ld_multiple * ld_multiple
    out = torch.full((N, d, ld), float("inf"), dtype=torch.float32, device=device)
    out[:, :, :m] = xt.reshape(N, d, m).to(device)
    return out, m


def make_pairs(X: torch.Tensor, m: int, ab: np.ndarray | Sequence[Sequence[int]],
               fmap: torch.Tensor | None = None, m_samples: int | None = None) -> list[KsgPair]:
    """nsg_ksg_pair descriptors for rows (a, b) of a packed trajectory."""
    assert X.is_cuda and X.dtype == torch.float32 and X.dim() == 3 and X.is_contiguous()
    N, d, ld = X.shape
    base = X.data_ptr()
    row = d * ld * 4
    fm = 0 if fmap is None else fmap.data_ptr()
    ms = m if m_samples is None else m_samples
    ab = np.asarray(ab, dtype=np.int64).reshape(-1, 2)
    if ab.size and (ab.min() < 0 or ab.max() >= N):
        raise ValueError("pair index outside the trajectory")
    return [KsgPair(base + int(a) * row, base + int(b) * row, fm or None, ld, ms) for a, b in ab]


def _pair_array(pairs: Sequence[KsgPair]):
    arr = (KsgPair * len(pairs))(*pairs)
    return arr


def ksg_pairs(pairs: Sequence[KsgPair], k: int, d: int, mi: torch.Tensor | None = None,
              gc: torch.Tensor | None = None, w: torch.Tensor | None = None,
              stream: torch.cuda.Stream | None = None) -> None:
    """All pairs in one persistent launch (+ finalize); synchronizes the stream."""
    arr = _pair_array(pairs)
    call("nsg_ksg_pairs_device", arr, len(pairs), int(k), int(d), _ptr(mi), _ptr(gc), _ptr(w),
         _stream(stream))


def ksg_pair_detail(xa: torch.Tensor, xb: torch.Tensor, m: int, k: int, d: int,
                    stream: torch.cuda.Stream | None = None) -> dict:
    """One pair with per-sample outputs. xa, xb: (d, ld) device tensors."""
    assert xa.shape == xb.shape and xa.dim() == 2 and xa.is_contiguous() and xb.is_contiguous()
    ld = xa.shape[1]
    dev = xa.device
    out = dict(
        n_x=torch.empty(m, dtype=torch.int32, device=dev),
        n_y=torch.empty(m, dtype=torch.int32, device=dev),
        eps_x=torch.empty(m, dtype=torch.float32, device=dev),
        eps_y=torch.empty(m, dtype=torch.float32, device=dev),
        kdist=torch.empty(m, dtype=torch.float32, device=dev),
        mi=torch.empty(1, dtype=torch.float32, device=dev),
    )
    call("nsg_ksg_pair_detail_device", xa.data_ptr(), xb.data_ptr(), ld, int(m), int(k), int(d),
         out["n_x"].data_ptr(), out["n_y"].data_ptr(), out["eps_x"].data_ptr(),
         out["eps_y"].data_ptr(), out["kdist"].data_ptr(), out["mi"].data_ptr(), _stream(stream))
    return out


class KsgPlan:
    """Reusable all-pairs plan (nsg_ksg_plan_*): descriptors, work queue and
    scratch built once; ``run`` replays one captured CUDA graph."""

    def __init__(self, pairs: Sequence[KsgPair], k: int, d: int, mi: torch.Tensor | None = None,
                 gc: torch.Tensor | None = None, w: torch.Tensor | None = None,
                 graph: bool = True, timing: bool = False, autotune: bool = False):
        self._keep = (mi, gc, w)
        arr = _pair_array(pairs)
        h = ctypes.c_void_p()
        flags = (1 if graph else 0) | (2 if timing else 0) | (4 if autotune else 0)
        call("nsg_ksg_plan_create", arr, len(pairs), int(k), int(d), _ptr(mi), _ptr(gc), _ptr(w),
             flags, ctypes.byref(h))
        self._h = h

    def run(self, stream: torch.cuda.Stream | None = None) -> None:
        call("nsg_ksg_plan_run", self._h, _stream(stream))

    def prepare(self) -> None:
        """Capture the CUDA graph now, so that the first run does not."""
        call("nsg_ksg_plan_prepare", self._h)

    def check(self) -> None:
        """Raise NsgError when a run recorded a device fault."""
        call("nsg_ksg_plan_check", self._h)

    @property
    def launches(self) -> int:
        v = ctypes.c_int()
        call("nsg_ksg_plan_launches", self._h, ctypes.byref(v))
        return v.value

    @property
    def shape(self) -> dict:
        v = [ctypes.c_int() for _ in range(6)]
        call("nsg_ksg_plan_shape", self._h, *(ctypes.byref(x) for x in v[:4]))
        call("nsg_ksg_plan_staging", self._h, ctypes.byref(v[4]))
        call("nsg_ksg_plan_search", self._h, ctypes.byref(v[5]))
        return dict(threads=v[0].value, r=v[1].value, frames=v[2].value, variant=v[3].value,
                    staging="bulk-copy" if v[4].value else "loads",
                    search="cell-grid" if v[5].value else "exhaustive")

    def evaluations(self) -> tuple[int, int, int]:
        """(joint distances, one-variable distances, eps comparisons) of the
        last run's cell-grid search and counts; zeros for exhaustive plans.
        A count kernel's distance is evaluated once per query and frame and
        compared with the eps of every pair of its count group."""
        a, b, c = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_ulonglong()
        call("nsg_ksg_plan_evaluations", self._h, ctypes.byref(a), ctypes.byref(b),
             ctypes.byref(c))
        return a.value, b.value, c.value

    def tied_samples(self) -> int:
        """Samples of the last run that went to the tie kernel."""
        v = ctypes.c_longlong()
        call("nsg_ksg_plan_tied_samples", self._h, ctypes.byref(v))
        return v.value

    def kernel_ms(self) -> tuple[float, float, float]:
        """Device ms of the last run's (search, count, tie) kernels, order
        kernels excluded; plans need timing=True."""
        a, b, c = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        call("nsg_ksg_plan_kernel_ms", self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return float(a.value), float(b.value), float(c.value)

    def count_ms(self) -> float:
        """Device time (ms) of the count kernels in the last run."""
        v = ctypes.c_float()
        call("nsg_ksg_plan_count_ms", self._h, ctypes.byref(v))
        return float(v.value)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().nsg_ksg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def release_cached_memory() -> None:
    """Return the device memory the library keeps for reuse to the driver."""
    call("nsg_release_cached_memory")


def set_ksg_shape(threads: int = 0, r: int = 0, frames: int = 0, variant: int = -1) -> None:
    """Force a KSG tile shape for later plans (threads=0: automatic)."""
    call("nsg_ksg_set_shape", int(threads), int(r), int(frames), int(variant))


def set_ksg_staging(staging: int = -1) -> None:
    """Tile staging for later plans: 1 bulk copies (TMA), 0 plain loads, -1 auto."""
    call("nsg_ksg_set_staging", int(staging))


def set_ksg_search(mode: int = -1) -> None:
    """Neighbour search for later plans: 1 cell grids, 0 exhaustive, -1 automatic."""
    call("nsg_ksg_set_search", int(mode))


def set_ksg_orders(mode: int = -1) -> None:
    """Block query orders of later cell-grid plans: 1 always, 0 never, -1 automatic."""
    call("nsg_ksg_set_orders", int(mode))


def issue_ceiling(d: int = 3) -> tuple[float, float]:
    """Measured operation rates (Gop/s) of the cell-grid search and count
    kernels' inner loops alone: the ceilings their rates are divided by."""
    a, b = ctypes.c_double(), ctypes.c_double()
    call("nsg_measure_issue_ceiling", int(d), ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def set_apsp_method(method: int = -1) -> None:
    """Shortest-path products for later solves: -1 automatic (squaring where
    bit-exact), 0 Jacobi steps only, 1 squaring on any weights."""
    call("nsg_apsp_set_method", int(method))


def apsp_lengths(A: torch.Tensor, max_path_length: int, H: torch.Tensor | None = None,
                 stream: torch.cuda.Stream | None = None) -> tuple[torch.Tensor, int]:
    n = A.shape[0]
    assert A.shape == (n, n) and A.is_cuda and A.dtype == torch.float32 and A.is_contiguous()
    H = torch.empty_like(A) if H is None else H
    steps = ctypes.c_int()
    call("nsg_apsp_lengths_device", A.data_ptr(), H.data_ptr(), n, int(max_path_length),
         ctypes.byref(steps), _stream(stream))
    return H, steps.value


def apsp_paths(A: torch.Tensor, max_path_length: int, tolerance: float,
               stream: torch.cuda.Stream | None = None) -> tuple[torch.Tensor, torch.Tensor]:
    n = A.shape[0]
    H = torch.empty_like(A)
    P = torch.empty(n * max_path_length * n, dtype=torch.int32, device=A.device)
    call("nsg_apsp_paths_device", A.data_ptr(), H.data_ptr(), P.data_ptr(), n,
         int(max_path_length), float(tolerance), _stream(stream))
    return H, P


def corr_to_adjacency(C: torch.Tensor, mode: int = 0,
                      stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    n = C.shape[0]
    A = torch.empty_like(C)
    call("nsg_corr_to_adjacency_device", C.data_ptr(), A.data_ptr(), n, int(mode),
         _stream(stream))
    return A
