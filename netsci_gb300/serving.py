"""Serving: continuous batching of MI / GC / APSP jobs (nsg_server_*).

``Server`` wraps the C++ request loop (include/netsci_gb300.h, section 4).
``c5_trace`` draws the mixed-request stream of the serving configuration
(Poisson arrivals; 60% all-pairs GC on trajectories with N log-uniform in
[20, 1000] and m uniform in [500, 5000]; 25% bivariate-Gaussian MI with n
uniform in [1000, 20000]; 15% APSP on random geometric graphs with N uniform
in [100, 2000]). ``run_served`` replays a trace against a Server with the
arrival times honoured; ``run_plain`` runs the same requests one at a time in
arrival order through the plain per-request entry points, the comparison
point for the batching.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np

from . import synthetic
from ._lib import call

STATE_NAMES = {0: "pending", 1: "running", 2: "done", 3: "failed"}


@dataclass
class Job:
    id: int
    kind: str
    out: np.ndarray
    keep: tuple = ()          # host inputs that must outlive the job


class Server:
    def __init__(self, budget_bytes: int = 16 << 30, tick_ops: float = 2.5e11,
                 max_m: int = 32768):
        h = ctypes.c_void_p()
        call("nsg_server_create", ctypes.c_size_t(budget_bytes), float(tick_ops), int(max_m),
             ctypes.byref(h))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            call("nsg_server_destroy", self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def register_trajectory(self, X: np.ndarray, d: int) -> int:
        X = np.ascontiguousarray(X, dtype=np.float32)
        N, dm = X.shape
        t = ctypes.c_int()
        call("nsg_server_register_trajectory", self._h, X.ctypes.data_as(ctypes.c_void_p), N,
             dm // d, d, ctypes.byref(t))
        return t.value

    def submit_gc(self, traj: int, N: int, k: int) -> Job:
        out = np.empty(N * (N - 1) // 2, np.float32)
        j = ctypes.c_longlong()
        call("nsg_server_submit_gc", self._h, int(traj), int(k),
             out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(j))
        return Job(j.value, "gc", out)

    def submit_mi(self, x: np.ndarray, y: np.ndarray, d: int, k: int) -> Job:
        x = np.ascontiguousarray(x, np.float32).ravel()
        y = np.ascontiguousarray(y, np.float32).ravel()
        out = np.empty(1, np.float32)
        j = ctypes.c_longlong()
        call("nsg_server_submit_mi", self._h, x.ctypes.data_as(ctypes.c_void_p),
             y.ctypes.data_as(ctypes.c_void_p), x.size // d, int(d), int(k),
             out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(j))
        return Job(j.value, "mi", out, (x, y))

    def submit_apsp(self, A: np.ndarray, max_path_length: int) -> Job:
        A = np.ascontiguousarray(A, np.float32)
        out = np.empty_like(A)
        j = ctypes.c_longlong()
        call("nsg_server_submit_apsp", self._h, A.ctypes.data_as(ctypes.c_void_p), A.shape[0],
             int(max_path_length), out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(j))
        return Job(j.value, "apsp", out, (A,))

    def wait(self, job: Job, timeout: float = 600.0) -> np.ndarray:
        st = ctypes.c_int()
        call("nsg_server_wait", self._h, ctypes.c_longlong(job.id), float(timeout),
             ctypes.byref(st))
        if st.value != 2:
            raise TimeoutError(f"job {job.id} is {STATE_NAMES.get(st.value)}")
        return job.out

    def info(self, job: Job) -> dict:
        st = ctypes.c_int()
        t = [ctypes.c_double() for _ in range(3)]
        call("nsg_server_job_info", self._h, ctypes.c_longlong(job.id), ctypes.byref(st),
             *(ctypes.byref(x) for x in t))
        return dict(state=st.value, submit=t[0].value, admit=t[1].value, done=t[2].value)

    def stats(self) -> dict:
        a, b, c = (ctypes.c_longlong() for _ in range(3))
        p = ctypes.c_size_t()
        call("nsg_server_stats", self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
             ctypes.byref(p))
        return dict(jobs_done=a.value, pairs_done=b.value, ticks=c.value, peak_bytes=p.value)


# ---------------------------------------------------------------------------
# C5 trace
# ---------------------------------------------------------------------------
@dataclass
class Request:
    t: float                  # arrival time (s from trace start)
    kind: str                 # "gc" | "mi" | "apsp"
    params: dict = field(default_factory=dict)
    data: tuple = ()


def c5_trace(n: int, seed: int = 5, rate: float = 200.0, scale: float = 1.0) -> list[Request]:
    """n requests of the serving mix. `scale` (<= 1) shrinks the GC node and
    frame ranges' upper ends for quick runs."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        u = rng.random()
        if u < 0.60:
            lo, hi = 20, max(21, int(1000 * scale))
            N = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
            m = int(rng.integers(500, max(501, int(5000 * scale)) + 1))
            X, _ = synthetic.protein_trajectory(N, m, seed=int(rng.integers(1 << 30)))
            out.append(Request(t, "gc", dict(N=N, m=m, d=3, k=6), (X,)))
        elif u < 0.85:
            n_s = int(rng.integers(1000, max(1001, int(20000 * scale)) + 1))
            rho = float(rng.uniform(0.0, 0.95))
            x, y = synthetic.gaussian_pair(n_s, rho, seed=int(rng.integers(1 << 30)))
            out.append(Request(t, "mi", dict(n=n_s, rho=rho, d=1, k=4), (x, y)))
        else:
            N = int(rng.integers(100, max(101, int(2000 * scale)) + 1))
            A = synthetic.random_geometric_graph(N, 12, seed=int(rng.integers(1 << 30)),
                                                 integer_weights=False)
            out.append(Request(t, "apsp", dict(N=N, L=N), (A,)))
    return out


def trace_ops(trace: list[Request]) -> float:
    ops = 0.0
    for r in trace:
        if r.kind == "gc":
            N, m = r.params["N"], r.params["m"]
            ops += N * (N - 1) / 2 * 8.0 * 3 * m * (m - 1)
        elif r.kind == "mi":
            n = r.params["n"]
            ops += 8.0 * n * (n - 1)
    return ops


def run_served(server: Server, trace: list[Request]) -> tuple[list, dict]:
    """Replay the trace with its arrival times; returns (results, summary)."""
    trajs = {}
    for i, r in enumerate(trace):
        if r.kind == "gc":
            trajs[i] = server.register_trajectory(r.data[0], 3)   # resident before the clock
    jobs = []
    t0 = time.perf_counter()
    for i, r in enumerate(trace):
        delay = r.t - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        if r.kind == "gc":
            jobs.append(server.submit_gc(trajs[i], r.params["N"], r.params["k"]))
        elif r.kind == "mi":
            jobs.append(server.submit_mi(r.data[0], r.data[1], 1, r.params["k"]))
        else:
            jobs.append(server.submit_apsp(r.data[0], r.params["L"]))
    results = [server.wait(j) for j in jobs]
    makespan = time.perf_counter() - t0
    lat = np.array([(lambda x: x["done"] - x["submit"])(server.info(j)) for j in jobs])
    return results, _summary(trace, lat, makespan)


def run_plain(trace: list[Request]) -> tuple[list, dict]:
    """The same requests one at a time, in arrival order, each through its
    own plain entry point (no batching across requests); a request's latency
    runs from its arrival to its completion."""
    import torch

    from . import device
    results, done_at = [], []
    t0 = time.perf_counter()
    for r in trace:
        now = time.perf_counter() - t0
        if r.t > now:
            time.sleep(r.t - now)
        if r.kind == "gc":
            X = r.data[0]
            Xd, m = device.pack_trajectory(X, 3)
            pairs = device.make_pairs(Xd, m, synthetic.all_pairs(r.params["N"]))
            gc = torch.empty(len(pairs), device="cuda")
            if pairs:
                device.ksg_pairs(pairs, r.params["k"], 3, gc=gc)
            results.append(gc.cpu().numpy())
        elif r.kind == "mi":
            x, y = r.data
            Xd, m = device.pack_trajectory(np.stack([x, y]), 1)
            pairs = device.make_pairs(Xd, m, [[0, 1]])
            mi = torch.empty(1, device="cuda")
            device.ksg_pairs(pairs, r.params["k"], 1, mi=mi)
            results.append(mi.cpu().numpy())
        else:
            A = torch.from_numpy(r.data[0]).cuda()
            H, _ = device.apsp_lengths(A, r.params["L"])
            results.append(H.cpu().numpy())
        torch.cuda.synchronize()
        done_at.append(time.perf_counter() - t0)
    makespan = time.perf_counter() - t0
    lat = np.array([d - r.t for d, r in zip(done_at, trace)])
    return results, _summary(trace, lat, makespan)


def _summary(trace, lat, makespan) -> dict:
    kinds = {}
    for k in ("gc", "mi", "apsp"):
        sel = np.array([r.kind == k for r in trace])
        if sel.any():
            kinds[k] = dict(n=int(sel.sum()), p50_ms=float(np.percentile(lat[sel], 50) * 1e3),
                            p99_ms=float(np.percentile(lat[sel], 99) * 1e3))
    return dict(requests=len(trace), makespan_s=makespan,
                requests_per_s=len(trace) / makespan,
                p50_ms=float(np.percentile(lat, 50) * 1e3),
                p99_ms=float(np.percentile(lat, 99) * 1e3), by_kind=kinds,
                gop_per_s=trace_ops(trace) / makespan / 1e9)
