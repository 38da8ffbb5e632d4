#!/usr/bin/env python
"""Benchmark of the netcalc hot path on GB300.

Workload (the large single-system configuration): all-pairs generalized
correlation of a synthetic protein trajectory with N = 2000 nodes,
m = 10000 frames, d = 3, k = 6 (1,999,000 node pairs in total). A step is
one batch of `--pairs-per-step` consecutive pairs of that all-pairs list;
the steps' batches are spread evenly over the whole list (first batch at its
start, last at its end), so the timed steps sample every part of the job.
The trajectory stays resident in HBM (X = 2000 x 3 x 10048 floats, 241 MB,
larger than the 129 MB L2, so every step streams it from HBM).

Lines reported (one JSON line from rank 0):
  value     pairs/s of the batched persistent plan (graph replay), device
            timed with CUDA events, max over ranks; inputs resident.
  e2e       pairs/s through the drop-in API (netcalc.generalizedCorrelation
            over host CuArrays): host->device upload of X and the pair list
            and device->host read of the results inside every step.
  roofline  the dominant kernel (the cell-grid search) against the CUDA-core
            issue model (SMs x 128 lanes x max SM clock) and against the
            measured rate of its own inner loop alone (mix_ceiling); the
            count kernel likewise under per_kernel. Operations are counted
            from the kernels' own evaluation counters: 4d per joint distance
            of the search; 2d-1 per one-variable distance of the counts (one
            per query and frame, shared by the pairs of a count group) plus
            one per eps comparison. algorithmic_pruning_gops is the rate an
            exhaustive search would need for the same steps, 8*d*m*(m-1)
            operations per pair: the gain of the cell grids, not a kernel
            fraction.
  parity    GC of random pairs of the timed batches through the drop-in API
            against the reference's own CPU code (compiled unmodified into
            oracle/_ref; the oracle restatement when that is absent), bit
            for bit.
  cpu_baseline  the same pairs on the reference's CPU code over all host
            cores (the timing of that comparison).
  reference_gpu the reference's own GPU code (compiled unmodified for
            sm_103a into oracle/_ref): one blocking generalizedCorrelationGpu
            call per pair on pairs of this workload and on the 56-node protein
            configuration, and its Hedetniemi kernel on the shortest-path
            graphs below.
  plain_per_call  pairs/s of one netcalc.generalizedCorrelationGpu call per
            pair of this library (the reference's call structure).
  exhaustive_search  the same steps with the exhaustive neighbour search.
  apsp      Hedetniemi shortest-path ms on N = 2000 random geometric graphs
            (mean degree 12), integer weights U[1,100] and float weights.
  c4_full   the whole all-pairs job (1,999,000 pairs) in one
            netcalc.generalizedCorrelation call, then the N = 2000 shortest
            paths on its -ln(GC) contact graph.
  uneven_batch  64 trajectories of uneven N and m in one plan vs the plain
            per-pair call, and one shortest-path solve per trajectory.
  bootstrap 100 frame resamples of a 100-node subset, all 4950 pairs of
            each, 495,000 pairs in one plan.
  serving   the mixed request stream: capacity (requests/s with all
            requests queued), then rows at 0.5x and 0.8x of that capacity
            and the stated 200 req/s (overload), continuous batching against
            one request at a time; p50/p99 latency per row.

``--impl reference`` runs only the reference's CPU code (oracle/_ref, else
the oracle port) on pairs of the same batches and prints its line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "netsci_gb300" / "dropin"))

N_NODES, M_FRAMES, DIM, K_NN = 2000, 10000, 3, 6
# DRAM bytes per pair of the search kernel at m = 10000, from an ncu capture
# of a 256-pair step of this workload (profiles/ksg_grid_kernels_N2000_m10000.md:
# 120.3 MB read + 15.8 MB written); the traffic is per pair (each pair's grid
# copies), so it scales with the pairs.
SEARCH_DRAM_BYTES_PER_PAIR = (120.3 + 15.8) * 1e6 / 256
SEED = 2000
METRIC = "GC pairs/sec (batched persistent), N=2000 nodes, m=10000 frames"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--pairs-per-step", type=int, default=8192)
    p.add_argument("--quick", action="store_true", help="small problem, for debugging")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=0, help="pairs in the CPU baseline sample")
    p.add_argument("--c3-trajectories", type=int, default=64,
                   help="uneven-batch configuration: trajectories (0 = skip)")
    p.add_argument("--bootstrap-resamples", type=int, default=100,
                   help="bootstrap: resamples of the 100-node subset (0 = skip)")
    p.add_argument("--serving-requests", type=int, default=120,
                   help="serving: requests per load row (0 = skip)")
    p.add_argument("--no-c4-full", action="store_true", help="skip the whole all-pairs job")
    p.add_argument("--no-reference-gpu", action="store_true")
    return p.parse_args()


def workload(quick: bool):
    from netsci_gb300 import synthetic
    if quick:
        N, m = 200, 2000
    else:
        N, m = N_NODES, M_FRAMES
    X, mean = synthetic.protein_trajectory(N, m, seed=SEED)
    return X, mean, N, m


def ops_per_pair(m: int, d: int = DIM) -> float:
    return 8.0 * d * m * (m - 1)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True,
                    timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 4 + i and s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# CPU legs: the reference's own CPU code (oracle/_ref), else the oracle port
# ---------------------------------------------------------------------------
def cpu_gc(X, m, ab, threads: int):
    """GC of the pairs `ab` on `threads` host threads: the reference's
    generalizedCorrelationCpu (oracle/_ref/liboracle_ref.so) when it was
    built, else the oracle restatement. Returns (values, seconds, kind)."""
    import oracle
    ref = oracle.ref_lib()
    t0 = time.perf_counter()
    if ref is not None:
        rows = [(np.ascontiguousarray(X[a]), np.ascontiguousarray(X[b])) for a, b in ab]
        with ThreadPoolExecutor(max_workers=threads) as ex:
            vals = list(ex.map(lambda r: ref.ref_gc_cpu(r[0], r[1], m, K_NN, DIM), rows))
        out, kind = np.asarray(vals, np.float32), "reference"
    else:
        out, kind = oracle.pairs(X, m, DIM, ab, K_NN, gc=True, threads=threads), "port"
    return out, time.perf_counter() - t0, kind


def timed_pair_pool(ab_all, world, S, W, B):
    """The pairs of every rank's timed batches (the pool the CPU samples
    are drawn from)."""
    from netsci_gb300 import sharding
    return np.concatenate([sharding.spread_batch(ab_all, r, world, S, s, B)
                           for r in range(world) for s in range(W, S)])


def reference_arm(args, rank: int):
    if rank != 0:
        return
    X, mean, N, m = workload(args.quick)
    from netsci_gb300 import synthetic
    ab_all = synthetic.all_pairs(N)
    threads = os.cpu_count() or 1
    per_step = args.cpu_sample or threads
    world = int(os.environ.get("WORLD_SIZE", "1"))
    S = args.warmup + args.steps
    pool = timed_pair_pool(ab_all, world, S, args.warmup, args.pairs_per_step)
    rng = np.random.default_rng(7)
    times, kind = [], "port"
    # warm-up steps: the same calls on the first 1000 frames of each pair
    # (nothing is cached between calls; they only bring the code and the
    # thread pool in), so that the timed steps dominate the run
    mw = min(m, 1000)
    Xw = np.ascontiguousarray(X.reshape(N, DIM, m)[:, :, :mw].reshape(N, DIM * mw))
    for s in range(args.warmup + args.steps):
        sel = pool[rng.choice(len(pool), size=per_step, replace=False)]
        if s < args.warmup:
            cpu_gc(Xw, mw, sel, threads)
            continue
        _, dt, kind = cpu_gc(X, m, sel, threads)
        times.append(dt)
    total = sum(times)
    value = per_step * args.steps / total
    sample = (f"{per_step} random pairs per step (one per thread) drawn from the pairs of the "
              f"batches the GPU arm times; warm-up steps on their first {mw} frames")
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "pairs/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"all-pairs GC, N={N} nodes, m={m} frames, d={DIM}, k={K_NN}",
                   "pairs_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": kind,
                         "sample": sample,
                         "code": ("netcalc::generalizedCorrelationCpu, the reference's own "
                                  "sources compiled unmodified (g++ -O3 -flto)"
                                  if kind == "reference" else "oracle restatement")},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU legs
# ---------------------------------------------------------------------------
def uneven_batch(n_traj: int, quick: bool):
    """Configuration C3: n_traj trajectories with N ~ U[50,500], m ~ U[500,5000]
    (d=3, k=6); all pairs of all of them in one persistent plan (CUDA graph,
    autotuned tile), against one netcalc.generalizedCorrelationGpu call per
    pair (the reference's call structure) on a sample; then one Hedetniemi
    solve per trajectory on its -ln(GC) contact graph."""
    import torch
    import cuarray
    import netcalc
    from netsci_gb300 import device, synthetic
    scale = 0.2 if quick else 1.0
    trajs = synthetic.uneven_batch(n_traj, n_range=(50, max(51, int(500 * scale))),
                                   m_range=(500, max(501, int(5000 * scale))), seed=64)
    keep, pairs, owners = [], [], []
    for t, (X, mean) in enumerate(trajs):
        Xd, m = device.pack_trajectory(X, DIM)
        keep.append(Xd)
        ab = synthetic.all_pairs(X.shape[0])
        pairs += device.make_pairs(Xd, m, ab)
        owners.append((len(pairs) - len(ab), len(ab)))
    P = len(pairs)
    gc = torch.empty(P, device="cuda")
    w = torch.empty(P, device="cuda")
    plan = device.KsgPlan(pairs, K_NN, DIM, gc=gc, w=w, graph=True, timing=True, autotune=True)
    plan.prepare()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    plan.run()
    ev1.record()
    torch.cuda.synchronize()
    batched_s = ev0.elapsed_time(ev1) / 1000.0
    ops = sum(8.0 * DIM * p.m * (p.m - 1) for p in pairs)
    # plain per-call sample
    rng = np.random.default_rng(3)
    sample = rng.choice(P, size=min(32, P), replace=False)
    flat = [(t, a, b) for t, (X, _) in enumerate(trajs) for a, b in synthetic.all_pairs(X.shape[0])]
    xs = []
    for i in sample:
        t, a, b = flat[i]
        X = trajs[t][0]
        xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
        xa.fromNumpy1D(X[a])
        xb.fromNumpy1D(X[b])
        xs.append((xa, xb, X.shape[1] // DIM, i))
    netcalc.generalizedCorrelationGpu(Xa=xs[0][0], Xb=xs[0][1], k=K_NN, n=xs[0][2], xd=2, d=DIM)
    t0 = time.perf_counter()
    plain_ops = 0.0
    for xa, xb, m, i in xs:
        netcalc.generalizedCorrelationGpu(Xa=xa, Xb=xb, k=K_NN, n=m, xd=2, d=DIM)
        plain_ops += 8.0 * DIM * m * (m - 1)
    plain_s = time.perf_counter() - t0
    # the plain rate is per pair of the sample; scale to the batch's pair mix by work
    plain_pairs_per_s = len(xs) / plain_s * (plain_ops / len(xs)) / (ops / P)
    # per-trajectory APSP on -ln(GC) contact graphs
    gcv = gc.cpu().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    apsp_steps = 0
    for t, (X, mean) in enumerate(trajs):
        off, cnt = owners[t]
        A = synthetic.contact_graph(mean, gcv[off:off + cnt], synthetic.all_pairs(X.shape[0]))
        H, st = device.apsp_lengths(torch.from_numpy(A).cuda(), X.shape[0])
        apsp_steps += st
    torch.cuda.synchronize()
    apsp_s = time.perf_counter() - t0
    shape = plan.shape
    plan.close()
    return {"trajectories": n_traj, "pairs": P, "batched_pairs_per_s": P / batched_s,
            "batched_s": batched_s, "batched_top_s": ops / batched_s / 1e12,
            "plain_per_call_pairs_per_s": plain_pairs_per_s,
            "speedup_vs_plain": (P / batched_s) / plain_pairs_per_s,
            "plain_sample": f"{len(xs)} pairs, one netcalc.generalizedCorrelationGpu call each, "
                            "rate scaled to the batch's mean work per pair",
            "tile": shape, "apsp_total_ms": 1000 * apsp_s, "apsp_steps": apsp_steps}


def c4_full(X, mean, m, ab_all):
    """The whole all-pairs job in one drop-in call (X and the pair list
    uploaded, all 1,999,000 GC values read back), then the shortest paths
    of its -ln(GC) contact graph on the device."""
    import torch
    import cuarray
    import netcalc
    from netsci_gb300 import device, synthetic
    Xc = cuarray.FloatCuArray()
    Xc.fromNumpy2D(X)
    abc = cuarray.IntCuArray()
    abc.fromNumpy2D(ab_all)
    R = cuarray.FloatCuArray()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    netcalc.generalizedCorrelation(X=Xc, R=R, ab=abc, k=K_NN, n=m, xd=2, d=DIM, platform=0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    gc = R.toNumpy1D()
    assert gc.shape[0] == len(ab_all) and np.all(np.isfinite(gc)) and np.all((gc >= 0) & (gc <= 1))
    A = synthetic.contact_graph(mean, gc, ab_all)
    Ad = torch.from_numpy(A).cuda()
    device.apsp_lengths(Ad, A.shape[0])
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    H, steps = device.apsp_lengths(Ad, A.shape[0])
    torch.cuda.synchronize()
    apsp_ms = 1000 * (time.perf_counter() - t1)
    # -ln(GC) weights are not integers: the automatic schedule runs Jacobi
    # steps (the reference's association, bit-exact); squaring on request
    # agrees within the rounding of a path sum
    device.set_apsp_method(1)
    try:
        t1 = time.perf_counter()
        Hs, products = device.apsp_lengths(Ad, A.shape[0])
        torch.cuda.synchronize()
        sq_ms = 1000 * (time.perf_counter() - t1)
    finally:
        device.set_apsp_method(-1)
    Hn, Hsn = H.cpu().numpy(), Hs.cpu().numpy()
    fin = np.isfinite(Hn)
    sq_rel = float(np.max(np.abs(Hsn[fin] - Hn[fin]) / np.maximum(np.abs(Hn[fin]), 1e-30)))
    out = {"pairs": int(len(ab_all)), "wall_s": wall, "pairs_per_s": len(ab_all) / wall,
           "api": "one netcalc.generalizedCorrelation call over host CuArrays",
           "h2d_bytes": int(X.nbytes + ab_all.nbytes), "d2h_bytes": int(gc.nbytes),
           "apsp_neglog_gc": {"n": int(A.shape[0]), "edges": int(np.isfinite(A).sum() - A.shape[0]),
                              "ms": apsp_ms, "jacobi_steps": steps,
                              "squaring_ms": sq_ms, "squaring_products": products,
                              "squaring_max_rel_diff": sq_rel}}
    return out, A, Hn, steps


def bootstrap(X, m, resamples: int):
    """Bootstrap part of the large configuration: resamples of the frames
    (with replacement, m' = m) of a fixed 100-node subset, all 4950 pairs per
    resample, every resample in one plan (frame maps on the device)."""
    import torch
    from netsci_gb300 import device, synthetic
    sub = np.ascontiguousarray(X[:100])
    Xd, mm = device.pack_trajectory(sub, DIM)
    rng = np.random.default_rng(100)
    maps, pairs = [], []
    ab = synthetic.all_pairs(100)
    for r in range(resamples):
        fm = torch.from_numpy(rng.integers(0, mm, size=mm).astype(np.int32)).cuda()
        maps.append(fm)
        pairs += device.make_pairs(Xd, mm, ab, fmap=fm, m_samples=mm)
    gc = torch.empty(len(pairs), device="cuda")
    t_plan = time.perf_counter()
    plan = device.KsgPlan(pairs, K_NN, DIM, gc=gc, graph=True, autotune=True)
    plan.prepare()
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t_plan
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    plan.run()
    ev1.record()
    torch.cuda.synchronize()
    dt = ev0.elapsed_time(ev1) / 1000.0
    plan.check()
    g = gc.cpu().numpy()
    assert np.all(np.isfinite(g))
    out = {"resamples": resamples, "pairs": len(pairs), "seconds": dt,
           "pairs_per_s": len(pairs) / dt, "plan_setup_s": plan_s, "search": plan.shape["search"],
           "timed": "one run of one plan holding every resample's pairs (CUDA events)"}
    plan.close()
    return out


def serving(n_req: int, quick: bool):
    """Configuration C5. One set of requests of the mixed stream; arrival
    times are a Poisson process whose rate is scaled per row (the same
    requests at every load). The overload row (the stated 200 req/s, all
    requests queued within a fraction of a second) gives the capacity;
    the rows at 0.5x and 0.8x of it are steady state. Each row runs the
    continuous-batching server and the plain one-request-at-a-time path on
    the same arrivals."""
    from netsci_gb300 import serving as sv
    base = sv.c5_trace(n_req, seed=5, rate=200.0, scale=0.25 if quick else 1.0)

    def at_rate(rate):
        return [sv.Request(r.t * 200.0 / rate, r.kind, r.params, r.data) for r in base]

    def row(trace, label, offered):
        with sv.Server(budget_bytes=150 << 30) as srv:
            res_b, sum_b = sv.run_served(srv, trace)
            st = srv.stats()
        res_p, sum_p = sv.run_plain(trace)
        same = all(np.array_equal(a, b) for a, b in zip(res_b, res_p))
        return {"load": label, "offered_req_per_s": offered, "requests": len(trace),
                "batched": sum_b, "plain": sum_p, "ticks": st["ticks"],
                "peak_device_bytes": st["peak_bytes"], "results_equal_alone_and_mixed": same}

    rows = [row(base, "overload (the stated 200 req/s)", 200.0)]
    capacity = rows[0]["batched"]["requests_per_s"]
    for f in (0.5, 0.8):
        r = row(at_rate(f * capacity), f"{f:.1f} x capacity", f * capacity)
        r["utilisation"] = f
        rows.append(r)
    return {"capacity_req_per_s": capacity,
            "capacity_source": "requests completed per second of the overload row's makespan",
            "plain_capacity_req_per_s": rows[0]["plain"]["requests_per_s"],
            "budget_bytes": 150 << 30, "rows": rows}


def reference_gpu(X, m, ab_pool, apsp_graphs):
    """The reference's own GPU code (oracle/_ref/libnetcalc_ref_gpu.so):
    one blocking generalizedCorrelationGpu call per pair, and its Hedetniemi
    kernel on the given graphs to the fixed point this library reaches."""
    import oracle
    G = oracle.ref_gpu_lib()
    if G is None:
        return {"unavailable": "reference GPU library not built (no reference sources)"}
    out = {"code": "netcalc/src/mutual_information_gpu.cu, generalized_correlation_gpu.cpp, "
                   "hedetniemi_gpu.cu compiled unmodified for sm_103a"}
    rows = [(np.ascontiguousarray(X[a]), np.ascontiguousarray(X[b])) for a, b in ab_pool]
    G.refgpu_gc(rows[0][0], rows[0][1], m, K_NN, DIM)
    t0 = time.perf_counter()
    for xa, xb in rows[1:]:
        G.refgpu_gc(xa, xb, m, K_NN, DIM)
    dt = time.perf_counter() - t0
    out["gc_per_call"] = {"pairs": len(rows) - 1, "pairs_per_s": (len(rows) - 1) / dt,
                          "workload": f"N={X.shape[0]}, m={m}, d={DIM}, k={K_NN}"}
    # the 56-node protein configuration (m = 1000)
    from netsci_gb300 import synthetic
    Xp, _ = synthetic.protein_trajectory(56, 1000, seed=56)
    abp = synthetic.all_pairs(56)[::24]
    t0 = time.perf_counter()
    for a, b in abp:
        G.refgpu_gc(np.ascontiguousarray(Xp[a]), np.ascontiguousarray(Xp[b]), 1000, K_NN, DIM)
    dt = time.perf_counter() - t0
    out["gc_per_call_protein56"] = {"pairs": len(abp), "pairs_per_s": len(abp) / dt,
                                    "workload": "N=56, m=1000, d=3, k=6"}
    aps = {}
    for name, (A, H_ours, steps) in apsp_graphs.items():
        L = steps + 2
        oracle.ref_gpu_apsp_lengths(A, 2)
        t0 = time.perf_counter()
        Href = oracle.ref_gpu_apsp_lengths(A, L)
        dt = time.perf_counter() - t0
        aps[name] = {"launches": L, "ms": 1000 * dt, "ms_per_launch": 1000 * dt / L,
                     "equals_ours_bit_exact": bool(np.array_equal(Href, H_ours))}
    out["apsp"] = aps
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank)
        return

    import torch
    import torch.distributed as dist
    from netsci_gb300 import device, sharding, synthetic

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(v: float) -> float:
        return sharding.max_over_ranks(v, device="cuda")

    X, mean, N, m = workload(args.quick)
    ab_all = synthetic.all_pairs(N)
    B = args.pairs_per_step
    S = args.warmup + args.steps
    need = sharding.pairs_needed(world, S, B)
    if need > len(ab_all):
        raise SystemExit(f"{need} pairs requested, the workload has {len(ab_all)}")

    Xd, mm = device.pack_trajectory(X, DIM)
    torch.cuda.synchronize()

    def slice_for(step: int) -> np.ndarray:
        return sharding.spread_batch(ab_all, rank, world, S, step, B)

    # ---- batched persistent plans (graph + kernel events) --------------------
    outs, plans = [], []
    for s in range(S):
        gc = torch.empty(B, device="cuda")
        plans.append(device.KsgPlan(device.make_pairs(Xd, mm, slice_for(s)), K_NN, DIM, gc=gc,
                                    graph=True, timing=True, autotune=True))
        outs.append(gc)
    for s in range(args.warmup):
        plans[s].run()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record()
        for s in range(args.warmup, S):
            plans[s].run()
        ev1.record()
        torch.cuda.synchronize()
    barrier()
    dev_ms = ev0.elapsed_time(ev1)
    kms = [plans[s].kernel_ms() for s in range(args.warmup, S)]
    tied = [plans[s].tied_samples() for s in range(args.warmup, S)]
    launches = sum(plans[s].launches for s in range(args.warmup, S))
    t_max = max_over_ranks(dev_ms) / 1000.0
    value = sharding.weak_scaling_value(world, args.steps, B, t_max)
    gc_vals = torch.cat([outs[s] for s in range(args.warmup, S)]).cpu().numpy()
    assert np.all(np.isfinite(gc_vals)) and np.all((gc_vals >= 0) & (gc_vals <= 1))

    # ---- roofline: the search kernel (dominant) and the count kernel --------------
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    props = torch.cuda.get_device_properties(local)
    sm_max = float(peaks.get("sm_max_mhz") or 2070.0)
    peak_gops = props.multi_processor_count * 128 * sm_max * 1e6 / 1e9
    ops_launch = ops_per_pair(m) * B
    search = plans[args.warmup].shape["search"]
    clocks = clk.summary()
    ceil_search, ceil_count = device.issue_ceiling(DIM)
    search_s = statistics.mean(k[0] for k in kms) / 1000.0
    count_s = statistics.mean(k[1] for k in kms) / 1000.0
    if search == "cell-grid":
        evs = [plans[s].evaluations() for s in range(args.warmup, S)]
        joint = statistics.mean(e[0] for e in evs)
        one_var = statistics.mean(e[1] for e in evs)
        compares = statistics.mean(e[2] for e in evs)
        search_ops = joint * 4 * DIM
        count_ops = one_var * (2 * DIM - 1) + compares
        per_kernel = {
            "ksg_grid_pass1_kernel": {
                "ms_per_launch": 1000 * search_s, "ops_per_launch": search_ops,
                "joint_evaluations": joint, "ops_per_evaluation": 4 * DIM,
                "achieved_gops": search_ops / search_s / 1e9,
                "frac": search_ops / search_s / 1e9 / peak_gops,
                "mix_ceiling_gops": ceil_search,
                "frac_of_mix_ceiling": search_ops / search_s / 1e9 / ceil_search},
            "ksg_grid_count_kernel": {
                "ms_per_launch": 1000 * count_s, "ops_per_launch": count_ops,
                "one_variable_evaluations": one_var, "eps_comparisons": compares,
                "ops": "2d-1 per one-variable distance + 1 per eps comparison",
                "achieved_gops": count_ops / count_s / 1e9,
                "frac": count_ops / count_s / 1e9 / peak_gops,
                "mix_ceiling_gops": ceil_count,
                "frac_of_mix_ceiling": count_ops / count_s / 1e9 / ceil_count},
            "ksg_tie_kernel": {
                "ms_per_launch": statistics.mean(k[2] for k in kms),
                "tied_samples_per_launch": statistics.mean(tied),
                "note": ("samples whose k-th distance ties between frames with different "
                         "marginals, replayed in the reference sort's order; O(m) per "
                         "sample")},
        }
        dom = per_kernel["ksg_grid_pass1_kernel"]
        kernel, achieved, traffic = "ksg_grid_pass1_kernel", dom["achieved_gops"], None
        if m == M_FRAMES:
            traffic = SEARCH_DRAM_BYTES_PER_PAIR * B
        mix = ceil_search
    else:
        per_kernel = None
        kernel, achieved, traffic, mix = "ksg_count_kernel", ops_launch / search_s / 1e9, None, None
    frac_at_clock = None
    if clocks.get("sm_mhz"):
        frac_at_clock = achieved / (props.multi_processor_count * 128 * clocks["sm_mhz"] * 1e6 / 1e9)
    roofline = {
        "bound": "cuda_core_issue", "kernel": kernel, "achieved": achieved, "peak": peak_gops,
        "unit": "Gop/s", "frac": achieved / peak_gops, "frac_at_median_clock": frac_at_clock,
        "mix_ceiling": mix, "frac_of_mix_ceiling": (achieved / mix) if mix else None,
        "traffic": traffic,
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the search kernel "
                           "on a 256-pair step, scaled by pairs" if traffic else None),
        "peak_source": (f"{props.multi_processor_count} SMs x 128 lanes x {sm_max:.0f} MHz "
                        "(sm_max_mhz of MEASURED_PEAKS.json; MEASURED_PEAKS.json has no "
                        "CUDA-core figure)"),
        "mix_ceiling_source": ("nsg_measure_issue_ceiling: the kernel's own inner loop alone on a "
                               "staged tile (no memory traffic, no range setup, no list updates), "
                               "measured on this GPU with CUDA events"),
        "search": search, "per_kernel": per_kernel,
        "algorithmic_pruning_gops": ops_launch / (search_s + count_s) / 1e9,
        "algorithmic_pruning_note": ("8*d*m*(m-1) operations per pair (what an exhaustive "
                                     "search does) over the two kernels' time: the cell grids' "
                                     "gain, not a kernel fraction"),
    }

    # ---- the exhaustive search on the same workload, for comparison ----------------
    exhaustive = None
    if not args.quick:
        device.set_ksg_search(0)
        try:
            ex_plans = []
            for s_ in range(3):
                g_ = torch.empty(B, device="cuda")
                ex_plans.append((device.KsgPlan(device.make_pairs(Xd, mm, slice_for(s_)), K_NN, DIM,
                                                gc=g_, graph=True, timing=True), g_))
            ex_plans[0][0].run()
            torch.cuda.synchronize()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for pl, _ in ex_plans[1:]:
                pl.run()
            e1.record()
            torch.cuda.synchronize()
            ex_ms = max_over_ranks(e0.elapsed_time(e1)) / (len(ex_plans) - 1)
            ex_count = statistics.mean(pl.kernel_ms()[0] for pl, _ in ex_plans[1:]) / 1000.0
            same = all(np.array_equal(g_.cpu().numpy(), outs[s_].cpu().numpy())
                       for s_, (_, g_) in enumerate(ex_plans[1:], start=1) if s_ < S)
            exhaustive = {"value": world * B / (ex_ms / 1000.0), "unit": "pairs/s", "ms_per_step": ex_ms,
                          "steps": len(ex_plans) - 1,
                          "count_kernel_frac_of_peak": ops_launch / ex_count / 1e9 / peak_gops,
                          "same_gc_as_cell_grid": bool(same)}
            for pl, _ in ex_plans:
                pl.close()
        finally:
            device.set_ksg_search(-1)

    # ---- e2e through the drop-in CuArray API -------------------------------------
    e2e = None
    if not args.no_e2e:
        import cuarray
        import netcalc
        Xc = cuarray.FloatCuArray()
        Xc.fromNumpy2D(X)
        abs_ = []
        for s in range(S):
            a = cuarray.IntCuArray()
            a.fromNumpy2D(slice_for(s))
            abs_.append(a)
        R = cuarray.FloatCuArray()
        for s in range(args.warmup):
            netcalc.generalizedCorrelation(X=Xc, R=R, ab=abs_[s], k=K_NN, n=m, xd=2, d=DIM,
                                           platform=0)
        barrier()
        t0 = time.perf_counter()
        for s in range(args.warmup, S):
            netcalc.generalizedCorrelation(X=Xc, R=R, ab=abs_[s], k=K_NN, n=m, xd=2, d=DIM,
                                           platform=0)
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": world * args.steps * B / dt, "unit": "pairs/s",
               "h2d_bytes_per_step": int(X.nbytes + B * 2 * 4),
               "d2h_bytes_per_step": int(B * 4),
               "api": "netcalc.generalizedCorrelation over host CuArrays (page-locked storage, as CuArray allocates arrays of 16 MB and more)"}
        last = R.toNumpy1D()
        assert np.array_equal(last, outs[S - 1].cpu().numpy()) or \
            np.max(np.abs(last - outs[S - 1].cpu().numpy())) <= 1e-6

    for p in plans:
        p.close()

    # ---- plain per-call (the reference's call structure) ------------------------
    plain = None
    if rank == 0:
        import cuarray
        import netcalc
        sample = 16 if not args.quick else 8
        rows = slice_for(0)[:sample]
        xs = []
        for a, b in rows:
            xa, xb = cuarray.FloatCuArray(), cuarray.FloatCuArray()
            xa.fromNumpy1D(X[a])
            xb.fromNumpy1D(X[b])
            xs.append((xa, xb))
        netcalc.generalizedCorrelationGpu(Xa=xs[0][0], Xb=xs[0][1], k=K_NN, n=m, xd=2, d=DIM)
        t0 = time.perf_counter()
        for xa, xb in xs:
            netcalc.generalizedCorrelationGpu(Xa=xa, Xb=xb, k=K_NN, n=m, xd=2, d=DIM)
        dt = time.perf_counter() - t0
        plain = {"value": sample / dt, "unit": "pairs/s", "sample": f"{sample} pairs, one call each"}

    # ---- APSP ------------------------------------------------------------------------
    def solve_apsp(A, n_g, method):
        """Timed solve (ms, products, H); method -1 automatic, 0 Jacobi."""
        device.set_apsp_method(method)
        try:
            device.apsp_lengths(A, n_g)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            H, steps = device.apsp_lengths(A, n_g)
            torch.cuda.synchronize()
            return 1000 * (time.perf_counter() - t0), steps, H
        finally:
            device.set_apsp_method(-1)

    apsp, apsp_graphs = None, {}
    if rank == 0:
        apsp = {}
        n_g = 2000 if not args.quick else 500
        for name, integer in (("rgg_int", True), ("rgg_float", False)):
            A_np = synthetic.random_geometric_graph(n_g, 12, seed=11, integer_weights=integer)
            A = torch.from_numpy(A_np).cuda()
            ms, products, H = solve_apsp(A, n_g, -1)
            ms_j, steps_j, H_j = solve_apsp(A, n_g, 0)
            assert torch.equal(H, H_j)
            apsp[f"{name}_ms"] = ms
            apsp[f"{name}_products"] = products
            apsp[f"{name}_schedule"] = "squaring" if products < steps_j else "jacobi"
            apsp[f"{name}_jacobi_ms"] = ms_j
            apsp[f"{name}_jacobi_steps"] = steps_j
            # min-plus terms (one add and one min per (i, j, k)) per second of
            # the Jacobi steps, against one term per lane per cycle (packed
            # add + 3-input min: two instructions per two terms)
            apsp[f"{name}_terms_per_s"] = n_g ** 3 * steps_j / (ms_j / 1000)
            apsp_graphs[name] = (A_np, H.cpu().numpy(), steps_j)
        apsp["n"] = n_g
        apsp["terms_peak_per_s"] = props.multi_processor_count * 128 * sm_max * 1e6
        apsp["frac"] = apsp["rgg_int_terms_per_s"] / apsp["terms_peak_per_s"]
        apsp["note"] = ("schedule: repeated squaring where it is bit-exact (symmetric, zero "
                        "diagonal, integer weights), else Jacobi steps; the Jacobi timing of "
                        "every graph is reported beside it, with equal results")

    # ---- other configurations (rank 0) ----------------------------------------------
    extra = {}

    def section(name, fn):
        """Run one secondary measurement; a failure is reported in the line
        (with its message) instead of losing the headline numbers."""
        try:
            return fn()
        except Exception as e:  # noqa: BLE001
            torch.cuda.synchronize()
            return {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        if not args.no_c4_full and not args.quick:
            def run_c4():
                full, A_c4, H_c4, steps_c4 = c4_full(X, mean, m, ab_all)
                apsp_graphs["c4_neglog_gc"] = (A_c4, H_c4, steps_c4)
                return full
            extra["c4_full"] = section("c4_full", run_c4)
        if args.c3_trajectories:
            extra["uneven_batch"] = section("uneven_batch",
                                            lambda: uneven_batch(args.c3_trajectories, args.quick))
        if args.bootstrap_resamples:
            extra["bootstrap"] = section("bootstrap",
                                         lambda: bootstrap(X, m, args.bootstrap_resamples))
        if args.serving_requests:
            extra["serving"] = section("serving", lambda: serving(args.serving_requests, args.quick))

    # ---- CPU baseline and parity: the reference's CPU code on pairs of the timed steps --
    cpu = parity = None
    if rank == 0 and world == 1:
        import cuarray
        import netcalc
        threads = os.cpu_count() or 1
        n_s = args.cpu_sample or threads
        pool = timed_pair_pool(ab_all, world, S, args.warmup, B)
        sel = pool[np.random.default_rng(3).choice(len(pool), size=n_s, replace=False)]
        want, dt, kind = cpu_gc(X, m, sel, threads)
        cpu = {"value": n_s / dt, "unit": "pairs/s", "cores": threads, "kind": kind,
               "sample": f"{n_s} random pairs of the timed batches, one per thread, {dt:.1f} s wall",
               "code": ("netcalc::generalizedCorrelationCpu, the reference's own sources compiled "
                        "unmodified (g++ -O3 -flto)" if kind == "reference"
                        else "oracle restatement")}
        Xc = cuarray.FloatCuArray()
        Xc.fromNumpy2D(X)
        abc = cuarray.IntCuArray()
        abc.fromNumpy2D(np.ascontiguousarray(sel, np.int32))
        R = cuarray.FloatCuArray()
        netcalc.generalizedCorrelation(X=Xc, R=R, ab=abc, k=K_NN, n=m, xd=2, d=DIM, platform=0)
        got = R.toNumpy1D()
        parity = {"pairs": int(n_s), "against": kind, "bit_exact": bool(np.array_equal(got, want)),
                  "max_abs_diff": float(np.max(np.abs(got - want))),
                  "path": "netcalc.generalizedCorrelation (GPU platform) vs the CPU leg's GC"}

    ref_gpu = None
    if rank == 0 and not args.no_reference_gpu and not args.quick:
        pool = timed_pair_pool(ab_all, world, S, args.warmup, B)
        sel = pool[np.random.default_rng(4).choice(len(pool), size=5, replace=False)]
        ref_gpu = section("reference_gpu", lambda: reference_gpu(X, m, sel, apsp_graphs))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"all-pairs GC, N={N} nodes, m={m} frames, d={DIM}, k={K_NN}",
                       "pairs_per_step": B, "total_pairs": int(len(ab_all)),
                       "batches": "consecutive pairs, batches spread evenly over the pair list",
                       "parallelism": f"pairs sharded over {world} GPU(s), no collective",
                       "l2": "inputs larger than L2 (X resident, 241 MB > 129 MB L2)"},
            "e2e": e2e, "parity": parity, "plain_per_call": plain,
            "exhaustive_search": exhaustive, "apsp": apsp, "reference_gpu": ref_gpu,
            "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
