#!/usr/bin/env python
"""Benchmark of the netcalc hot path on GB300.

Workload (the large single-system configuration): all-pairs generalized
correlation of a synthetic protein trajectory with N = 2000 nodes,
m = 10000 frames, d = 3, k = 6 (1,999,000 node pairs in total). A step is
one batch of `--pairs-per-step` consecutive pairs of that all-pairs list;
different steps (and ranks) take different batches. The trajectory stays
resident in HBM (X = 2000 x 3 x 10048 floats, 241 MB, larger than the
129 MB L2, so every step streams it from HBM).

Lines reported (one JSON line from rank 0):
  value     pairs/s of the batched persistent plan (graph replay), device
            timed with CUDA events, max over ranks; inputs resident.
  e2e       pairs/s through the drop-in API (netcalc.generalizedCorrelation
            over host CuArrays): host->device upload of X and the pair list
            and device->host read of the results inside every step.
  plain_per_call  pairs/s of one netcalc.generalizedCorrelationGpu call per
            pair (the reference's call structure) on a small sample.
  exhaustive_search  the same steps with the exhaustive neighbour search (every
            frame against every query): pairs/s, its count kernel's fraction of
            the issue peak, and whether its GC equals the cell-grid run's.
  apsp      Hedetniemi shortest-path ms on N = 2000 random geometric graphs
            (mean degree 12), integer weights U[1,100] and float weights.
  roofline  the neighbour-search kernels against the CUDA-core issue peak
            (SMs x 128 lanes x max SM clock). Work is the executed distance
            evaluations counted by the cell-grid kernels (4d ops per joint,
            2d per one-variable evaluation); effective_gops is the rate an
            exhaustive search would need, 8*d*m*(m-1) ops per pair.
  cpu_baseline  the CPU oracle port (restatement of the reference CPU path)
            on all host cores, on a bounded sample of pairs of this workload.
  uneven_batch  64 trajectories of uneven N and m in one plan vs the plain
            per-pair call, and one shortest-path solve per trajectory.
  bootstrap frame-resampled pairs of a 100-node subset (sampled resamples).
  serving   a trace of the mixed request stream: continuous batching vs
            one request at a time; p50/p99 latency and throughput.

``--impl reference`` runs only the CPU oracle port arm and prints its line.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "netsci_gb300" / "dropin"))

N_NODES, M_FRAMES, DIM, K_NN = 2000, 10000, 3, 6
# DRAM bytes per pair of the search + count kernels at m = 10000, from an ncu
# capture of a 256-pair step of this workload (profiles/ksg_grid_kernels_N2000_m10000.md:
# pass 1 109.6 MB read + 13.5 MB written, counts 63.1 + 5.7 MB); the traffic
# is per pair (each pair's grid copies and rows), so it scales with the pairs.
GRID_DRAM_BYTES_PER_PAIR = (112.1 + 15.0 + 64.4 + 8.9) * 1e6 / 256
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
    p.add_argument("--bootstrap-resamples", type=int, default=4,
                   help="bootstrap sample: resamples of the 100-node subset (0 = skip)")
    p.add_argument("--serving-requests", type=int, default=32,
                   help="serving trace length (0 = skip)")
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


def cpu_baseline(X, m, ab, threads: int):
    """The oracle port on `threads` host threads over len(ab) pairs."""
    import oracle
    t0 = time.perf_counter()
    oracle.pairs(X, m, DIM, ab, K_NN, gc=True, threads=threads)
    dt = time.perf_counter() - t0
    return len(ab) / dt, dt


def reference_arm(args, rank: int):
    if rank != 0:
        return
    X, mean, N, m = workload(args.quick)
    from netsci_gb300 import synthetic
    ab_all = synthetic.all_pairs(N)
    threads = os.cpu_count() or 1
    per_step = args.cpu_sample or threads
    rng = np.random.default_rng(7)
    times = []
    for s in range(args.warmup + args.steps):
        sel = ab_all[rng.choice(len(ab_all), size=per_step, replace=False)]
        rate, dt = cpu_baseline(X, m, sel, threads)
        if s >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = per_step * args.steps / total
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "pairs/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"all-pairs GC, N={N} nodes, m={m} frames, d={DIM}, k={K_NN}",
                   "pairs_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} random pairs per step, one per thread"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    plan.prepare()   # one timed run (about half a minute); the tuner's probes warmed the GPU
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
    return {"trajectories": n_traj, "pairs": P, "batched_pairs_per_s": P / batched_s,
            "batched_s": batched_s, "batched_top_s": ops / batched_s / 1e12,
            "plain_per_call_pairs_per_s": plain_pairs_per_s,
            "speedup_vs_plain": (P / batched_s) / plain_pairs_per_s,
            "plain_sample": f"{len(xs)} pairs, one netcalc.generalizedCorrelationGpu call each, "
                            "rate scaled to the batch's mean work per pair",
            "tile": plan.shape, "apsp_total_ms": 1000 * apsp_s, "apsp_steps": apsp_steps}


def bootstrap(X, m, resamples: int):
    """Bootstrap part of the large configuration: resamples of the frames
    (with replacement, m' = m) of a fixed 100-node subset, all 4950 pairs per
    resample in one plan (frame maps on the device)."""
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
    plan = device.KsgPlan(pairs, K_NN, DIM, gc=gc, graph=True, autotune=True)
    plan.run()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    plan.run()
    ev1.record()
    torch.cuda.synchronize()
    dt = ev0.elapsed_time(ev1) / 1000.0
    plan.check()
    return {"resamples": resamples, "pairs": len(pairs), "pairs_per_s": len(pairs) / dt,
            "full_job_estimate_s": 495000 / (len(pairs) / dt),
            "note": "100 resamples x 4950 pairs is the full job; timed here on a sample"}


def serving(n_req: int, quick: bool):
    """Configuration C5: a trace of the mixed request stream replayed at its
    arrival times against the continuous-batching server, and the same
    requests one at a time through the plain per-request entry points."""
    from netsci_gb300 import serving as sv
    trace = sv.c5_trace(n_req, seed=5, rate=200.0, scale=0.25 if quick else 1.0)
    with sv.Server(budget_bytes=150 << 30) as srv:
        res_b, sum_b = sv.run_served(srv, trace)
        st = srv.stats()
    res_p, sum_p = sv.run_plain(trace)
    same = all(np.array_equal(a, b) for a, b in zip(res_b, res_p))
    return {"requests": n_req, "batched": sum_b, "plain": sum_p, "ticks": st["ticks"],
            "peak_device_bytes": st["peak_bytes"], "results_equal_alone_and_mixed": same,
            "budget_bytes": 150 << 30}


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
        return sharding.rank_batch(ab_all, rank, S, step, B)

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
    count_ms = [plans[s].count_ms() for s in range(args.warmup, S)]
    launches = sum(plans[s].launches for s in range(args.warmup, S))
    t_max = max_over_ranks(dev_ms) / 1000.0
    value = sharding.weak_scaling_value(world, args.steps, B, t_max)
    gc_vals = torch.cat([outs[s] for s in range(args.warmup, S)]).cpu().numpy()
    assert np.all(np.isfinite(gc_vals)) and np.all((gc_vals >= 0) & (gc_vals <= 1))

    # ---- roofline of the count kernel ------------------------------------------
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    props = torch.cuda.get_device_properties(local)
    sm_max = float(peaks.get("sm_max_mhz") or 2070.0)
    peak_gops = props.multi_processor_count * 128 * sm_max * 1e6 / 1e9
    ops_launch = ops_per_pair(m) * B
    avg_launch_s = statistics.mean(count_ms) / 1000.0
    search = plans[args.warmup].shape["search"]
    # exhaustive-equivalent rate: the work an exhaustive search needs
    effective = ops_launch / avg_launch_s / 1e9
    if search == "cell-grid":
        # executed work: each joint-distance evaluation is 4d ops (2d
        # subtractions, 2d-1 max, 1 compare), each one-variable evaluation of
        # the counts 2d (d, d-1, 1), counted by the kernels
        evs = [plans[s].evaluations() for s in range(args.warmup, S)]
        exec_ops = statistics.mean(e[0] * 4 * DIM + e[1] * 2 * DIM for e in evs)
        evals = {"joint": statistics.mean(e[0] for e in evs),
                 "one_variable": statistics.mean(e[1] for e in evs)}
        kernel = "ksg_grid_pass1_kernel + ksg_grid_count_kernel"
        traffic = GRID_DRAM_BYTES_PER_PAIR * B if m == M_FRAMES else None
    else:
        exec_ops = ops_launch
        evals = None
        kernel = "ksg_count_kernel"
        traffic = None
    achieved = exec_ops / avg_launch_s / 1e9
    clocks = clk.summary()
    frac_at_clock = None
    if clocks.get("sm_mhz"):
        frac_at_clock = achieved / (props.multi_processor_count * 128 * clocks["sm_mhz"] * 1e6 / 1e9)

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
            ex_count = statistics.mean(pl.count_ms() for pl, _ in ex_plans[1:]) / 1000.0
            same = all(np.array_equal(g_.cpu().numpy(), outs[s_].cpu().numpy())
                       for s_, (_, g_) in enumerate(ex_plans[1:], start=1) if s_ < S)
            exhaustive = {"value": world * B / (ex_ms / 1000.0), "unit": "pairs/s", "ms_per_step": ex_ms,
                          "steps": len(ex_plans) - 1, "count_kernel_frac_of_peak": ops_launch / ex_count / 1e9 / peak_gops,
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
               "api": "netcalc.generalizedCorrelation over host CuArrays (pageable host memory)"}
        last = R.toNumpy1D()
        assert np.array_equal(last, outs[S - 1].cpu().numpy()) or \
            np.max(np.abs(last - outs[S - 1].cpu().numpy())) <= 1e-6

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
    apsp = None
    if rank == 0:
        apsp = {}
        n_g = 2000 if not args.quick else 500
        for name, integer in (("rgg_int", True), ("rgg_float", False)):
            A = torch.from_numpy(synthetic.random_geometric_graph(n_g, 12, seed=11,
                                                                  integer_weights=integer)).cuda()
            device.apsp_lengths(A, n_g)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            H, steps = device.apsp_lengths(A, n_g)
            torch.cuda.synchronize()
            dt_a = time.perf_counter() - t0
            apsp[f"{name}_ms"] = 1000 * dt_a
            apsp[f"{name}_steps"] = steps
            # min-plus terms (one add and one min per (i, j, k)) per second,
            # against one term per lane per cycle (packed add + 3-input min:
            # two instructions per two terms)
            apsp[f"{name}_terms_per_s"] = n_g ** 3 * steps / dt_a
        apsp["n"] = n_g
        apsp["terms_peak_per_s"] = props.multi_processor_count * 128 * sm_max * 1e6
        apsp["frac"] = apsp["rgg_int_terms_per_s"] / apsp["terms_peak_per_s"]

    # ---- other configurations (rank 0) ----------------------------------------------
    extra = {}
    if rank == 0:
        if args.c3_trajectories:
            extra["uneven_batch"] = uneven_batch(args.c3_trajectories, args.quick)
        if args.bootstrap_resamples:
            extra["bootstrap"] = bootstrap(X, m, args.bootstrap_resamples)
        if args.serving_requests:
            extra["serving"] = serving(args.serving_requests, args.quick)

    # ---- CPU baseline (oracle port on host cores) --------------------------------------
    cpu = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        n_s = args.cpu_sample or threads
        sel = ab_all[np.random.default_rng(3).choice(len(ab_all), size=n_s, replace=False)]
        rate, dt = cpu_baseline(X, m, sel, threads)
        cpu = {"value": rate, "unit": "pairs/s", "cores": threads, "kind": "port",
               "sample": f"{n_s} random pairs of the workload, {dt:.1f} s wall"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"all-pairs GC, N={N} nodes, m={m} frames, d={DIM}, k={K_NN}",
                       "pairs_per_step": B, "total_pairs": int(len(ab_all)),
                       "parallelism": f"pairs sharded over {world} GPU(s), no collective",
                       "l2": "inputs larger than L2 (X resident, 241 MB > 129 MB L2)",
                       "tile": plans[0].shape},
            "e2e": e2e, "plain_per_call": plain, "exhaustive_search": exhaustive, "apsp": apsp,
            "gpu_launches": launches,
            "roofline": {"bound": "cuda_core_issue", "achieved": achieved,
                         "peak": peak_gops, "unit": "Gop/s", "frac": achieved / peak_gops,
                         "frac_at_median_clock": frac_at_clock, "traffic": traffic,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a "
                                            "256-pair step, scaled by pairs" if traffic else None),
                         "kernel": kernel, "search": search,
                         "ops_per_launch": exec_ops, "evaluations_per_launch": evals,
                         "exhaustive_ops_per_launch": ops_launch,
                         "effective_gops": effective,
                         "peak_source": (f"{props.multi_processor_count} SMs x 128 lanes x "
                                         f"{sm_max:.0f} MHz (sm_max_mhz of MEASURED_PEAKS.json)")},
            "cpu_baseline": cpu, "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    for p in plans:
        p.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
