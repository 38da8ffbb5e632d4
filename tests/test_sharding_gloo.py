"""The multi-GPU layout on CPU ranks (gloo, world size 2): disjoint pair
batches per rank, the max-over-ranks timing reduction, weak-scaling value,
and a sharded all-pairs MI job gathered back equal to the oracle over the
same pairs. Each rank runs the product's own pair-list call on its batches
(netcalc.mutualInformation over CuArrays: the library's pair-list driver,
here on its CPU platform, ksg_cpu.cpp, since these ranks have no GPU).
Rendezvous on 127.0.0.1."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import cuarray
        import netcalc
        from netsci_gb300 import sharding, synthetic
        X, _ = synthetic.protein_trajectory(6, 200, seed=5)
        ab = synthetic.all_pairs(6)               # 15 pairs
        steps, per = 2, 3                        # 2 ranks x 2 steps x 3 pairs = 12 pairs
        mine = [sharding.rank_batch(ab, rank, steps, s, per) for s in range(steps)]
        Xc = cuarray.FloatCuArray()
        Xc.fromNumpy2D(X)
        parts = []
        for b in mine:
            abc = cuarray.IntCuArray()
            abc.fromNumpy2D(np.ascontiguousarray(b, np.int32))
            I = cuarray.FloatCuArray()
            assert netcalc.mutualInformation(X=Xc, I=I, ab=abc, k=6, n=200, xd=2, d=3,
                                             platform=netcalc.CPU_PLATFORM) == 1
            parts.append(I.toNumpy1D())
        mi = np.concatenate(parts)
        t = sharding.max_over_ranks(1.0 + rank)
        # gather the results and the batches on every rank
        out = [None] * world
        dist.all_gather_object(out, (rank, np.concatenate(mine).tolist(), mi.tolist(), t))
        q.put(out)
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    gathered = results[0]
    assert gathered == results[1]
    import oracle
    from netsci_gb300 import sharding, synthetic
    X, _ = synthetic.protein_trajectory(6, 200, seed=5)
    ab = synthetic.all_pairs(6)
    pairs_by_rank = {r: np.array(b) for r, b, _, _ in gathered}
    # disjoint batches, in rank order, covering the first 12 pairs
    both = np.concatenate([pairs_by_rank[0], pairs_by_rank[1]])
    assert np.array_equal(both, ab[:12])
    # the maximum of the per-rank times reached every rank
    assert all(t == 2.0 for _, _, _, t in gathered)
    # sharded results equal one process over the same pairs
    mi = np.concatenate([np.array(m, np.float32) for _, _, m, _ in sorted(gathered)])
    assert np.array_equal(mi, oracle.pairs(X, 200, 3, ab[:12], 6))
    assert sharding.weak_scaling_value(2, 2, 3, 0.5) == 24.0


def test_spread_batches_cover_the_list_disjointly():
    """bench.py's batches: world*steps batches spread evenly from the start
    to the end of the pair list, disjoint, rank-major."""
    from netsci_gb300 import sharding, synthetic
    ab = synthetic.all_pairs(2000)
    for world, steps, per in ((1, 25, 8192), (2, 8, 8192), (4, 5, 1000), (1, 1, 8192)):
        got = [sharding.spread_batch(ab, r, world, steps, s, per)
               for r in range(world) for s in range(steps)]
        assert all(len(b) == per for b in got)
        assert np.array_equal(got[0][0], ab[0])
        if world * steps > 1:
            assert np.array_equal(got[-1][-1], ab[-1])
        keys = np.concatenate([b[:, 0].astype(np.int64) * 4000 + b[:, 1] for b in got])
        assert len(np.unique(keys)) == len(keys)


def test_reference_arm_only_rank0_prints(tmp_path):
    """bench.py --impl reference under a 2-rank launch: rank 0 prints one
    JSON line, rank 1 exits 0 without work."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--quick", "--steps", "1", "--warmup", "0", "--cpu-sample", "2"]
    r = subprocess.run(cmd, cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    import json
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
